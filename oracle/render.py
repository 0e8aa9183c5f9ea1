"""Restatement of the reference's screen-space fluid pipeline in NumPy, for
tests only (the same passes as pibiti_gb300/csrc/sph_render.cu; the GL
semantics are the reference's: Graphics/render_particles.cpp ScreenSpaceSet
(depth test GL_LESS, blend SRC_ALPHA / ONE_MINUS_SRC_ALPHA, particles drawn
in index order), Gbuffer.vs / Gbuffer.fs (point sprites, disc discard,
thickness 0.02 exp(-d^2 / 6)), CurvatureFlow.fs, BilateralFilter.fs,
ScreenSpaceRender.fs; depth textures sampled nearest with repeat wrap), and
the foam overlay of SetFoam (render_particles.cpp:306-334; Foam.vs, Foam.gs,
Foam.fs; blending off, depth test GL_ALWAYS).

Single precision, with the kernel's operation order for everything up to
the depth buffer (so depth and coverage agree bit for bit); the exponentials
and powers come from NumPy, so thickness, smoothing and colour agree to a
tolerance.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def _mul4(m, x, y, z, w):
    """Column-major 4x4 times (x, y, z, w), summed left to right in float32."""
    m = np.asarray(m, f32)
    r = []
    for row in range(4):
        a = (m[row] * x + m[4 + row] * y).astype(f32)
        a = (a + (m[8 + row] * z).astype(f32)).astype(f32)
        a = (a + (m[12 + row] * w).astype(f32)).astype(f32)
        r.append(a)
    return r


def project(pos, mv, pr, W, H, radius, scale):
    """Per particle: (wx, wy, wz, size) float32; size 0 where not drawn."""
    p = np.asarray(pos, f32)
    one = np.ones(len(p), f32)
    ex, ey, ez, ew = _mul4(mv, p[:, 0], p[:, 1], p[:, 2], one)
    cx, cy, cz, cw = _mul4(pr, ex, ey, ez, ew)
    ok = (cw > 0) & (np.abs(cx) <= cw) & (np.abs(cy) <= cw) & (np.abs(cz) <= cw)
    dist = np.sqrt(((ex * ex + ey * ey).astype(f32) + (ez * ez)).astype(f32)).astype(f32)
    with np.errstate(divide="ignore", invalid="ignore"):
        # pointRadius * (pointScale / dist) with the uniforms bound crossed
        # (render_particles.cpp:274-275, :791-792): scale * (radius / dist)
        size = (f32(scale) * (f32(radius) / dist).astype(f32)).astype(f32)
        size = np.minimum(np.maximum(size, f32(1)), f32(1024)).astype(f32)
        nx, ny, nz = (cx / cw).astype(f32), (cy / cw).astype(f32), (cz / cw).astype(f32)
    wx = ((nx + f32(1)).astype(f32) * f32(0.5 * W)).astype(f32)
    wy = ((ny + f32(1)).astype(f32) * f32(0.5 * H)).astype(f32)
    wz = ((nz + f32(1)).astype(f32) * f32(0.5)).astype(f32)
    size = np.where(ok, size, f32(0)).astype(f32)
    return wx, wy, wz, size


def _mag(wx, wy, size, px, py):
    sx = (f32(0.5) + ((px.astype(f32) + f32(0.5)).astype(f32) - wx).astype(f32) / size).astype(f32)
    ty = (f32(0.5) - ((py.astype(f32) + f32(0.5)).astype(f32) - wy).astype(f32) / size).astype(f32)
    nx = ((sx * f32(2)).astype(f32) - f32(1)).astype(f32)
    ny = ((ty * f32(-2)).astype(f32) + f32(1)).astype(f32)
    return ((nx * nx).astype(f32) + (ny * ny).astype(f32)).astype(f32)


def gbuffer(sprites, W, H):
    """Depth (cleared 1.0) and thickness (cleared 0) after drawing the
    sprites in index order."""
    wx, wy, wz, size = sprites
    depth = np.ones((H, W), f32)
    thick = np.zeros((H, W), f32)
    for i in np.nonzero(size > 0)[0]:
        h = f32(0.5) * size[i]
        x0 = max(int(np.ceil(f32(f32(wx[i] - h) - f32(0.5)))), 0)
        x1 = min(int(np.ceil(f32(f32(wx[i] + h) - f32(0.5)))) - 1, W - 1)
        y0 = max(int(np.ceil(f32(f32(wy[i] - h) - f32(0.5)))), 0)
        y1 = min(int(np.ceil(f32(f32(wy[i] + h) - f32(0.5)))) - 1, H - 1)
        if x1 < x0 or y1 < y0:
            continue
        py, px = np.mgrid[y0:y1 + 1, x0:x1 + 1]
        mag = _mag(wx[i], wy[i], size[i], px, py)
        inside = mag <= 1
        sub_d = depth[y0:y1 + 1, x0:x1 + 1]
        sub_t = thick[y0:y1 + 1, x0:x1 + 1]
        passed = inside & (wz[i] < sub_d)
        tv = (f32(0.02) * np.exp((-mag / f32(6)).astype(f32)).astype(f32)).astype(f32)
        sub_d[passed] = wz[i]
        sub_t[passed] = ((tv * tv).astype(f32) + (sub_t * (f32(1) - tv)).astype(f32)).astype(f32)[passed]
    return depth, thick


def fragment_count(sprites, W, H) -> int:
    """Number of (pixel, sprite) fragments: pixel centres in a sprite's
    square and inside its disc."""
    wx, wy, wz, size = sprites
    total = 0
    for i in np.nonzero(size > 0)[0]:
        h = f32(0.5) * size[i]
        x0 = max(int(np.ceil(f32(f32(wx[i] - h) - f32(0.5)))), 0)
        x1 = min(int(np.ceil(f32(f32(wx[i] + h) - f32(0.5)))) - 1, W - 1)
        y0 = max(int(np.ceil(f32(f32(wy[i] - h) - f32(0.5)))), 0)
        y1 = min(int(np.ceil(f32(f32(wy[i] + h) - f32(0.5)))) - 1, H - 1)
        if x1 < x0 or y1 < y0:
            continue
        py, px = np.mgrid[y0:y1 + 1, x0:x1 + 1]
        total += int((_mag(wx[i], wy[i], size[i], px, py) <= 1).sum())
    return total


def _tex(z, dx, dy):
    """z sampled at (x + dx, y + dy) with repeat wrap."""
    return np.roll(np.roll(z, -dy, axis=0), -dx, axis=1)


def _derivs(z):
    dx = lambda n: ((_tex(z, 1 + n, 0) - _tex(z, -1 + n, 0)) / f32(2)).astype(f32)  # noqa: E731
    dy = lambda n: ((_tex(z, 0, 1 + n) - _tex(z, 0, -1 + n)) / f32(2)).astype(f32)  # noqa: E731
    return (dx(0), dy(0), ((dx(1) - dx(-1)) / f32(2)).astype(f32),
            ((dy(1) - dy(-1)) / f32(2)).astype(f32))


def _coords(W, H):
    i = ((np.arange(W, dtype=f32) + f32(0.5)) / f32(W)).astype(f32)[None, :]
    j = ((np.arange(H, dtype=f32) + f32(0.5)) / f32(H)).astype(f32)[:, None]
    return np.broadcast_to(i, (H, W)), np.broadcast_to(j, (H, W))


def curvature(z):
    """One CurvatureFlow.fs pass (float64 arithmetic on the float32 inputs)."""
    H, W = z.shape
    i, j = (a.astype(np.float64) for a in _coords(W, H))
    Z = z.astype(np.float64)
    dzx, dzy, dzx2, dzy2 = (a.astype(np.float64) for a in _derivs(z))
    Cx, Cy = 2.0 / (W * i), 2.0 / (H * j)
    D = Cy * Cy * dzx * dzx + Cx * Cx * dzy * dzy + Cx * Cx * Cy * Cy * Z * Z
    inv = 1.0 / D ** 1.5
    ky, kx = 4.0 / H / H, 4.0 / W / W
    dDx = ky * j ** -2 * 2 * dzx * dzx2 + kx * dzy * dzy * -2 * i ** -3 + ky * j ** -2 * kx * (
        -2 * i ** -3 * Z * Z + i ** -2 * 2 * Z * dzx)
    dDy = kx * i ** -2 * 2 * dzy * dzy2 + ky * dzx * dzx * -2 * j ** -3 + kx * i ** -2 * ky * (
        -2 * j ** -3 * Z * Z + j ** -2 * 2 * Z * dzy)
    Ex = 0.5 * dzx * dDx - dzx2 * D
    Ey = 0.5 * dzy * dDy - dzy2 * D
    flow = np.clip((Cy * Ex + Cx * Ey) * inv / 2.0, -1.0, 1.0)
    out = np.clip(Z - flow * 0.001, 0.0, 1.0)
    return np.where((Z <= 0) | (Z == 1), 1.0, out).astype(f32)


def kernel(kc: int):
    return np.array([np.exp(-i * i * 0.1) for i in range(-kc, kc + 1)], f32)


def bilateral(z, kc: int, sigma: float):
    """One BilateralFilter.fs pass (along y, see sph_render.cu)."""
    k = kernel(kc).astype(np.float64)
    Z = z.astype(np.float64)
    norm = lambda x: 0.39894 * np.exp(-0.5 * x * x / (sigma * sigma)) / sigma  # noqa: E731
    bZ = 1.0 / norm(0.0)
    num = np.zeros_like(Z)
    den = np.zeros_like(Z)
    for a in range(-kc, kc + 1):
        for b in range(-kc, kc + 1):
            cv = _tex(z, 0, b).astype(np.float64)
            f = norm(cv - Z) * bZ * k[kc + a] * k[kc + b]
            den += f
            num += f * cv
    return np.where((Z == 0) | (Z == 1), 1.0, num / den).astype(f32)


def shade(z, thick, mv, pr, env, bg):
    """ScreenSpaceRender.fs (float64 arithmetic); background where empty."""
    with np.errstate(divide="ignore", invalid="ignore"):  # empty pixels are replaced below
        return _shade(z, thick, mv, pr, env, bg)


def _shade(z, thick, mv, pr, env, bg):
    H, W = z.shape
    i, j = (a.astype(np.float64) for a in _coords(W, H))
    Z = z.astype(np.float64)
    dzx, dzy, _, _ = (a.astype(np.float64) for a in _derivs(z))
    Cx, Cy = 2.0 / (W * i), 2.0 / (H * j)
    D = Cy * Cy * dzx * dzx + Cx * Cx * dzy * dzy + Cx * Cx * Cy * Cy * Z * Z
    rv = 1.0 / np.sqrt(D)
    n = np.stack([-Cy * dzx * rv, -Cx * dzy * rv, Cx * Cy * (1 - Z) * rv], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    gamma = 2.2
    light = np.array([0.0, -10.0, -1.0])
    li = np.array([0.252, 0.212, 0.15]) ** gamma
    prm = np.asarray(pr, np.float64).reshape(4, 4)  # [column][row]
    px, py = (i - 0.5) * 2.0, (j - 0.5) * 2.0
    e0 = np.stack([Z * (-px * prm[0, 0]), Z * (-py * prm[1, 1]), Z], -1)
    minv = np.linalg.inv(np.asarray(mv, np.float64).reshape(4, 4).T)  # matrix [row][col]
    eye = e0 @ minv[:3, :3] + minv[3, :3]  # row vector times matrix
    fe = eye / np.linalg.norm(eye, axis=-1, keepdims=True)
    wc = np.array([0.2, 0.5, 0.7]) ** gamma
    lam = np.maximum(0.0, n @ (light / np.linalg.norm(light)))
    ld = light - eye
    cos = np.maximum(0.0, np.sum(ld / np.linalg.norm(ld, axis=-1, keepdims=True) * n, -1))
    t1 = np.sum(n * -fe, -1)
    r = 1.0 / 1.33
    t2 = np.sqrt(1.0 - r * r * (1.0 - t1 * t1))
    rs = ((t1 - 1.33 * t2) / (t1 + 1.33 * t2)) ** 2
    rp = ((t2 - 1.33 * t1) / (t2 + 1.33 * t1)) ** 2
    F = np.clip((rs + rp) / 2.0, 0.0, 1.0)
    ab = np.exp(-np.asarray(thick, np.float64) * 0.075)
    out = np.empty((H, W, 4))
    for c in range(3):
        absorb = li[c] * (wc[c] + wc[c] * cos) * ab
        surf = (lam + 0.2) * absorb * (1 - F) + F * env[c] / 2.0
        out[..., c] = (surf * 0.5 + bg[c] / 2.0 * 0.5) ** (1.0 / gamma)
    absorb_a = (1.0 + cos) * ab
    out[..., 3] = ((lam + 0.2) * absorb_a * (1 - F) + F / 2.0) * 0.5 + 0.25
    empty = (Z <= 0) | (Z == 1)
    out[empty] = [bg[0], bg[1], bg[2], 1.0]
    return out.astype(f32)


FOAM_THRESHOLD = f32(0.05)


def foam(pos, clr, mv, pr, W, H, radius, scale, rgba):
    """The foam overlay over `rgba` ((H, W, 4), row 0 at the bottom):
    returns (rgba with the foam drawn, foam depth with 1.0 where none).

    Foam.vs: eye = ModelView * (x, y, z, w) with the particle's own w; the
    size from |ModelView * (x, y, z, 1)|.  Foam.gs: copy k of the point at
    gl_Position + vec4(-k) for every k < clr.x, at most max_vertices = 2, in
    draw order after the particle's earlier copies.  Foam.fs: normal.xy from
    gl_PointCoord, discard where its length d > clamp(w / 0.05, 0, 1),
    normal.z = sqrt(1 - d), the sphere point eye + normal * r / H projected
    and linearised with near 0.1 and far 1000; colour (1, 1, 1, 1) for
    w >= 0.05, else (1, 1, 1, 1 - w / 0.05).  The last fragment in draw order
    stays.  Single precision in the kernel's operation order.
    """
    p = np.asarray(pos, f32)
    w = np.asarray(clr, f32)[:, 0]
    n = len(p)
    one = np.ones(n, f32)
    ex, ey, ez, ew = _mul4(mv, p[:, 0], p[:, 1], p[:, 2], p[:, 3])
    qx, qy, qz, _ = _mul4(mv, p[:, 0], p[:, 1], p[:, 2], one)
    cx, cy, cz, cw = _mul4(pr, ex, ey, ez, ew)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        dist = np.sqrt(((qx * qx + qy * qy).astype(f32) + (qz * qz)).astype(f32)).astype(f32)
        r = (f32(scale) * (f32(radius) / dist).astype(f32)).astype(f32)
        size = np.fmin(np.fmax(r, f32(1)), f32(1024)).astype(f32)  # fminf / fmaxf: NaN -> 1
    out = np.array(rgba, f32, copy=True)
    depth = np.ones((H, W), f32)
    near, far = f32(0.1), f32(1000)
    for i in range(n):
        for k in (0, 1):
            if not (f32(k) < w[i]):
                continue
            c = [f32(v + f32(-k)) for v in (cx[i], cy[i], cz[i], cw[i])]
            if not (c[3] > 0) or abs(c[0]) > c[3] or abs(c[1]) > c[3] or abs(c[2]) > c[3]:
                continue
            wx = f32(f32(f32(c[0] / c[3]) + f32(1)) * f32(f32(0.5) * f32(W)))
            wy = f32(f32(f32(c[1] / c[3]) + f32(1)) * f32(f32(0.5) * f32(H)))
            sz = size[i]
            h = f32(0.5) * sz
            x0 = max(int(np.ceil(f32(f32(wx - h) - f32(0.5)))), 0)
            x1 = min(int(np.ceil(f32(f32(wx + h) - f32(0.5)))) - 1, W - 1)
            y0 = max(int(np.ceil(f32(f32(wy - h) - f32(0.5)))), 0)
            y1 = min(int(np.ceil(f32(f32(wy + h) - f32(0.5)))) - 1, H - 1)
            if x1 < x0 or y1 < y0:
                continue
            py, px = np.mgrid[y0:y1 + 1, x0:x1 + 1]
            sx = (f32(0.5) + ((px.astype(f32) + f32(0.5)).astype(f32) - wx).astype(f32) / sz).astype(f32)
            ty = (f32(0.5) - ((py.astype(f32) + f32(0.5)).astype(f32) - wy).astype(f32) / sz).astype(f32)
            nx = ((sx - f32(0.5)).astype(f32) * f32(2)).astype(f32)
            ny = ((ty - f32(0.5)).astype(f32) * f32(2)).astype(f32)
            d = np.sqrt(((nx * nx).astype(f32) + (ny * ny).astype(f32)).astype(f32)).astype(f32)
            fac = f32(min(max(f32(w[i] / FOAM_THRESHOLD), f32(0)), f32(1)))
            keep = ~(d > fac)
            if not keep.any():
                continue
            with np.errstate(invalid="ignore"):
                nz = np.sqrt((f32(1) - d).astype(f32)).astype(f32)
            l = np.sqrt((((nx * nx).astype(f32) + (ny * ny).astype(f32)).astype(f32)
                         + (nz * nz).astype(f32)).astype(f32)).astype(f32)
            ux, uy, uz = (nx / l).astype(f32), (-ny / l).astype(f32), (nz / l).astype(f32)
            fh = f32(H)
            fx = (ex[i] + ((ux * r[i]).astype(f32) / fh).astype(f32)).astype(f32)
            fy = (ey[i] + ((uy * r[i]).astype(f32) / fh).astype(f32)).astype(f32)
            fz = (ez[i] + ((uz * r[i]).astype(f32) / fh).astype(f32)).astype(f32)
            _, _, pz, pw = _mul4(pr, fx, fy, fz, np.ones_like(fx))
            dd = (pz / pw).astype(f32)
            z01 = ((dd * f32(0.5)).astype(f32) + f32(0.5)).astype(f32)
            den = (f32(far + near) - (z01 * f32(far - near)).astype(f32)).astype(f32)
            fd = (f32(f32(2) * near) / den).astype(f32)
            a = f32(1) if w[i] >= FOAM_THRESHOLD else f32(f32(1) - fac)
            sub_c = out[y0:y1 + 1, x0:x1 + 1]
            sub_d = depth[y0:y1 + 1, x0:x1 + 1]
            sub_c[keep] = np.array([1, 1, 1, a], f32)
            sub_d[keep] = np.fmin(np.fmax(fd, f32(0)), f32(1))[keep]
    return out, depth
