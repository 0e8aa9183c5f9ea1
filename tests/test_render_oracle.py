"""The NumPy restatement of the foam overlay (oracle/render.py foam), on the
CPU: what Foam.vs / Foam.gs / Foam.fs draw for single particles, checked
against the shaders' formulas evaluated independently in double precision.
"""
import math

import numpy as np

from oracle import render as orender
from pibiti_gb300.render import look_at, perspective, point_scale

W, H = 64, 48
R = 0.1


def _view():
    mv = look_at((0.0, 0.0, 3.0), (0.0, 0.0, 0.0))
    pr = perspective(40.0, W / H, 0.1, 10.0)
    return mv, pr, point_scale(H, 40.0)


def _foam(pos, wvals, base=None):
    mv, pr, sc = _view()
    pos = np.asarray(pos, np.float32).reshape(-1, 4)
    clr = np.zeros((len(pos), 4), np.float32)
    clr[:, 0] = wvals
    if base is None:
        base = np.zeros((H, W, 4), np.float32)
    return orender.foam(pos, clr, mv, pr, W, H, R, sc, base)


def test_no_foam_leaves_the_frame():
    base = np.random.default_rng(0).uniform(size=(H, W, 4)).astype(np.float32)
    for w in (0.0, -1.0, np.nan):
        out, d = _foam([0, 0, 0, 1], [w], base)
        np.testing.assert_array_equal(out, base)
        assert np.all(d == 1)


def test_full_disc_and_alpha():
    """w >= 0.05: one copy (k = 1 needs w > 1), a full disc of the point's
    size, colour (1, 1, 1, 1)."""
    out, d = _foam([0, 0, 0, 1], [0.5])
    drawn = d < 1
    size = point_scale(H, 40.0) * (R / 3.0)
    assert abs(drawn.sum() - math.pi * (size / 2) ** 2) < 2.5 * size
    assert np.all(out[drawn] == 1)


def test_partial_disc_alpha():
    """w < 0.05: the disc is cut to radius w / 0.05 and alpha is 1 - w / 0.05."""
    full = (_foam([0, 0, 0, 1], [0.5])[1] < 1).sum()
    out, d = _foam([0, 0, 0, 1], [0.025])
    drawn = d < 1
    assert abs(drawn.sum() - full / 4) < 0.2 * full
    np.testing.assert_allclose(out[drawn][:, 3], 0.5, rtol=1e-6)
    np.testing.assert_array_equal(out[drawn][:, :3], 1)


def test_second_copy():
    """w > 1 draws a second copy at clip position gl_Position - 1; w > 2
    draws no third (max_vertices = 2)."""
    one = (_foam([0.2, 0.1, 0, 1], [1.0])[1] < 1).sum()
    two = (_foam([0.2, 0.1, 0, 1], [1.5])[1] < 1).sum()
    three = (_foam([0.2, 0.1, 0, 1], [7.0])[1] < 1).sum()
    assert two > one and three == two


def test_last_fragment_wins():
    """Blending off and depth test GL_ALWAYS: the later particle's colour
    stays, also when it lies behind the earlier one."""
    pos = [[0, 0, 0.5, 1], [0, 0, -0.5, 1]]
    out, d = _foam(pos, [0.5, 0.03])
    near_alone = _foam(pos[:1], [0.5])[1]
    far_alone = _foam(pos[1:], [0.03])[1]
    both = (near_alone < 1) & (far_alone < 1)
    assert both.any() and np.all(near_alone[both] < far_alone[both])
    np.testing.assert_allclose(out[both][:, 3], 0.4, rtol=1e-6)
    np.testing.assert_array_equal(d[both], far_alone[both])


def test_fragment_depth():
    """gl_FragDepth of every drawn pixel against Foam.fs evaluated in double
    precision: normal from gl_PointCoord, normal.z = sqrt(1 - |normal.xy|),
    the eye point moved by normal * r / H, projected, linearised with near 0.1
    and far 1000."""
    mv, pr, sc = _view()
    p = np.array([0.1, -0.05, 0.2, 1.0])
    out, d = _foam(p, [0.5])
    M = np.asarray(mv, np.float64).reshape(4, 4).T
    P = np.asarray(pr, np.float64).reshape(4, 4).T
    e = M @ p
    r = sc * (R / np.linalg.norm(e[:3]))
    c = P @ e
    wx, wy = (c[0] / c[3] + 1) * W / 2, (c[1] / c[3] + 1) * H / 2
    size = min(max(r, 1.0), 1024.0)
    ys, xs = np.nonzero(d < 1)
    assert len(ys) > 10
    for y, x in zip(ys, xs):
        nx = ((0.5 + (x + 0.5 - wx) / size) - 0.5) * 2
        ny = ((0.5 - (y + 0.5 - wy) / size) - 0.5) * 2
        dist = math.hypot(nx, ny)
        n = np.array([nx, -ny, math.sqrt(1 - dist)])
        n /= np.linalg.norm(n)
        f = P @ np.append(e[:3] + n * r / H, 1.0)
        zn = f[2] / f[3]
        want = 0.2 / (1000.1 - (zn * 0.5 + 0.5) * 999.9)
        np.testing.assert_allclose(d[y, x], want, rtol=2e-5)


def test_sprite_size_rounding_order():
    """The sprite shaders compute pointRadius * (pointScale / dist) with the
    uniforms bound crossed (pointRadius = m_ParScale, pointScale =
    m_ParRadius, render_particles.cpp:274-275, :791-792): the size rounds
    as scale * (radius / dist), which differs from radius * (scale / dist)
    in the last bit for some distances."""
    f32 = np.float32
    mv = np.eye(4, dtype=np.float32).ravel()
    mv[14] = -2.0  # camera 2 units in front of the particles
    pr = perspective(60.0, 1.0, 0.1, 10.0)
    rng = np.random.default_rng(3)
    pos = np.ones((4000, 4), np.float32)
    pos[:, :2] = rng.uniform(-0.3, 0.3, (4000, 2))
    pos[:, 2] = rng.uniform(-0.5, 0.5, 4000)
    radius, scale = 0.0173, 93.7
    _, _, _, size = orender.project(pos, mv, pr, 256, 256, radius, scale)
    ex, ey, ez = pos[:, 0], pos[:, 1], (pos[:, 2] + f32(-2.0)).astype(f32)
    dist = np.sqrt(((ex * ex + ey * ey).astype(f32) + (ez * ez)).astype(f32)).astype(f32)
    ref = (f32(scale) * (f32(radius) / dist).astype(f32)).astype(f32)
    other = (f32(radius) * (f32(scale) / dist).astype(f32)).astype(f32)
    drawn = size > 0
    assert drawn.sum() > 3000
    np.testing.assert_array_equal(size[drawn], np.clip(ref, 1, 1024)[drawn])
    assert np.any(ref[drawn] != other[drawn])
