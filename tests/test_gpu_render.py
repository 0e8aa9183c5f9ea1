"""The headless screen-space renderer (sph_render_*) against the NumPy
restatement of the reference's GL pipeline (oracle/render.py).

Depth and coverage: bit for bit (the same single-precision operations).
Thickness: within 1e-5 relative (exp of CUDA vs NumPy).  Smoothed depth:
within 2e-6 per curvature-flow pass and 1e-5 after the bilateral passes (the
restatement evaluates those in double precision).  Colour: within 2e-4.
Foam overlay (colour and depth): bit for bit.
"""
import numpy as np
import pytest

from oracle import render as orender
from pibiti_gb300 import configs
from pibiti_gb300.render import Renderer, look_at, perspective

pytestmark = pytest.mark.gpu

W, H = 96, 64
ENV, BG = (0.6, 0.7, 0.8), (0.1, 0.1, 0.12)


def _scene(n=400, seed=0):
    rng = np.random.default_rng(seed)
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = rng.uniform([0.2, 0.1, 0.2], [0.8, 0.6, 0.8], size=(n, 3))
    pos[:5, :3] = [0.5, 0.35, -30.0]  # behind the camera: clipped
    mv = look_at((0.5, 0.8, 2.0), (0.5, 0.35, 0.5))
    pr = perspective(50.0, W / H, 0.1, 10.0)
    return pos, mv, pr


def _frame(torch, pos, mv, pr, w=W, h=H, **kw):
    with Renderer(w, h) as r:
        p = r.params(mv, pr, radius=0.03, env=ENV, background=BG, **kw)
        d, t, c = r.frame_params(torch.from_numpy(pos).cuda(), p)
        frags = r.fragments
    return d.cpu().numpy(), t.cpu().numpy(), c.cpu().numpy(), p, frags


@pytest.mark.parametrize("w,h", [(W, H), (101, 70)])  # 101 x 70: partial 16 x 16 tiles
def test_gbuffer_and_shading(cuda, w, h):
    pos, mv, pr = _scene()
    pr = perspective(50.0, w / h, 0.1, 10.0)
    d, t, c, p, frags = _frame(cuda, pos, mv, pr, w, h, method=0)
    sprites = orender.project(pos, mv, pr, w, h, 0.03, p.point_scale)
    od, ot = orender.gbuffer(sprites, w, h)
    assert (od < 1).sum() > w * h // 20
    assert frags > (od < 1).sum()  # overlapping sprites
    assert frags == orender.fragment_count(sprites, w, h)
    np.testing.assert_array_equal(d, od)
    np.testing.assert_allclose(t, ot, rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(c, orender.shade(od, ot, mv, pr, ENV, BG), rtol=0, atol=2e-4)


def test_crowded_tiles(cuda):
    """Tile lists past the warp-sort (1024) and the shared-memory-sort
    (16384) limits: 30,000 sprites of 6-9 px over a 64 x 48 image, about
    20,000 in each of the two middle tiles."""
    torch = cuda
    rng = np.random.default_rng(5)
    n = 30000
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = rng.uniform([0.3, 0.2, 0.3], [0.7, 0.5, 0.7], size=(n, 3))
    mv = look_at((0.5, 0.35, 1.6), (0.5, 0.35, 0.5))
    pr = perspective(50.0, 64 / 48, 0.1, 10.0)
    with Renderer(64, 48) as r:
        p = r.params(mv, pr, radius=0.1, method=0)
        d, t, _ = (x.cpu().numpy() for x in r.frame_params(torch.from_numpy(pos).cuda(), p))
        frags = r.fragments
    sprites = orender.project(pos, mv, pr, 64, 48, 0.1, p.point_scale)
    od, ot = orender.gbuffer(sprites, 64, 48)
    assert frags == orender.fragment_count(sprites, 64, 48)
    np.testing.assert_array_equal(d, od)
    np.testing.assert_allclose(t, ot, rtol=1e-5, atol=1e-9)


@pytest.mark.parametrize("iters", [1, 6])
def test_curvature_flow(cuda, iters):
    pos, mv, pr = _scene(seed=1)
    d, t, c, p, _ = _frame(cuda, pos, mv, pr, method=1, iterations=iters)
    od, ot = orender.gbuffer(orender.project(pos, mv, pr, W, H, 0.03, p.point_scale), W, H)
    for _ in range(iters):
        od = orender.curvature(od)
    np.testing.assert_allclose(d, od, rtol=0, atol=2e-6 * iters)
    assert np.any(d != orender.gbuffer(orender.project(pos, mv, pr, W, H, 0.03, p.point_scale), W, H)[0])


def test_bilateral(cuda):
    pos, mv, pr = _scene(seed=2)
    d, t, c, p, _ = _frame(cuda, pos, mv, pr, method=2, iterations=2, kernel_center=3, sigma=0.01)
    od, ot = orender.gbuffer(orender.project(pos, mv, pr, W, H, 0.03, p.point_scale), W, H)
    for _ in range(2):
        od = orender.bilateral(od, 3, 0.01)
    np.testing.assert_allclose(d, od, rtol=0, atol=1e-5)


def test_dam_break_frame(cuda):
    """A 32,768-particle dam break after 50 steps at 320x240: deterministic,
    finite, depth in [0, 1], the fluid covers part of the image."""
    torch = cuda
    from pibiti_gb300.sph import ARRAY_POS, ARRAY_VEL, SPH, Scene
    w = configs.dambreak_small(side=32)
    with SPH(Scene.parse(w.xml).params) as s:
        s.set_array(ARRAY_POS, w.pos)
        s.set_array(ARRAY_VEL, w.vel)
        s.update(50)
        pos = torch.empty((s.n, 4), dtype=torch.float32, device="cuda")
        s.get_array(ARRAY_POS, out=pos)
    mv = look_at((0.5, 0.6, 1.8), (0.5, 0.2, 0.5))
    pr = perspective(60.0, 320 / 240, 0.1, 10.0)
    with Renderer(320, 240) as r:
        a = [x.cpu().numpy() for x in r.frame(pos, mv, pr, radius=0.02, method=1, iterations=4)]
        b = [x.cpu().numpy() for x in r.frame(pos, mv, pr, radius=0.02, method=1, iterations=4)]
        assert r.fragments > 0
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    depth, thick, rgba = a
    assert np.all((depth >= 0) & (depth <= 1)) and np.isfinite(rgba).all()
    assert 0.05 < (depth < 1).mean() < 0.95


def test_nothing_visible(cuda):
    """Every particle behind the camera: no fragment, depth 1, background."""
    torch = cuda
    pos = np.ones((50, 4), np.float32)
    pos[:, :3] = [0.5, 0.35, 30.0]
    mv = look_at((0.5, 0.8, 2.0), (0.5, 0.35, 0.5))
    pr = perspective(50.0, W / H, 0.1, 10.0)
    with Renderer(W, H) as r:
        d, t, c = (x.cpu().numpy() for x in r.frame(torch.from_numpy(pos).cuda(), mv, pr, radius=0.03,
                                                     background=BG))
        assert r.fragments == 0
    assert np.all(d == 1) and np.all(t == 0)
    np.testing.assert_allclose(c[..., :3], np.broadcast_to(np.array(BG, np.float32), (H, W, 3)))


FOAM_VALUES = np.array([0.0, np.nan, -0.5, 0.01, 0.03, 0.05, 0.3, 1.0, 1.5, 3.0], np.float32)


def _foam_scene(n=700, seed=3):
    rng = np.random.default_rng(seed)
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = rng.uniform([0.0, 0.0, 0.0], [1.0, 0.7, 1.0], size=(n, 3))
    pos[7:12, 3] = 0.5  # the foam shader's eye position uses the particle's own w
    clr = np.zeros((n, 4), np.float32)
    clr[:, 0] = FOAM_VALUES[rng.integers(0, len(FOAM_VALUES), n)]
    clr[:, 1:] = rng.uniform(0, 1, (n, 3))
    mv = look_at((0.5, 0.6, 4.0), (0.5, 0.35, 0.5))
    pr = perspective(40.0, W / H, 0.1, 10.0)
    return pos, clr, mv, pr


def test_foam_overlay(cuda):
    """sph_render_foam over a shaded frame against the restatement: every
    foam value case (none, NaN, negative, partial disc, full disc, a second
    copy at gl_Position - 1, more than two requested), overlapping sprites."""
    torch = cuda
    pos, clr, mv, pr = _foam_scene()
    with Renderer(W, H) as r:
        p = r.params(mv, pr, radius=0.12, env=ENV, background=BG, method=0)
        dp = torch.from_numpy(pos).cuda()
        _, _, rgba = r.frame_params(dp, p)
        base = rgba.cpu().numpy()
        fd = r.foam_params(dp, torch.from_numpy(clr).cuda(), p, rgba)
        got, gd = rgba.cpu().numpy(), fd.cpu().numpy()
    want, wd = orender.foam(pos, clr, mv, pr, W, H, 0.12, p.point_scale, base)
    drawn = wd < 1
    assert 50 < drawn.sum() < W * H - 50
    assert np.any(drawn & (want[..., 3] > 0) & (want[..., 3] < 1))  # partial discs on top
    np.testing.assert_array_equal(gd, wd)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(got[~drawn], base[~drawn])


def test_foam_none(cuda):
    """No foam value above 0: the frame is unchanged and the foam depth is 1;
    without a frame, only the depth is written."""
    torch = cuda
    pos, clr, mv, pr = _foam_scene(seed=4)
    clr[:, 0] = 0.0
    with Renderer(W, H) as r:
        p = r.params(mv, pr, radius=0.12, env=ENV, background=BG, method=0)
        dp = torch.from_numpy(pos).cuda()
        _, _, rgba = r.frame_params(dp, p)
        base = rgba.cpu().numpy()
        fd = r.foam_params(dp, torch.from_numpy(clr).cuda(), p, rgba)
        np.testing.assert_array_equal(rgba.cpu().numpy(), base)
        assert np.all(fd.cpu().numpy() == 1)
        clr[:, 0] = 0.5
        fd = r.foam_params(dp, torch.from_numpy(clr).cuda(), p, None)
    np.testing.assert_array_equal(fd.cpu().numpy(), orender.foam(pos, clr, mv, pr, W, H, 0.12, p.point_scale,
                                                                 base)[1])
