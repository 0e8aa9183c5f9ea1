"""The learned 4x dt step: features, the density-check fallback, and the
gain of a trained network over the coarse step without it."""
import numpy as np
import pytest

from pibiti_gb300 import configs, learned
from pibiti_gb300.sph import ARRAY_POS, ARRAY_VEL, SPH, Scene

pytestmark = pytest.mark.gpu


def _sys(xml, pos, vel):
    s = SPH(Scene.parse(xml).params)
    s.set_array(ARRAY_POS, pos)
    s.set_array(ARRAY_VEL, vel)
    return s


def test_features(cuda):
    torch = cuda
    w = configs.dambreak_small(side=12)
    with _sys(w.xml, w.pos, w.vel) as s:
        s.update(10)
        f = torch.empty((s.n, 16), dtype=torch.float32, device="cuda")
        ids = torch.empty(s.n, dtype=torch.int32, device="cuda")
        learned.features_step(s, f, ids)
        dens, _ = s.fields()
        f = f.cpu().numpy()
        ids = ids.cpu().numpy()
        p = s.params()
    assert np.isfinite(f).all()
    assert np.array_equal(np.sort(ids), np.arange(len(ids)))
    np.testing.assert_allclose(f[:, 0], dens / p.restDensity - 1, rtol=1e-6, atol=1e-6)
    assert f[:, 2].max() > 0.2  # neighbour counts / 64


def test_featured_walks_agree(cuda):
    """The featured force pass of the field walk (walk shape 4) and of the
    row walk (shape 1) accumulate the same sums in the same order: features,
    ids and the learned steps that follow are the same bits."""
    torch = cuda
    w = configs.dambreak_small(side=32)
    model = learned.Model.load()
    out = {}
    for shape in (1, 4):
        with _sys(w.xml, w.pos, w.vel) as s:
            s.set_walk_shape(shape)
            s.update(30)
            f = torch.empty((s.n, 16), dtype=torch.float32, device="cuda")
            ids = torch.empty(s.n, dtype=torch.int32, device="cuda")
            learned.features_step(s, f, ids)
            model.install(s)
            fb = learned.learned_step(s, 10, 4, 0.02)
            out[shape] = (f.cpu().numpy(), ids.cpu().numpy(), s.get_array(ARRAY_POS),
                          s.get_array(ARRAY_VEL), fb)
    for a, b in zip(out[1], out[4]):
        assert np.array_equal(a, b)


def test_fallback_reproduces_fine_steps(cuda):
    """With tol = 0 every coarse step fails the density check, is undone and
    replaced by 4 plain steps: the result equals 12 plain steps bit for bit."""
    w = configs.dambreak_small(side=12)
    model = learned.Model(np.zeros(5443, np.float32), np.zeros(16, np.float32),
                          np.ones(16, np.float32), np.ones(3, np.float32), {})
    with _sys(w.xml, w.pos, w.vel) as a, _sys(w.xml, w.pos, w.vel) as b:
        a.update(1)
        b.update(1)
        model.install(a)
        fb = learned.learned_step(a, 3, 4, tol=0.0)
        b.update(12)
        assert fb == 3
        np.testing.assert_array_equal(a.get_array(ARRAY_POS), b.get_array(ARRAY_POS))
        np.testing.assert_array_equal(a.get_array(ARRAY_VEL), b.get_array(ARRAY_VEL))


def test_nonfinite_corrections_fall_back(cuda):
    """NaN network outputs (here from NaN output biases; the tcgen05 forward
    pass also writes NaN rows when a wait for the tensor cores runs out) make
    the corrected state non-finite: with a density tolerance that never
    fails, the finiteness check alone rejects every coarse step, and the
    result equals the plain steps bit for bit."""
    w = configs.dambreak_small(side=12)
    params = np.zeros(5443, np.float32)
    params[5440:5443] = np.nan  # b3
    model = learned.Model(params, np.zeros(16, np.float32), np.ones(16, np.float32),
                          np.ones(3, np.float32), {})
    with _sys(w.xml, w.pos, w.vel) as a, _sys(w.xml, w.pos, w.vel) as b:
        a.update(1)
        b.update(1)
        model.install(a)
        fb = learned.learned_step(a, 3, 4, tol=1e9)
        b.update(12)
        assert fb == 3
        np.testing.assert_array_equal(a.get_array(ARRAY_POS), b.get_array(ARRAY_POS))
        np.testing.assert_array_equal(a.get_array(ARRAY_VEL), b.get_array(ARRAY_VEL))


def test_training_lowers_loss(cuda):
    """The project's own forward/backward kernels and Adam, run on a small
    ensemble, lower the training loss."""
    e = configs.ensemble(scenes=8, nmin=4096, nmax=8192, seed=3)
    f, t = learned.generate(e.xmls, e.pos, e.vel, e.sizes, snapshots=4)
    model = learned.train(f, t, epochs=4, batch=16384)
    h = model.info["loss_history"]
    assert np.isfinite(model.params).all()
    assert h[-1] < 0.9 * h[0], h


def test_trained_network_gains(cuda):
    """The shipped network (trained on the 256-scene ensemble with the
    project's kernels) against the same coarse step without it, on dam
    breaks it has not seen: one coarse step's velocity error against four
    dt steps, early (40 steps in) for two sizes; and over 200 coarse steps
    of a 32,768-particle dam break, the time-mean of the mean-density error
    relative to the fine-dt run.  Also: the drift correction alone halves
    the one-step position error."""
    model = learned.Model.load()
    for side, seed in ((16, 9), (24, 11)):
        w = configs.dambreak_small(side=side, seed=seed)
        err = learned.one_step_errors(model, w.xml, w.pos, w.vel)
        assert err["dv_learned"] < 0.9 * err["dv_coarse"], (side, err)
        assert err["dx_drift"] < 0.5 * err["dx_coarse"], (side, err)
    w = configs.dambreak_small(side=32, seed=13)
    r = learned.rollout(model, w.xml, w.pos, w.vel, 800, tol=1e9)
    assert r["err_learned_mean"] < 0.8 * r["err_drift_mean"], r
