"""The persistent step (sph_set_persistent: k steps as one cooperative
launch) against the launch-per-stage path: the same bits for one scene, for
an ensemble of uneven scenes, and for crowded cells of every sort tier;
no barrier timeout (bit 2 of the flags); and a forced timeout that leaves
the handle usable."""
import numpy as np
import pytest

from pibiti_gb300 import configs
from pibiti_gb300.sph import ARRAY_POS, ARRAY_VEL, SPH, Scene

pytestmark = pytest.mark.gpu


def _run(params, pos, vel, steps, persistent):
    with SPH(params) as s:
        s.set_array(ARRAY_POS, pos)
        s.set_array(ARRAY_VEL, vel)
        if persistent:
            s.set_persistent(True)
        for k in steps:
            s.update(k)
        out = s.get_array(ARRAY_POS), s.get_array(ARRAY_VEL), s.cells()[0], s.flags()
    return out


def _same(a, b):
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(a[2], b[2])
    assert not (b[3] & 4), "persistent barrier timed out"


def test_barrier_timeout_leaves_handle_usable(cuda):
    """Block 0 withheld from the barriers (test hook): the other blocks'
    bounded waits run out, flag bit 2 is set, the state does not advance,
    and the handle then steps exactly as the launch-per-stage path does."""
    import ctypes
    from pibiti_gb300 import _lib
    w = configs.dambreak_small(side=16)
    p = Scene.parse(w.xml).params
    expect = _run(p, w.pos, w.vel, [10], False)
    with SPH(p) as s:
        s.set_array(ARRAY_POS, w.pos)
        s.set_array(ARRAY_VEL, w.vel)
        s.set_persistent(True)
        flags = ctypes.c_uint32(0)
        _lib.check(_lib.lib().sph_persistent_withheld(s._h, ctypes.byref(flags)))
        assert flags.value & 4
        np.testing.assert_array_equal(s.get_array(ARRAY_POS), np.asarray(w.pos, np.float32))
        np.testing.assert_array_equal(s.get_array(ARRAY_VEL), np.asarray(w.vel, np.float32))
        s.update(10)
        got = s.get_array(ARRAY_POS), s.get_array(ARRAY_VEL), s.cells()[0], s.flags()
    _same(expect, got)


@pytest.mark.parametrize("steps", [[40], [7, 1, 12]])
def test_single_scene(cuda, steps):
    w = configs.dambreak_small(side=16)
    p = Scene.parse(w.xml).params
    _same(_run(p, w.pos, w.vel, steps, False), _run(p, w.pos, w.vel, steps, True))


def test_uneven_ensemble(cuda):
    ws = [configs.dambreak_small(side=s, seed=i) for i, s in enumerate((8, 13, 20))]
    ps = []
    for i, w in enumerate(ws):
        p = Scene.parse(w.xml).params
        p.stiffness = 1.0 + 2 * i
        ps.append(p)
    pos = np.concatenate([w.pos for w in ws])
    vel = np.concatenate([w.vel for w in ws])
    _same(_run(ps, pos, vel, [25], False), _run(ps, pos, vel, [25], True))


def test_crowded_cells(cuda):
    rng = np.random.default_rng(5)
    h = configs.H_DAMBREAK
    parts = [rng.uniform([lo] * 3, [lo + 0.3 * h] * 3, (n, 3))
             for lo, n in ((0.30, 20000), (0.51, 3000), (0.71, 600))]
    parts.append(rng.uniform([0.15] * 3, [0.85] * 3, (6400, 3)))
    pos = np.ones((30000, 4), np.float32)
    pos[:, :3] = np.concatenate(parts)
    pos = pos[rng.permutation(len(pos))]
    vel = np.zeros_like(pos)
    p = Scene.parse(configs.scene_xml(**configs.dambreak_attrs(len(pos), (0, 0, 0), (1, 1, 1)))).params
    _same(_run(p, pos, vel, [3], False), _run(p, pos, vel, [3], True))
