"""Edge cases of the fused step, each against the oracle's single-precision
step (the same IEEE operations, so bit for bit): one particle, coincident
particles (r = minDist clamp), particles exactly on cell faces, a cell
capacity of one (maxParInCell = 1), positions outside the world box, and
stage entry points called with no particles."""
import numpy as np
import pytest

import oracle
from pibiti_gb300 import configs
from pibiti_gb300.sph import ARRAY_POS, ARRAY_VEL, SPH, Scene

pytestmark = pytest.mark.gpu


def _run(p, pos, vel, steps):
    with SPH(p) as s:
        s.set_array(ARRAY_POS, pos)
        s.set_array(ARRAY_VEL, vel)
        s.update(steps)
        return s.get_array(ARRAY_POS), s.get_array(ARRAY_VEL), s.cells()


def _check(p, pos, vel, steps):
    gp, gv, (sh, _, _) = _run(p, pos, vel, steps)
    op, ov = oracle.step(p, pos, vel, steps=steps)
    np.testing.assert_array_equal(gp, op)
    np.testing.assert_array_equal(gv, ov)
    # the last step's structures: a stable sort of the hashes of the
    # positions that step integrated (the oracle's step before the last)
    prev_p, prev_v = oracle.step(p, pos, vel, steps=steps - 1) if steps > 1 else (pos, vel)
    ip, _ = oracle.integrate(p, prev_p, prev_v)
    np.testing.assert_array_equal(sh, oracle.sort_pairs(oracle.calc_hash(p, ip), 32))


def _base(side=8):
    w = configs.dambreak_small(side=side)
    return w, Scene.parse(w.xml).params


def test_single_particle(cuda):
    w, p = _base()
    p.numParticles = 1
    _check(p, w.pos[:1].copy(), w.vel[:1].copy(), 20)


def test_coincident_particles(cuda):
    w, p = _base()
    pos = w.pos.copy()
    pos[1::7, :3] = pos[0:len(pos) - 1:7, :3][: len(pos[1::7])]  # pairs at one point
    pos[100:110, :3] = pos[99, :3]  # eleven at one point
    _check(p, pos, w.vel, 10)


def test_particles_on_cell_faces(cuda):
    w, p = _base()
    p.gravity.y = 0.0
    cs = p.cellSize.x
    rng = np.random.default_rng(3)
    cells = rng.integers(3, 15, size=(len(w.pos), 3))
    pos = w.pos.copy()
    pos[:, :3] = (np.array([p.worldMin.x, p.worldMin.y, p.worldMin.z], np.float32)
                  + cells.astype(np.float32) * np.float32(cs))
    _check(p, pos, np.zeros_like(w.vel), 3)


def test_cell_capacity_one(cuda):
    w, p = _base(10)
    p.maxParInCell = 1
    _check(p, w.pos, w.vel, 10)


def test_positions_outside_the_box(cuda):
    w, p = _base()
    pos = w.pos.copy()
    pos[::5, 0] = p.worldMax.x + 0.3
    pos[1::9, 1] = p.worldMin.y - 0.2
    pos[2::11, 2] = p.worldMax.z + 5.0
    _check(p, pos, w.vel, 5)


def test_stage_calls_with_no_particles(cuda):
    torch = cuda
    from pibiti_gb300.sph import stage
    _, p = _base()
    stage.set_parameters(p)
    a = torch.zeros((1, 4), dtype=torch.float32, device="cuda")
    kv = torch.zeros((1, 2), dtype=torch.int32, device="cuda")
    cs = torch.zeros(p.numCells, dtype=torch.int32, device="cuda")
    f = torch.zeros(1, dtype=torch.float32, device="cuda")
    stage.integrate(a, a, a, a, 0)
    stage.calc_hash(a, kv, 0)
    stage.radix_sort(kv, kv.clone(), 0, 16)
    stage.reorder(a, a, a, a, kv, cs, 0, p.numCells)
    stage.collide(a, a, a, f, f, kv, cs, 0, p.numCells)
    stage.sync()
    assert torch.all(cs.view(torch.int32) == -1)  # reorder still clears cellStart
