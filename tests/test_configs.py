"""The synthetic workloads the bench and the tests are quoted on: particle
counts, grids and constants as the bench line and the docs state them, every
particle inside its box, and the ensemble's size rules."""
import numpy as np

from pibiti_gb300 import configs
from pibiti_gb300.sph import Scene


def _inside(w, p):
    lo = np.array([p.worldMin.x, p.worldMin.y, p.worldMin.z], np.float32)
    hi = np.array([p.worldMax.x, p.worldMax.y, p.worldMax.z], np.float32)
    return np.all((w.pos[:, :3] > lo) & (w.pos[:, :3] < hi))


def test_dam_break_32k():
    w = configs.dambreak_small()
    p = Scene.parse(w.xml).params
    assert w.n == 32768 == p.numParticles and _inside(w, p)
    assert (p.gridSize.x, p.gridSize.y, p.gridSize.z) == (22, 22, 22)
    assert p.numCells == 22 ** 3 and p.numCells < 65536  # two sort passes


def test_double_dam_break_1m():
    w = configs.dambreak_double()
    p = Scene.parse(w.xml).params
    assert w.n == 1048576 == p.numParticles and _inside(w, p)
    assert (p.gridSize.x, p.gridSize.y, p.gridSize.z) == (132, 75, 38)
    assert p.numCells == 376200
    assert p.h == np.float32(0.0457) and p.restDensity == 1000.0 and p.maxParInCell == 16
    assert p.stiffness == 3.0 and p.viscosity == np.float32(3.5) and p.timeStep == np.float32(1e-3)
    assert np.all(w.vel == 0) and np.all(w.pos[:, 3] == 1)


def test_uniform_block_grid():
    w = configs.uniform_stress(n=1 << 16)  # the 16.7M case at a CPU-test size
    p = Scene.parse(w.xml).params
    assert w.n == p.numParticles == 1 << 16 and _inside(w, p)
    assert np.all(w.pos[:, 1] <= 0.6 + 1e-6)  # the lower 60% of the 1 m height


def test_ensemble_rules():
    e = configs.ensemble()
    assert len(e.xmls) == len(e.sizes) == 256 and e.n == sum(e.sizes)
    assert all(s % 512 == 0 and 4096 <= s <= 65536 for s in e.sizes)
    ps = [Scene.parse(x).params for x in e.xmls[:16]]
    assert all(p.numParticles == s for p, s in zip(ps, e.sizes))
    assert all(1.0 <= p.stiffness <= 5.0 and 1.0 <= p.viscosity <= 6.0 for p in ps)
