"""GPU parity of the fused system step (sph_step) through the C ABI.

Against the golden fixtures (the reference's own kernels): sorted hash,
cellStart and integrated positions bit-exact; density within DENS_RTOL;
velocities within the force tolerance of test_gpu_stage.  Against the
oracle: multi-step trajectories, the ensemble, and size-independent
properties at the 1,048,576-particle workload.
"""
import numpy as np
import pytest

import oracle
from conftest import params_from
from pibiti_gb300 import configs
from pibiti_gb300.sph import ARRAY_POS, ARRAY_VEL, SPH, Scene

pytestmark = pytest.mark.gpu

DENS_RTOL = 1e-5
CASES = ["dambreak", "truncate", "features", "bigrid", "tiny", "rotor", "propeller", "hmapxz",
         "hmapyz"]


def system_from(p, pos, vel):
    s = SPH(p)
    s.set_array(ARRAY_POS, pos)
    s.set_array(ARRAY_VEL, vel)
    return s


@pytest.mark.parametrize("case", CASES)
def test_step_vs_reference(cuda, golden, case):
    g = golden(f"step_{case}.npz")
    p = params_from(g["params"])
    with system_from(p, g["pos_in"], g["vel_in"]) as s:
        s.update(1)
        pos, vel = s.get_array(ARRAY_POS), s.get_array(ARRAY_VEL)
        sh, cs, ce = s.cells()
        dens, pres = s.fields()
        flags = s.flags()
    np.testing.assert_array_equal(sh, g["sorted"])
    np.testing.assert_array_equal(cs, g["cell_start"])
    cnt = np.bincount(g["sorted"][:, 0], minlength=p.numCells)
    np.testing.assert_array_equal(ce[cnt > 0], g["cell_start"][cnt > 0] + cnt[cnt > 0])
    assert np.all(ce[cnt == 0] == 0xFFFFFFFF)
    np.testing.assert_array_equal(pos, g["pos"])
    d64, _ = oracle.density(p, g["sorted_pos"], g["sorted"], g["cell_start"], fp64=True)
    np.testing.assert_allclose(dens, d64, rtol=DENS_RTOL, atol=1e-2)
    np.testing.assert_allclose(dens, g["density"], rtol=DENS_RTOL, atol=1e-2)
    from test_gpu_stage import check_force
    check_force(p, g["sorted"], g["sorted_pos"], g["sorted_vel"], dens, pres, g["cell_start"], vel)
    # truncation is reported (bit 0) exactly when a cell overflowed
    overflow = cnt.max() > p.maxParInCell
    assert bool(flags & 1) == overflow


def test_multistep_matches_oracle(cuda):
    """100 steps of the 4,096-particle dam break: the fused GPU step and the
    single-precision oracle perform the same IEEE operations."""
    w = configs.dambreak_small(side=16)
    p = Scene.parse(w.xml).params
    with system_from(p, w.pos, w.vel) as s:
        s.update(100)  # graph-replayed pairs of steps
        pos, vel = s.get_array(ARRAY_POS), s.get_array(ARRAY_VEL)
    opos, ovel = oracle.step(p, w.pos, w.vel, steps=100)
    np.testing.assert_array_equal(pos, opos)
    np.testing.assert_array_equal(vel, ovel)


# Drift of the single-precision GPU trajectory from the double-precision
# one (oracle.step_fp64: the same step with the state and every stage in
# double), 1000 steps of the 32,768-particle dam break, sampled every 100
# steps.  Kinetic energy is compared against the run's largest kinetic
# energy (it falls by an order of magnitude after the impact near step 350,
# where the splash makes the two trajectories part); mean density relative.
# Measured: before the impact (steps <= 300) 2.2e-4 of the peak and 3e-4
# relative; over the whole run 3.5e-3 and 8.5e-3.
DRIFT_EARLY_STEPS = 300
DRIFT_KE_EARLY, DRIFT_KE_ALL = 1e-3, 1e-2      # |KE32 - KE64| / max KE64
DRIFT_RHO_EARLY, DRIFT_RHO_ALL = 1e-3, 2e-2    # |rho32 - rho64| / rho64


def test_drift_against_fp64_trajectory(cuda):
    w = configs.dambreak_small(side=32)
    p = Scene.parse(w.xml).params
    ke32, rho32 = [], []
    with system_from(p, w.pos, w.vel) as s:
        for _ in range(10):
            s.update(100)
            st = s.stats()[0]
            assert st[3] == 0
            ke32.append(st[0])
            rho32.append(st[1])
    ke64, rho64 = [], []
    pos, vel = w.pos, w.vel
    m = float(p.particleMass)
    for _ in range(10):
        pos, vel, md = oracle.step_fp64(p, pos, vel, steps=100, with_density=True)
        ke64.append(0.5 * m * float((vel[:, :3] ** 2).sum()))
        rho64.append(md)
    ke32, rho32, ke64, rho64 = map(np.asarray, (ke32, rho32, ke64, rho64))
    steps = 100 * np.arange(1, 11)
    early = steps <= DRIFT_EARLY_STEPS
    dke = np.abs(ke32 - ke64) / ke64.max()
    drho = np.abs(rho32 - rho64) / rho64
    assert dke[early].max() <= DRIFT_KE_EARLY, dke
    assert dke.max() <= DRIFT_KE_ALL, dke
    assert drho[early].max() <= DRIFT_RHO_EARLY, drho
    assert drho.max() <= DRIFT_RHO_ALL, drho
    # k=3 is soft: the 0.73 m column compresses to about twice rest density
    assert p.restDensity < rho32[-1] < 4 * p.restDensity


# Measured: kinetic energy 1.8e-6 and 5.7e-6, mean density 4.9e-6 and 2.5e-6
# (relative, at steps 100 and 200).
DRIFT_1M_STEPS = 200
DRIFT_1M_KE, DRIFT_1M_RHO = 1e-4, 1e-4          # relative, at steps 100 and 200


def test_drift_against_fp64_trajectory_1m(cuda):
    """200 steps of the 1,048,576-particle double dam break (the columns
    falling, before they meet): the GPU's kinetic energy and mean density
    against the double-precision trajectory's, every 100 steps."""
    w = configs.dambreak_double()
    p = Scene.parse(w.xml).params
    ke32, rho32 = [], []
    with system_from(p, w.pos, w.vel) as s:
        for _ in range(DRIFT_1M_STEPS // 100):
            s.update(100)
            st = s.stats()[0]
            assert st[3] == 0
            ke32.append(st[0])
            rho32.append(st[1])
    ke64, rho64 = [], []
    pos, vel = w.pos, w.vel
    m = float(p.particleMass)
    for _ in range(DRIFT_1M_STEPS // 100):
        pos, vel, md = oracle.step_fp64(p, pos, vel, steps=100, with_density=True)
        ke64.append(0.5 * m * float((vel[:, :3] ** 2).sum()))
        rho64.append(md)
    ke32, rho32, ke64, rho64 = map(np.asarray, (ke32, rho32, ke64, rho64))
    dke = np.abs(ke32 - ke64) / ke64
    drho = np.abs(rho32 - rho64) / rho64
    print("1M drift vs FP64: KE", dke, "mean density", drho)
    assert dke.max() <= DRIFT_1M_KE, dke
    assert drho.max() <= DRIFT_1M_RHO, drho


def test_stats_reductions_at_1m(cuda):
    """The GPU's kinetic-energy and mean-density reductions after 200 steps
    of the 1,048,576-particle double dam break, against double-precision sums
    of the same state read back to the host."""
    w = configs.dambreak_double()
    p = Scene.parse(w.xml).params
    with system_from(p, w.pos, w.vel) as s:
        s.update(200)
        st = s.stats()[0]
        vel = s.get_array(ARRAY_VEL).astype(np.float64)
        dens, _ = s.fields()
    ke = 0.5 * float(p.particleMass) * float((vel[:, :3] ** 2).sum())
    rho = float(dens.astype(np.float64).mean())
    assert abs(st[0] - ke) <= 1e-5 * ke
    assert abs(st[1] - rho) <= 1e-6 * rho
    assert st[3] == 0


@pytest.mark.parametrize("shape", [1, 4, 9])
def test_ensemble_equals_separate_runs(cuda, shape):
    """Three scenes of different size and parameters in one handle give the
    same bits as three separate handles (with a global, the default staged
    and the warp-cooperative walk: staged blocks over two scenes walk global
    memory)."""
    ws = [configs.dambreak_small(side=s, seed=i) for i, s in enumerate((8, 12, 16))]
    ps = []
    for i, w in enumerate(ws):
        p = Scene.parse(w.xml).params
        p.stiffness = 1.0 + i
        p.viscosity = 2.0 + i
        ps.append(p)
    with SPH(ps) as e:
        e.set_walk_shape(shape)
        e.set_array(ARRAY_POS, np.concatenate([w.pos for w in ws]))
        e.set_array(ARRAY_VEL, np.concatenate([w.vel for w in ws]))
        e.update(20)
        epos, evel = e.get_array(ARRAY_POS), e.get_array(ARRAY_VEL)
        offs = e.offsets
        sh, cs, ce = e.cells()
    for k, (w, p) in enumerate(zip(ws, ps)):
        with system_from(p, w.pos, w.vel) as s:
            s.update(20)
            np.testing.assert_array_equal(epos[offs[k]:offs[k + 1]], s.get_array(ARRAY_POS))
            np.testing.assert_array_equal(evel[offs[k]:offs[k + 1]], s.get_array(ARRAY_VEL))
            ssh, scs, _ = s.cells()
            np.testing.assert_array_equal(sh[offs[k]:offs[k + 1]], ssh)


def test_set_get_roundtrip(cuda):
    torch = cuda
    w = configs.dambreak_small(side=10)
    p = Scene.parse(w.xml).params
    with system_from(p, w.pos, w.vel) as s:
        np.testing.assert_array_equal(s.get_array(ARRAY_POS), w.pos)
        s.update(3)
        # partial write in original indices after the state has been permuted
        new = np.full((17, 4), 0.5, np.float32)
        s.set_array(ARRAY_VEL, new, start=100)
        v = s.get_array(ARRAY_VEL)
        np.testing.assert_array_equal(v[100:117], new)
        # device-to-device through torch tensors
        t = torch.empty((s.n, 4), dtype=torch.float32, device="cuda")
        s.get_array(ARRAY_POS, out=t)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(t.cpu().numpy(), s.get_array(ARRAY_POS))


def test_pinned_host_buffers_match_pageable(cuda):
    """Pinned host buffers (read and written by the GPU in one pass) give the
    records pageable buffers (staged through device memory) give: whole and
    partial writes after steps have permuted the stored order, and reads,
    for a three-scene handle."""
    torch = cuda
    ws = [configs.dambreak_small(side=s, seed=i) for i, s in enumerate((8, 12, 10))]
    ps = [Scene.parse(w.xml).params for w in ws]
    pos = np.concatenate([w.pos for w in ws])
    vel = np.concatenate([w.vel for w in ws])
    n = len(pos)
    hpos = torch.from_numpy(pos.copy()).pin_memory()
    hvel = torch.from_numpy(vel.copy()).pin_memory()
    with SPH(ps) as a, SPH(ps) as b:
        a.set_array(ARRAY_POS, hpos.numpy())
        a.set_array(ARRAY_VEL, hvel.numpy())
        b.set_array(ARRAY_POS, pos)
        b.set_array(ARRAY_VEL, vel)
        a.update(5)
        b.update(5)
        new = torch.full((333, 4), 0.25, dtype=torch.float32).pin_memory()
        a.set_array(ARRAY_VEL, new.numpy(), start=700)
        b.set_array(ARRAY_VEL, new.numpy().copy(), start=700)
        a.update(2)
        b.update(2)
        out_p = torch.empty((n, 4), dtype=torch.float32).pin_memory()
        out_v = torch.empty((n, 4), dtype=torch.float32).pin_memory()
        a.get_array(ARRAY_POS, out_p.numpy())
        a.get_array(ARRAY_VEL, out_v.numpy())
        np.testing.assert_array_equal(out_p.numpy(), b.get_array(ARRAY_POS))
        np.testing.assert_array_equal(out_v.numpy(), b.get_array(ARRAY_VEL))


def test_snapshot_resume(cuda, tmp_path):
    """A checkpoint after 20 steps, restored into a new handle, continues bit
    for bit like the uninterrupted run: the step keeps no state beyond the
    parameters, positions, velocities and original particle ids (one scene,
    and a three-scene ensemble)."""
    w = configs.dambreak_small(side=16)
    e = configs.ensemble(scenes=3, nmin=4096, nmax=8192, seed=7)
    cases = [(Scene.parse(w.xml).params, w.pos, w.vel),
             ([Scene.parse(x).params for x in e.xmls], e.pos, e.vel)]
    for k, (p, pos, vel) in enumerate(cases):
        path = str(tmp_path / f"snap{k}.npz")
        with SPH(p) as s:
            s.set_array(ARRAY_POS, pos)
            s.set_array(ARRAY_VEL, vel)
            s.update(20)
            s.snapshot(path, step=20, extra={"dye": np.arange(3)})
            s.update(20)
            want_pos, want_vel = s.get_array(ARRAY_POS), s.get_array(ARRAY_VEL)
        r, step, extra = SPH.restore(path)
        with r:
            assert step == 20 and list(extra["dye"]) == [0, 1, 2]
            r.update(20)
            np.testing.assert_array_equal(r.get_array(ARRAY_POS), want_pos)
            np.testing.assert_array_equal(r.get_array(ARRAY_VEL), want_vel)


def test_nan_is_flagged(cuda):
    w = configs.dambreak_small(side=8)
    p = Scene.parse(w.xml).params
    pos = w.pos.copy()
    pos[5, 1] = np.nan
    with system_from(p, pos, w.vel) as s:
        s.update(1)
        assert s.flags() & 2
        assert s.stats()[0][3] > 0


def test_grid_too_small_rejected(cuda):
    from pibiti_gb300 import _lib
    xml = configs.scene_xml(**configs.dambreak_attrs(64, (0, 0, 0), (0.1, 1.0, 1.0)))
    p = Scene.parse(xml).params
    with pytest.raises(_lib.SphError) as e:
        SPH(p)
    assert e.value.code == 3


def _check_structures(p, n, sh, cs, ce, dens, pos):
    """Size-independent properties of one step's neighbour structures: a
    stable sort of (hash, original index), cell ranges that partition the
    particles, hashes of the sorted positions, density against the
    double-precision oracle on the GPU's own sorted positions."""
    keys, ids = sh[:, 0].astype(np.int64), sh[:, 1].astype(np.int64)
    assert np.all(np.diff(keys) >= 0)
    same = np.diff(keys) == 0
    assert np.all(np.diff(ids)[same] > 0)
    assert np.array_equal(np.sort(ids), np.arange(n))
    cnt = np.bincount(keys, minlength=p.numCells)
    nz = cnt > 0
    starts = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    np.testing.assert_array_equal(cs[nz], starts[nz])
    np.testing.assert_array_equal(ce[nz], starts[nz] + cnt[nz])
    spos = pos[ids]
    np.testing.assert_array_equal(oracle.calc_hash(p, spos)[:, 0], sh[:, 0])
    kv = np.stack([sh[:, 0], ids.astype(np.uint32)], axis=1)
    d64, _ = oracle.density(p, spos, kv, cs, fp64=True)
    np.testing.assert_allclose(dens, d64, rtol=DENS_RTOL, atol=1e-2)


def test_million_particle_properties(cuda):
    """The 1,048,576-particle double dam break after 20 steps."""
    w = configs.dambreak_double(steps=20)
    p = Scene.parse(w.xml).params
    with system_from(p, w.pos, w.vel) as s:
        s.update(20)
        sh, cs, ce = s.cells()
        dens, _ = s.fields()
        pos = s.get_array(ARRAY_POS)
    _check_structures(p, len(w.pos), sh, cs, ce, dens, pos)


def test_stress_16m_properties(cuda):
    """The stress configuration at full size: 16,777,216 particles uniform-
    random in the lower 60% of a 4x1x4 box, h for ~40 neighbours (2.96 M
    cells, 32-bit keys), after 3 steps with the grid rebuilt every step."""
    w = configs.uniform_stress(steps=3)
    p = Scene.parse(w.xml).params
    assert p.numCells > 65536
    with system_from(p, w.pos, w.vel) as s:
        s.update(3)
        sh, cs, ce = s.cells()
        dens, _ = s.fields()
        pos = s.get_array(ARRAY_POS)
        st = s.stats()[0]
    assert st[3] == 0  # nothing non-finite
    _check_structures(p, len(w.pos), sh, cs, ce, dens, pos)


def test_full_ensemble_scenes_match_separate_runs(cuda):
    """The batched ensemble at full size (256 scenes, 4k-64k particles,
    5.3 M in all): after 10 steps in one handle, every scene's structures
    are a stable sort of (local hash, local index), and scenes 0, 127 and
    255 equal separate
    handles bit for bit (state and neighbour structures)."""
    e = configs.ensemble()
    ps = [Scene.parse(x).params for x in e.xmls]
    with SPH(ps) as h:
        h.set_array(ARRAY_POS, e.pos)
        h.set_array(ARRAY_VEL, e.vel)
        h.update(10)
        epos, evel = h.get_array(ARRAY_POS), h.get_array(ARRAY_VEL)
        offs = np.asarray(h.offsets, dtype=np.int64)
        sh, _, _ = h.cells()
    # hashes and original indices are local to each scene
    keys, ids = sh[:, 0].astype(np.int64), sh[:, 1].astype(np.int64)
    scene = np.repeat(np.arange(len(ps)), np.diff(offs))
    inner = scene[1:] == scene[:-1]
    dk = np.diff(keys)
    assert np.all(dk[inner] >= 0)
    assert np.all(np.diff(ids)[inner & (dk == 0)] > 0)
    np.testing.assert_array_equal(np.sort(ids + offs[scene]), np.arange(len(e.pos)))
    for k in (0, 127, 255):
        a, b = offs[k], offs[k + 1]
        with system_from(ps[k], e.pos[a:b], e.vel[a:b]) as s:
            s.update(10)
            np.testing.assert_array_equal(epos[a:b], s.get_array(ARRAY_POS))
            np.testing.assert_array_equal(evel[a:b], s.get_array(ARRAY_VEL))
            np.testing.assert_array_equal(sh[a:b], s.cells()[0])


def test_walk_shapes_and_graph_lengths_agree(cuda):
    """Every walk launch shape and every graph length gives the same bits."""
    w = configs.dambreak_small(side=12)
    p = Scene.parse(w.xml).params
    ref = None
    for shape in range(len(SPH.WALK_THREADS)):
        for gsteps in (2, 6):
            with system_from(p, w.pos, w.vel) as s:
                s.set_walk_shape(shape)
                s.set_graph_steps(gsteps)
                s.update(13)  # graph launches plus a direct remainder
                out = (s.get_array(ARRAY_POS), s.get_array(ARRAY_VEL))
            if ref is None:
                ref = out
            else:
                np.testing.assert_array_equal(out[0], ref[0])
                np.testing.assert_array_equal(out[1], ref[1])


@pytest.mark.parametrize("case", ["features", "truncate", "rotor", "propeller", "hmapxz", "hmapyz", "bigrid"])
def test_walk_shapes_agree_on_golden_scenes(cuda, golden, case):
    """The golden scenes (colliders, accelerators, rotors, height maps,
    truncated cells, a 32-bit hash grid) step to the same bits with every
    walk shape as with the default one, which test_step_vs_reference checks
    against the reference."""
    g = golden(f"step_{case}.npz")
    p = params_from(g["params"])
    outs = []
    for shape in range(len(SPH.WALK_THREADS)):
        with system_from(p, g["pos_in"], g["vel_in"]) as s:
            s.set_walk_shape(shape)
            s.update(2)
            outs.append((s.get_array(ARRAY_POS), s.get_array(ARRAY_VEL), s.fields()[0]))
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            np.testing.assert_array_equal(a, b)


def test_staged_walks_match_global_walks_on_sparse_particles(cuda):
    """Particles strewn over many cells: blocks of the staged walks whose
    cells span too large a box walk global memory instead; every shape gives
    the bits of the one-particle-per-thread walk."""
    rng = np.random.default_rng(11)
    w = configs.dambreak_small(side=16)
    p = Scene.parse(w.xml).params
    pos = w.pos.copy()
    pos[:, :3] = rng.uniform(0.05, 0.95, size=(len(pos), 3)).astype(np.float32)
    pos[:2048, :3] = pos[:2048, :3] * 0.2 + 0.1  # a crowded corner too
    # and particles in the grid's first cells along every axis (their
    # neighbour cells at -1 lie outside the grid; cell 0 itself stays empty)
    cs = p.cellSize.x
    edge = rng.uniform(0.2, 0.8, size=(256, 3)).astype(np.float32) * cs
    edge[:128, 0] += cs  # cells (1, 0, 0)
    edge[128:, 1] += cs  # cells (0, 1, 0)
    pos[2048:2304, :3] = edge
    vel = rng.normal(0.0, 0.5, size=pos.shape).astype(np.float32)
    outs = []
    for shape in range(len(SPH.WALK_THREADS)):
        with system_from(p, pos, vel) as s:
            s.set_walk_shape(shape)
            s.update(3)
            outs.append((s.get_array(ARRAY_POS), s.get_array(ARRAY_VEL), s.fields()[0]))
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            np.testing.assert_array_equal(a, b)


def test_autotune_keeps_state(cuda):
    w = configs.dambreak_small(side=12)
    p = Scene.parse(w.xml).params
    with system_from(p, w.pos, w.vel) as a, system_from(p, w.pos, w.vel) as b:
        a.update(5)
        b.update(5)
        chosen, ms = a.autotune(trial_steps=4)
        assert 0 <= chosen < len(SPH.WALK_THREADS) and all(m > 0 for m in ms)
        assert a.walk_shape() == chosen
        a.update(7)
        b.update(7)
        np.testing.assert_array_equal(a.get_array(ARRAY_POS), b.get_array(ARRAY_POS))
        np.testing.assert_array_equal(a.get_array(ARRAY_VEL), b.get_array(ARRAY_VEL))


def test_crowded_cells_keep_stable_order(cuda):
    """Cells of every size tier (<= 32, <= 1024, <= 16384 and beyond, the
    last sorted through global scratch) come out in (hash, original index)
    order, as the reference's stable sort leaves them."""
    rng = np.random.default_rng(5)
    h = configs.H_DAMBREAK
    # clusters inside single cells (cell = h): 20000, 3000 and 600 particles
    def cluster(lo, n):
        return rng.uniform([lo] * 3, [lo + 0.3 * h] * 3, (n, 3))
    parts = [cluster(0.30, 20000), cluster(0.51, 3000), cluster(0.71, 600),
             rng.uniform([0.15, 0.15, 0.15], [0.85, 0.85, 0.85], (6400, 3))]
    pos = np.ones((30000, 4), np.float32)
    pos[:, :3] = np.concatenate(parts)
    pos = pos[rng.permutation(len(pos))]
    vel = np.zeros_like(pos)
    xml = configs.scene_xml(**configs.dambreak_attrs(len(pos), (0, 0, 0), (1, 1, 1)))
    p = Scene.parse(xml).params
    with system_from(p, pos, vel) as s:
        s.update(1)
        sh, cs, _ = s.cells()
    o = oracle.full_stages(p, pos, vel)
    cnt = np.bincount(o["sorted"][:, 0], minlength=p.numCells)
    assert cnt.max() > 16384 and ((cnt > 1024) & (cnt <= 16384)).any() and ((cnt > 32) & (cnt <= 1024)).any()
    np.testing.assert_array_equal(sh, o["sorted"])
    np.testing.assert_array_equal(cs, o["cell_start"])


def test_cell_sort_size_boundaries(cuda):
    """One cell at each boundary of the cell sorts: the warp networks of 2,
    4, 8, 16 and 32 ids per lane (33-64, ..., 513-1024 ids), the block sort
    (1025-16384) and the sort through global scratch (above 16384), with the
    ids of each cell scattered through the input; sorted pairs and cell
    starts equal the oracle's."""
    rng = np.random.default_rng(11)
    h = configs.H_DAMBREAK
    sizes = [33, 64, 65, 128, 129, 256, 257, 512, 513, 1024, 1025, 16384, 16385]
    parts = []
    for k, n in enumerate(sizes):
        cx, cy = (2 + 2 * (k % 8)) * h, (2 + 2 * (k // 8)) * h
        lo = np.array([cx, cy, 4 * h]) + 0.35 * h  # inside one cell, away from its faces
        parts.append(rng.uniform(lo, lo + 0.3 * h, (n, 3)))
    pos = np.ones((sum(sizes), 4), np.float32)
    pos[:, :3] = np.concatenate(parts)
    pos = pos[rng.permutation(len(pos))]
    vel = np.zeros_like(pos)
    xml = configs.scene_xml(**configs.dambreak_attrs(len(pos), (0, 0, 0), (1, 1, 1)))
    p = Scene.parse(xml).params
    with system_from(p, pos, vel) as s:
        s.update(1)
        sh, cs, _ = s.cells()
    o = oracle.full_stages(p, pos, vel)
    cnt = np.bincount(o["sorted"][:, 0], minlength=p.numCells)
    assert sorted(cnt[cnt > 0].tolist()) == sorted(sizes)
    np.testing.assert_array_equal(sh, o["sorted"])
    np.testing.assert_array_equal(cs, o["cell_start"])


@pytest.mark.parametrize("n,nb", [(100_000, 1001), (200_000, 2000)])
def test_cell_ranks_with_bunched_ids(cuda, n, nb):
    """A cell whose ids bunch at one end of their range (ids 0..nb-1 and
    n-1 together; nb = 2000 makes it a cell above 1024 ids, ranked per
    block with 4096 buckets): the bucket ranking sorts it instead, and a
    cell of spread ids next to it is ranked by buckets; both come out in
    (hash, original index) order."""
    rng = np.random.default_rng(21)
    h = configs.H_DAMBREAK
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0.05, 0.95, size=(n, 3))
    lo = np.array([6.35, 6.35, 6.35]) * h  # inside one cell, away from its faces
    bunch = np.r_[np.arange(nb), n - 1]
    pos[bunch, :3] = rng.uniform(lo, lo + 0.3 * h, (len(bunch), 3))
    spread = rng.choice(np.arange(2000, n - 1), 700, replace=False)
    lo2 = lo + np.array([2.0, 0.0, 0.0]) * h
    pos[spread, :3] = rng.uniform(lo2, lo2 + 0.3 * h, (len(spread), 3))
    vel = np.zeros_like(pos)
    xml = configs.scene_xml(**configs.dambreak_attrs(n, (0, 0, 0), (1, 1, 1)))
    p = Scene.parse(xml).params
    with system_from(p, pos, vel) as s:
        s.update(1)
        sh, cs, _ = s.cells()
    o = oracle.full_stages(p, pos, vel)
    cnt = np.bincount(o["sorted"][:, 0], minlength=p.numCells)
    top = sorted(cnt)[-2:]  # the two cells, with a few of the spread particles
    assert 700 <= top[0] <= 1024 and nb + 1 <= top[1] <= nb + 100
    np.testing.assert_array_equal(sh, o["sorted"])
    np.testing.assert_array_equal(cs, o["cell_start"])


@pytest.mark.parametrize("case", ["features", "foam", "foam_edges", "foam_tiny"])
def test_fused_color_and_dye(cuda, golden, case):
    """Colour and dye from the fused step against the reference's collide()
    on the same step (golden fixture, original order), every particle: the
    CLR_VelAcc colour with dye, and the CLR_Vel foam colour, whose walk
    visits the reference's wrapped cell hashes (cells on the other side of
    the grid count within the foam radius)."""
    torch = cuda
    g = golden(f"step_{case}.npz")
    p = params_from(g["params"])
    n = len(g["pos_in"])
    clr = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    dye = torch.zeros(n, dtype=torch.float32, device="cuda")
    with system_from(p, g["pos_in"], g["vel_in"]) as s:
        s.set_color_output(clr, dye)
        s.update(1)
        torch.cuda.synchronize()
        c, d = clr.cpu().numpy(), dye.cpu().numpy()
        s.set_color_output(None)
    np.testing.assert_allclose(d, g["dye"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(c, g["clr"], rtol=1e-4, atol=1e-5)
