"""GPU parity of the stage entry points (the reference's wrappers) through
the C ABI, against the golden fixtures made by the reference's own kernels
and against the oracle.

Bit-exact: integrate, calcHash, RadixSort, reorder.  Density: within
DENS_RTOL of the double-precision oracle; new velocity: the difference to
the double-precision oracle within VEL_RTOL times the sum of the magnitudes
of the increments that were added (plus 4 ulp of the velocity itself, and
for the height-map and rotor colliders a conditioning term, check_force).
"""
import numpy as np
import pytest

import oracle
from conftest import params_from

pytestmark = pytest.mark.gpu

DENS_RTOL = 1e-5
VEL_RTOL = 1e-5
CASES = ["dambreak", "truncate", "features", "foam", "foam_edges", "foam_tiny", "bigrid", "tiny", "rotor", "propeller",
         "hmapxz", "hmapyz"]


def dev(torch, a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    return torch.from_numpy(a.copy()).cuda()


def host(t, dtype=None):
    a = t.cpu().numpy()
    if dtype == np.uint32:
        a = a.view(np.uint32)
    return a


COND_ULPS = 4


def _conditioning(p, g_sorted, spos, svel, dens, pres, cs, v64, idx):
    """Largest change of the FP64 new velocity of particles `idx` (original
    indices) when their positions move by one ulp along any axis.  The
    height-map and rotor colliders are steep or discontinuous in position
    (sample windows, contact tests), so an FP32 evaluation is defined only to
    within a few of these."""
    rank = np.empty(len(g_sorted), np.int64)
    rank[g_sorted[:, 1]] = np.arange(len(g_sorted))
    k = rank[idx]
    sens = np.zeros(len(idx))
    for ax in range(3):
        for to in (np.float32(np.inf), np.float32(-np.inf)):
            sp = spos.copy()
            sp[k, ax] = np.nextafter(sp[k, ax], to)
            v2, _ = oracle.force(p, sp, svel, dens, pres, g_sorted, cs, fp64=True)
            sens = np.maximum(sens, np.abs(v2[idx, :3] - v64[idx, :3]).max(axis=1))
    return sens


def check_force(p, g_sorted, spos, svel, dens, pres, cs, vel_gpu):
    """New velocities within VEL_RTOL of the FP64 oracle, relative to the sum
    of the magnitudes of the increments; with the height-map or rotor
    collider, plus COND_ULPS times the velocity change that a one-ulp move of
    the particle's position causes (computed for the particles that need it)."""
    v64, scale = oracle.force(p, spos, svel, dens, pres, g_sorted, cs, fp64=True)
    vin = np.empty((len(spos), 4))
    vin[g_sorted[:, 1]] = svel
    err = np.abs(vel_gpu[:, :3].astype(np.float64) - v64[:, :3]).max(axis=1)
    bound = VEL_RTOL * scale + 4 * np.finfo(np.float32).eps * np.abs(vin[:, :3]).max(axis=1) + 1e-12
    if p.iHmap > 0 or p.rotType > 0:
        idx = np.nonzero(err > bound)[0]
        assert len(idx) <= max(8, len(err) // 200), f"{len(idx)} particles outside the plain bound"
        if len(idx):
            bound[idx] += COND_ULPS * _conditioning(p, g_sorted, spos, svel, dens, pres, cs, v64, idx)
    assert np.all(err <= bound), f"worst err/bound {float((err / bound).max()):.3g}"
    np.testing.assert_array_equal(vel_gpu[:, 3], vin[:, 3])


@pytest.mark.parametrize("case", CASES)
def test_stages_vs_reference(cuda, golden, case):
    torch = cuda
    from pibiti_gb300.sph import stage
    g = golden(f"step_{case}.npz")
    p = params_from(g["params"])
    n = len(g["pos_in"])
    stage.set_parameters(p)
    # integrate
    pos_in, vel_in = dev(torch, g["pos_in"]), dev(torch, g["vel_in"])
    npos, nvel = torch.empty_like(pos_in), torch.empty_like(vel_in)
    stage.integrate(pos_in, npos, vel_in, nvel, n)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(host(npos), g["pos"])
    np.testing.assert_array_equal(host(nvel), g["vel_int"])
    # calcHash on the reference's integrated positions
    gpos = dev(torch, g["pos"])
    kv = torch.empty((n, 2), dtype=torch.int32, device="cuda")
    stage.calc_hash(gpos, kv, n)
    np.testing.assert_array_equal(host(kv, np.uint32), g["hash"])
    # RadixSort: 16 or 32 bits as cSPH::Update chooses
    tmp = torch.empty_like(kv)
    stage.radix_sort(kv, tmp, n, 32 if p.numCells >= 65536 else 16)
    np.testing.assert_array_equal(host(kv, np.uint32), g["sorted"])
    # reorder
    spos, svel = torch.empty_like(gpos), torch.empty_like(gpos)
    cs = torch.empty(p.numCells, dtype=torch.int32, device="cuda")
    stage.reorder(gpos, dev(torch, g["vel_int"]), spos, svel, dev(torch, g["sorted"]), cs, n,
                  p.numCells)
    np.testing.assert_array_equal(host(cs, np.uint32), g["cell_start"])
    np.testing.assert_array_equal(host(spos), g["sorted_pos"])
    np.testing.assert_array_equal(host(svel), g["sorted_vel"])
    # collide on the reference's sorted arrays
    gs = dev(torch, g["sorted"])
    gcs = dev(torch, g["cell_start"])
    gsp, gsv = dev(torch, g["sorted_pos"]), dev(torch, g["sorted_vel"])
    dens = torch.empty(n, dtype=torch.float32, device="cuda")
    pres = torch.empty_like(dens)
    newv = torch.zeros_like(gsp)
    clr = torch.zeros_like(gsp)
    dye = torch.zeros(n, dtype=torch.float32, device="cuda")
    stage.collide(gsp, gsv, newv, pres, dens, gs, gcs, n, p.numCells, clr=clr, dye=dye)
    torch.cuda.synchronize()
    d_gpu = host(dens)
    d64, p64 = oracle.density(p, g["sorted_pos"], g["sorted"], g["cell_start"], fp64=True)
    np.testing.assert_allclose(d_gpu, d64, rtol=DENS_RTOL, atol=1e-2)
    np.testing.assert_allclose(d_gpu, g["density"], rtol=DENS_RTOL, atol=1e-2)
    check_force(p, g["sorted"], g["sorted_pos"], g["sorted_vel"], d_gpu, host(pres),
                g["cell_start"], host(newv))
    # the single-precision oracle performs the same IEEE operations
    d32, _ = oracle.density(p, g["sorted_pos"], g["sorted"], g["cell_start"])
    np.testing.assert_array_equal(d_gpu, d32)
    if case in ("features", "foam"):
        np.testing.assert_allclose(host(dye), g["dye"], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(host(clr), g["clr"], rtol=1e-4, atol=1e-5)


@pytest.mark.parametrize("case", ["box", "cyl_y", "cyl_z", "cyl_yz", "sphere", "wrap", "cycle",
                                  "wave", "pump", "pump_s"])
def test_integrate_boundaries(cuda, golden, case):
    torch = cuda
    from pibiti_gb300.sph import stage
    g = golden("integrate.npz")
    p = params_from(g[f"{case}_params"])
    stage.set_parameters(p)
    pos_in, vel_in = dev(torch, g[f"{case}_pos_in"]), dev(torch, g[f"{case}_vel_in"])
    npos, nvel = torch.empty_like(pos_in), torch.empty_like(vel_in)
    stage.integrate(pos_in, npos, vel_in, nvel, len(pos_in))
    torch.cuda.synchronize()
    if case in ("box", "wrap", "cycle"):
        np.testing.assert_array_equal(host(npos), g[f"{case}_pos"])
        np.testing.assert_array_equal(host(nvel), g[f"{case}_vel"])
    else:  # device sqrt/sin/cos/atan vs the host C library
        np.testing.assert_allclose(host(npos), g[f"{case}_pos"], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(host(nvel), g[f"{case}_vel"], rtol=1e-4, atol=1e-5)


@pytest.mark.parametrize("n,bits", [(1, 32), (777, 16), (5000, 8), (4096, 24), (70001, 32),
                                    (300000, 16)])
def test_radix_sort_stable(cuda, n, bits):
    """Stable by the low `bits` bits of the key; the result lands in pData0
    after an even number of 8-bit passes and in pData1 after an odd one."""
    torch = cuda
    from pibiti_gb300.sph import stage
    rng = np.random.default_rng(n)
    kv = np.stack([rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32),
                   rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)], axis=1)
    kv[: n // 3, 0] &= 0xFF  # many equal keys
    d0, d1 = dev(torch, kv), torch.empty((n, 2), dtype=torch.int32, device="cuda")
    stage.radix_sort(d0, d1, n, bits)
    passes = (bits + 7) // 8
    out = host(d0 if passes % 2 == 0 else d1, np.uint32)
    np.testing.assert_array_equal(out, oracle.sort_pairs(kv, bits))


def test_stage_errors(cuda):
    """Parameter sets the kernels do not cover are refused with a status."""
    from pibiti_gb300 import _lib
    from pibiti_gb300.sph import Scene, stage
    p = Scene.default().params
    p.bndType = 9
    with pytest.raises(_lib.SphError) as e:
        stage.set_parameters(p)
    assert e.value.code == 3
