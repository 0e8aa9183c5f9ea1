"""The reference's own CUDA kernels on the GPU (oracle/ref_gpu.py: its
System.cu and radixsort_kernel.cu compiled for sm_103a, launched as its
wrappers launch them) against the fused step, from the same state.

Bit for bit: the positions after integrate, the sorted (hash, index) pairs
and cellStart.  Density (sorted order) and the new velocities within 1e-5
relative (velocities: of their largest magnitude): the reference sums
density with pow(c, 3) and contracts nothing (built with --fmad=false, like
its host build that pins the oracle), the fused step with FMAs in the
places the oracle has them.

The last tests time the reference's step (nvcc's default flags, every
wrapper synchronising as the reference's do) against the fused step on the
three single-scene workloads (32,768, 1,048,576 and 16,777,216 particles) and
print one JSON line each.
"""
import json
import time

import numpy as np
import pytest

from conftest import params_from
from oracle import ref_gpu
from pibiti_gb300 import configs
from pibiti_gb300.sph import ARRAY_POS, ARRAY_VEL, SPH, Scene

pytestmark = pytest.mark.gpu

DENS_RTOL = 1e-5
VEL_RTOL = 1e-5


@pytest.fixture(scope="module")
def ref(cuda):
    if not ref_gpu.available():
        pytest.skip("the reference's kernels were not compiled to PTX (reference tree absent at build)")
    return ref_gpu


def _state(w, warm):
    p = Scene.parse(w.xml).params
    with SPH(p) as s:
        s.set_array(ARRAY_POS, w.pos)
        s.set_array(ARRAY_VEL, w.vel)
        s.update(warm)
        return p, s.get_array(ARRAY_POS), s.get_array(ARRAY_VEL)


def _compare(p, pos, vel, ref):
    r = ref.RefStep(p, pos, vel)
    r.update(1)
    got = r.results()
    with SPH(p) as s:
        s.set_array(ARRAY_POS, pos)
        s.set_array(ARRAY_VEL, vel)
        s.update(1)
        sh, cs, ce = s.cells()
        dens, _ = s.fields()
        opos, ovel = s.get_array(ARRAY_POS), s.get_array(ARRAY_VEL)
    np.testing.assert_array_equal(opos, got["pos"])
    np.testing.assert_array_equal(sh, got["sorted"])
    nz = ce > cs
    np.testing.assert_array_equal(cs[nz], got["cell_start"][nz])
    assert np.all(got["cell_start"][~nz] == 0xFFFFFFFF)
    np.testing.assert_allclose(dens, got["density"], rtol=DENS_RTOL, atol=1e-3)
    scale = np.abs(got["vel"][:, :3]).max()
    np.testing.assert_allclose(ovel[:, :3], got["vel"][:, :3], rtol=0, atol=VEL_RTOL * scale)
    return got


@pytest.mark.parametrize("case", ["box", "cyl_y", "cyl_z", "cyl_yz", "sphere", "wrap", "cycle",
                                  "wave", "pump", "pump_s"])
def test_integrate_boundaries_bit_exact(ref, golden, case):
    """integrate on every boundary type and z effect (the golden fixture's
    inputs): bit for bit against the reference's own integrate on the GPU,
    where both evaluate the curved walls with the same device sqrt, sin,
    cos and atan2 (against the host-emulated reference they agree within
    the C library's tolerance)."""
    import torch
    from pibiti_gb300.sph import stage
    g = golden("integrate.npz")
    p = params_from(g[f"{case}_params"])
    pos, vel = g[f"{case}_pos_in"], g[f"{case}_vel_in"]
    rpos, rvel = ref.integrate(p, pos, vel)
    stage.set_parameters(p)
    dp = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).cuda()
    dv = torch.from_numpy(np.ascontiguousarray(vel, np.float32)).cuda()
    npos, nvel = torch.empty_like(dp), torch.empty_like(dv)
    stage.integrate(dp, npos, dv, nvel, len(pos))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(npos.cpu().numpy(), rpos)
    np.testing.assert_array_equal(nvel.cpu().numpy(), rvel)


def test_single_dam_break_32k(ref):
    """32,768 particles (a 32^3 lattice at spacing 0.5h in a unit box),
    after 30 steps."""
    w = configs.dambreak_small(side=32)
    p, pos, vel = _state(w, 30)
    got = _compare(p, pos, vel, ref)
    assert np.count_nonzero(got["cell_start"] != 0xFFFFFFFF) > 100


def test_double_dam_break_1m(ref):
    """The 1,048,576-particle double dam break after 20 steps (376,200
    cells: 32-bit keys, four radix passes)."""
    w = configs.dambreak_double()
    p, pos, vel = _state(w, 20)
    _compare(p, pos, vel, ref)


def test_uniform_stress_16m(ref):
    """16,777,216 particles uniform-random in the lower 60% of a 4x1x4 box
    (2.96 M cells), after 3 steps."""
    w = configs.uniform_stress()
    p, pos, vel = _state(w, 3)
    _compare(p, pos, vel, ref)


TIMED = {
    "single dam break, 32,768 particles": (lambda: configs.dambreak_small(side=32), 200),
    "double dam break, 1,048,576 particles": (lambda: configs.dambreak_double(), 200),
    "uniform stress, 16,777,216 particles": (lambda: configs.uniform_stress(), 3),
}


@pytest.mark.parametrize("name", list(TIMED))
def test_reference_step_time(ref, name):
    """Step time of the reference's kernels (default nvcc flags, each wrapper
    synchronising) and of the fused step, from the same state after the
    given number of fused steps."""
    import torch
    make, warm = TIMED[name]
    w = make()
    p, pos, vel = _state(w, warm)
    r = ref.RefStep(p, pos, vel, fast=True)
    r.update(2)
    stage = {}
    k = 10
    t0 = time.perf_counter()
    r.update(k, stage)
    ref_ms = (time.perf_counter() - t0) / k * 1e3
    with SPH(p) as s:
        s.set_array(ARRAY_POS, pos)
        s.set_array(ARRAY_VEL, vel)
        s.update(5)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.update(50)
        torch.cuda.synchronize()
        ours_ms = (time.perf_counter() - t0) / 50 * 1e3
    n = len(pos)
    line = {"workload": f"{name}, steps {warm}-{warm + 12} (reference), {warm}-{warm + 55} (fused)",
            "reference_gpu_ms_per_step": ref_ms,
            "reference_gpu_particle_steps_per_s": n / ref_ms * 1e3,
            "reference_gpu_stage_ms": {kk: v / k * 1e3 for kk, v in stage.items()},
            "fused_ms_per_step": ours_ms, "fused_particle_steps_per_s": n / ours_ms * 1e3,
            "speedup": ref_ms / ours_ms}
    print(json.dumps(line))
    assert ours_ms < ref_ms
