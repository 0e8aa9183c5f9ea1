"""TEST INFRASTRUCTURE ONLY: the reference's own CUDA kernels, run on the GPU.

``oracle/ref_gpu/build_ref_gpu.sh`` compiles the kernel sections of the
reference's System.cu and radixsort_kernel.cu to PTX (where the reference tree
is mounted; the PTX travels with the repository copy), and
``oracle/_build/libref_gpu.so`` (``oracle/ref_gpu/ref_gpu.cpp``) loads it
through the CUDA driver API and launches the kernels as the reference's
wrappers do.  ``RefStep`` runs ``cSPH::Update`` (SPH_Update.cpp:12-81) on
device buffers: integrate, swap, calcHash, RadixSort, reorder, collide
(density, then force), swap.  The tests use it to compare the fused step
with the reference's GPU execution and to time the reference's kernels.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(HERE, "_build", "libref_gpu.so")
PTX_SYSTEM = os.path.join(REF_DIR, "ref_system.ptx")            # --fmad=false (parity)
PTX_SYSTEM_FAST = os.path.join(REF_DIR, "ref_system_fast.ptx")  # nvcc defaults (timing)
PTX_RADIX = os.path.join(REF_DIR, "ref_radix.ptx")
ENTRIES = os.path.join(REF_DIR, "ref_gpu_entries.txt")
REF_ROOT = os.environ.get("PIBITI_REFERENCE_ROOT", "/root/reference")

_lib = None
_loaded = None


def build_ptx() -> bool:
    """Compiles the reference's kernels to PTX if the reference tree is here."""
    if not os.path.isdir(os.path.join(REF_ROOT, "source", "CUDA")):
        return all(os.path.exists(f) for f in (PTX_SYSTEM, PTX_SYSTEM_FAST, PTX_RADIX, ENTRIES))
    r = subprocess.run([os.path.join(HERE, "ref_gpu", "build_ref_gpu.sh"), REF_ROOT],
                       capture_output=True, text=True)
    return r.returncode == 0


def available() -> bool:
    """True where the PTX and the harness exist and a GPU can load them."""
    if not all(os.path.exists(f) for f in (LIB_PATH, PTX_SYSTEM, PTX_SYSTEM_FAST, PTX_RADIX, ENTRIES)):
        return False
    try:
        import torch
        if not torch.cuda.is_available():
            return False
        _load(fast=False)
        return True
    except (OSError, RuntimeError):
        return False


def _lib_handle() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB_PATH)
        vp, u32 = ctypes.c_void_p, ctypes.c_uint32
        L.ref_gpu_error.restype = ctypes.c_char_p
        L.ref_gpu_load.argtypes = [ctypes.c_char_p] * 3
        L.ref_gpu_unload.argtypes = []
        L.ref_gpu_params_bytes.restype = ctypes.c_ulonglong
        L.ref_gpu_set_params.argtypes = [vp, ctypes.c_ulonglong]
        L.ref_gpu_integrate.argtypes = [vp] * 4 + [u32]
        L.ref_gpu_calc_hash.argtypes = [vp, vp, u32]
        L.ref_gpu_radix_sort.argtypes = [vp, vp, u32, u32]
        L.ref_gpu_reorder.argtypes = [vp] * 6 + [u32, u32]
        L.ref_gpu_collide.argtypes = [vp] * 9 + [u32, u32]
        _lib = L
    return _lib


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"reference GPU {what} (rc={rc}): {_lib_handle().ref_gpu_error().decode()}")


def _load(fast: bool) -> ctypes.CDLL:
    """Loads the parity (--fmad=false) or the default-flags build."""
    global _loaded
    import torch
    torch.zeros(1, device="cuda")  # the primary context the harness shares
    L = _lib_handle()
    if _loaded is not None and _loaded != fast:
        _check(L.ref_gpu_unload(), "unload")
        _loaded = None
    if _loaded is None:
        system = PTX_SYSTEM_FAST if fast else PTX_SYSTEM
        _check(L.ref_gpu_load(system.encode(), PTX_RADIX.encode(), ENTRIES.encode()), "load")
        _loaded = fast
    return L


def integrate(params, pos, vel, fast: bool = False):
    """The reference's integrate wrapper (System.cu:653-667, with
    boundary()) alone on the GPU: (new positions, new velocities)."""
    import torch
    L = _load(fast)
    raw = params.to_bytes()
    buf = ctypes.create_string_buffer(raw, len(raw))
    _check(L.ref_gpu_set_params(buf, len(raw)), "setParameters")
    n = len(pos)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32).reshape(n, 4)).cuda()  # noqa: E731
    p0, v0 = dev(pos), dev(vel)
    p1, v1 = torch.empty_like(p0), torch.empty_like(v0)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    _check(L.ref_gpu_integrate(vp(p0), vp(p1), vp(v0), vp(v1), n), "integrate")
    return p1.cpu().numpy(), v1.cpu().numpy()


class RefStep:
    """The reference's buffers (cSPH, SPH_Mem.cpp) for one scene of N
    particles on the GPU, and its Update.  N must be <= 64 or a multiple of
    512 (the reference's kernels have no tail guard)."""

    def __init__(self, params, pos, vel, fast: bool = False):
        import torch
        self.L = _load(fast)
        self.p = params
        self.n = n = len(pos)
        self.cells = int(params.numCells)
        f4 = lambda: torch.zeros((n, 4), dtype=torch.float32, device="cuda")  # noqa: E731
        self.pos = [f4(), f4()]
        self.vel = [f4(), f4()]
        self.spos, self.svel, self.clr = f4(), f4(), f4()
        self.pres = torch.zeros(n, dtype=torch.float32, device="cuda")
        self.dens = torch.zeros(n, dtype=torch.float32, device="cuda")
        self.dye = torch.zeros(n, dtype=torch.float32, device="cuda")
        self.hash = [torch.zeros((n, 2), dtype=torch.int32, device="cuda") for _ in range(2)]
        self.cell_start = torch.zeros(self.cells, dtype=torch.int32, device="cuda")
        self.pos[0].copy_(torch.from_numpy(np.ascontiguousarray(pos, np.float32).reshape(n, 4)))
        self.vel[0].copy_(torch.from_numpy(np.ascontiguousarray(vel, np.float32).reshape(n, 4)))
        self.pr = self.vr = 0  # curPosRead, curVelRead
        raw = params.to_bytes()
        self._params = ctypes.create_string_buffer(raw, len(raw))
        if self.L.ref_gpu_params_bytes() != len(raw):
            raise RuntimeError("SimParams size differs from the reference's")
        _check(self.L.ref_gpu_set_params(self._params, len(raw)), "setParameters")

    @staticmethod
    def _p(t):
        return ctypes.c_void_p(t.data_ptr())

    STAGES = ("integrate", "calcHash", "RadixSort", "reorder", "collide")

    def update(self, steps: int = 1, stage_s: dict | None = None) -> None:
        """`steps` x cSPH::Update (SPH_Update.cpp:12-81), without its debug
        copies of a few particles to the host.  Every wrapper ends with a
        device synchronisation, as the reference's do, so `stage_s` (if
        given) accumulates each wrapper's wall time in seconds."""
        L, p, n, c = self.L, self._p, self.n, self.cells
        bits = 32 if c >= 65536 else 16
        clock = time.perf_counter
        for _ in range(steps):
            t = [clock()]
            pw, vw = 1 - self.pr, 1 - self.vr
            _check(L.ref_gpu_integrate(p(self.pos[self.pr]), p(self.pos[pw]), p(self.vel[self.vr]),
                                       p(self.vel[vw]), n), "integrate")
            t.append(clock())
            self.pr, self.vr = pw, vw
            _check(L.ref_gpu_calc_hash(p(self.pos[self.pr]), p(self.hash[0]), n), "calcHash")
            t.append(clock())
            _check(L.ref_gpu_radix_sort(p(self.hash[0]), p(self.hash[1]), n, bits), "RadixSort")
            t.append(clock())
            _check(L.ref_gpu_reorder(p(self.pos[self.pr]), p(self.vel[self.vr]), p(self.spos),
                                     p(self.svel), p(self.hash[0]), p(self.cell_start), n, c), "reorder")
            t.append(clock())
            _check(L.ref_gpu_collide(p(self.spos), p(self.svel), p(self.vel[1 - self.vr]), p(self.clr),
                                     p(self.pres), p(self.dens), p(self.dye), p(self.hash[0]),
                                     p(self.cell_start), n, c), "collide")
            t.append(clock())
            self.vr = 1 - self.vr
            if stage_s is not None:
                for k, name in enumerate(self.STAGES):
                    stage_s[name] = stage_s.get(name, 0.0) + t[k + 1] - t[k]

    def results(self) -> dict:
        """The last Update's arrays on the host: positions after integrate
        and the new velocities (original order), the sorted (hash, index)
        pairs, cellStart (0xffffffff when empty), and density and pressure
        (sorted order)."""
        u32 = lambda t: t.cpu().numpy().view(np.uint32)  # noqa: E731
        return dict(pos=self.pos[self.pr].cpu().numpy(), vel=self.vel[self.vr].cpu().numpy(),
                    sorted=u32(self.hash[0]), cell_start=u32(self.cell_start),
                    sorted_pos=self.spos.cpu().numpy(), density=self.dens.cpu().numpy(),
                    pressure=self.pres.cpu().numpy())
