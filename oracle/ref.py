"""TEST INFRASTRUCTURE ONLY: the reference's own kernels, run on the CPU.

Wraps ``oracle/_ref/libref_emu.so`` (built by ``oracle/ref_emu/build_ref.sh``
from the reference tree, which exists only where the reference is mounted).
Used to pin the oracle and to generate the golden fixtures under
``tests/golden/``; ``available()`` is False wherever the library is absent.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libref_emu.so")
REF_ROOT = os.environ.get("PIBITI_REFERENCE_ROOT", "/root/reference")

_lib = None


def build() -> bool:
    """Build the library if the reference tree is present; True when usable."""
    if os.path.exists(LIB_PATH):
        return True
    if not os.path.isdir(os.path.join(REF_ROOT, "source", "CUDA")):
        return False
    r = subprocess.run([os.path.join(HERE, "ref_emu", "build_ref.sh"), REF_ROOT],
                       capture_output=True, text=True)
    return r.returncode == 0 and os.path.exists(LIB_PATH)


def available() -> bool:
    return build()


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not build():
            raise RuntimeError("reference emulation library unavailable")
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        L.ref_set_params.argtypes = [vp]
        for name, nargs in (("ref_integrate", 4), ("ref_calc_hash", 2)):
            getattr(L, name).argtypes = [vp] * nargs + [ctypes.c_int]
            getattr(L, name).restype = ctypes.c_int
        L.ref_radix_sort.argtypes = [vp, vp, ctypes.c_uint, ctypes.c_uint]
        L.ref_reorder.argtypes = [vp] * 6 + [ctypes.c_uint, ctypes.c_uint]
        L.ref_reorder.restype = ctypes.c_int
        L.ref_collide.argtypes = [vp] * 9 + [ctypes.c_uint, ctypes.c_uint]
        L.ref_collide.restype = ctypes.c_int
        L.ref_scene_count.argtypes = [ctypes.c_char_p]
        L.ref_scene_load.argtypes = [ctypes.c_char_p, ctypes.c_int, vp, vp]
        L.ref_scene_default.argtypes = [vp, vp]
        L.ref_scene_motion.argtypes = [ctypes.c_char_p, ctypes.c_int, vp]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.flags.c_contiguous
    return ctypes.c_void_p(a.ctypes.data)


def set_params(params) -> None:
    buf = ctypes.create_string_buffer(params.to_bytes(), 560)
    lib().ref_set_params(buf)


def _check(rc, what):
    if rc != 0:
        raise ValueError(f"reference {what} refused (rc={rc}): N must be <=64 or a multiple of 512")


def integrate(params, pos, vel):
    set_params(params)
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 4)
    vel = np.ascontiguousarray(vel, np.float32).reshape(-1, 4)
    npos, nvel = np.empty_like(pos), np.empty_like(vel)
    _check(lib().ref_integrate(_ptr(pos), _ptr(npos), _ptr(vel), _ptr(nvel), len(pos)),
           "integrate")
    return npos, nvel


def calc_hash(params, pos):
    set_params(params)
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 4)
    kv = np.empty((len(pos), 2), np.uint32)
    _check(lib().ref_calc_hash(_ptr(pos), _ptr(kv), len(pos)), "calcHash")
    return kv


def radix_sort(kv, bits):
    d0 = np.ascontiguousarray(kv, np.uint32).copy()
    d1 = np.empty_like(d0)
    lib().ref_radix_sort(_ptr(d0), _ptr(d1), len(d0), bits)
    return d0


def reorder(params, kv, pos, vel):
    set_params(params)
    kv = np.ascontiguousarray(kv, np.uint32)
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 4)
    vel = np.ascontiguousarray(vel, np.float32).reshape(-1, 4)
    spos, svel = np.empty_like(pos), np.empty_like(vel)
    cs = np.empty(params.numCells, np.uint32)
    _check(lib().ref_reorder(_ptr(pos), _ptr(vel), _ptr(spos), _ptr(svel), _ptr(kv), _ptr(cs),
                             len(pos), params.numCells), "reorder")
    return spos, svel, cs


def collide(params, spos, svel, kv, cs, dye=None):
    """Density then force pass; returns (density, pressure, new_vel_orig, clr, dye)."""
    set_params(params)
    spos = np.ascontiguousarray(spos, np.float32).reshape(-1, 4)
    svel = np.ascontiguousarray(svel, np.float32).reshape(-1, 4)
    kv = np.ascontiguousarray(kv, np.uint32)
    cs = np.ascontiguousarray(cs, np.uint32)
    n = len(spos)
    dens = np.zeros(n, np.float32)
    pres = np.zeros(n, np.float32)
    nvel = np.zeros((n, 4), np.float32)
    clr = np.zeros((n, 4), np.float32)
    dye = np.zeros(n, np.float32) if dye is None else np.ascontiguousarray(dye, np.float32).copy()
    _check(lib().ref_collide(_ptr(spos), _ptr(svel), _ptr(nvel), _ptr(clr), _ptr(pres),
                             _ptr(dens), _ptr(dye), _ptr(kv), _ptr(cs), n, params.numCells),
           "collide")
    return dens, pres, nvel, clr, dye


def update(params, pos, vel):
    """One cSPH::Update (SPH_Update.cpp:12-81) through the reference's kernels."""
    npos, nvel = integrate(params, pos, vel)
    kv = calc_hash(params, npos)
    skv = radix_sort(kv, 32 if params.numCells >= 65536 else 16)
    spos, svel, cs = reorder(params, skv, npos, nvel)
    dens, pres, vel2, clr, dye = collide(params, spos, svel, skv, cs)
    return dict(pos=npos, vel_int=nvel, hash=kv, sorted=skv, sorted_pos=spos, sorted_vel=svel,
                cell_start=cs, density=dens, pressure=pres, vel=vel2, clr=clr, dye=dye)


def scene_count(path: str) -> int:
    return lib().ref_scene_count(path.encode())


def scene_load(path: str, index: int):
    from pibiti_gb300.params import SimParams
    buf = ctypes.create_string_buffer(560)
    extra = (ctypes.c_float * 16)()
    rc = lib().ref_scene_load(path.encode(), index, buf, extra)
    if rc != 0:
        raise ValueError(f"reference scene loader failed rc={rc}")
    return SimParams.from_bytes(buf.raw), list(extra)[:13]


def scene_motion(path: str, index: int) -> np.ndarray:
    """Emitters (4 x [pos3, rot3, vel, size, size2]) and rVel, r2Vel."""
    out = (ctypes.c_float * 38)()
    rc = lib().ref_scene_motion(path.encode(), index, out)
    if rc != 0:
        raise ValueError(f"reference scene loader failed rc={rc}")
    return np.array(list(out), np.float32)


def scene_default():
    from pibiti_gb300.params import SimParams
    buf = ctypes.create_string_buffer(560)
    extra = (ctypes.c_float * 16)()
    lib().ref_scene_default(buf, extra)
    return SimParams.from_bytes(buf.raw), list(extra)[:13]
