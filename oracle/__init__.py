"""TEST INFRASTRUCTURE ONLY: numpy front end of the oracle.

The oracle is the CPU restatement of the reference's SPH step in
``oracle/sph_oracle.c`` (single- and double-precision forms).  Only tests/,
``__graft_entry__.smoke()`` (as its check) and ``bench.py``'s CPU-baseline leg
use it.  The product package never imports this module.

``oracle.ref`` wraps the reference's own kernels compiled for the host
(``oracle/_ref/libref_emu.so``, built by ``oracle/ref_emu/build_ref.sh`` where
the reference tree is present).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsph_oracle.so")

_lib = None
_u32p = ctypes.POINTER(ctypes.c_uint32)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)


def build(force: bool = False) -> str:
    """Compile the oracle library with the Makefile beside this file."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        u32 = ctypes.c_uint32
        L.orc_calc_hash.argtypes = [vp, _f32p, u32, _u32p]
        L.orc_sort_pairs.argtypes = [_u32p, u32, u32]
        L.orc_reorder.argtypes = [vp, _u32p, _f32p, _f32p, u32, _f32p, _f32p, _u32p]
        L.orc_density_f32.argtypes = [vp, _f32p, _u32p, _u32p, u32, _f32p, _f32p]
        L.orc_density_f64.argtypes = [vp, _f32p, _u32p, _u32p, u32, _f64p, _f64p, _i32p]
        L.orc_force_f32.argtypes = [vp, _f32p, _f32p, _f32p, _f32p, _u32p, _u32p, u32, _f32p]
        L.orc_force_f64.argtypes = [vp, _f32p, _f32p, _f64p, _f64p, _u32p, _u32p, u32, _f64p,
                                    _f64p]
        L.orc_force_color_f32.argtypes = [vp, _f32p, _f32p, _f32p, _f32p, _u32p, _u32p, u32,
                                          _f32p, _f32p, _f32p]
        L.orc_integrate_f32.argtypes = [vp, _f32p, _f32p, u32, _f32p, _f32p]
        L.orc_integrate_f64.argtypes = [vp, _f32p, _f32p, u32, _f64p, _f64p]
        L.orc_step_f32.argtypes = [vp, _f32p, _f32p, u32, u32, ctypes.c_int]
        L.orc_step_f32.restype = ctypes.c_int
        L.orc_step_d64.argtypes = [vp, _f64p, _f64p, u32, u32, _f64p]
        L.orc_step_d64.restype = ctypes.c_int
        L.orc_threads.restype = ctypes.c_int
        L.orc_reduce.argtypes = [vp, _f32p, _f32p, u32, _f64p]
        _lib = L
    return _lib


def _p(a: np.ndarray, ctype):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def _pb(params) -> ctypes.c_char_p:
    b = params if isinstance(params, (bytes, bytearray)) else params.to_bytes()
    buf = ctypes.create_string_buffer(bytes(b), len(b))
    return buf


def _f4(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32).reshape(-1, 4)


def calc_hash(params, pos) -> np.ndarray:
    pos = _f4(pos)
    kv = np.empty((len(pos), 2), np.uint32)
    lib().orc_calc_hash(_pb(params), _p(pos, ctypes.c_float), len(pos), _p(kv, ctypes.c_uint32))
    return kv


def sort_pairs(kv, bits: int) -> np.ndarray:
    kv = np.ascontiguousarray(kv, dtype=np.uint32).copy()
    lib().orc_sort_pairs(_p(kv, ctypes.c_uint32), len(kv), bits)
    return kv


def reorder(params, kv, pos, vel):
    kv = np.ascontiguousarray(kv, dtype=np.uint32)
    pos, vel = _f4(pos), _f4(vel)
    n = len(pos)
    spos = np.empty_like(pos)
    svel = np.empty_like(vel)
    cs = np.empty(params.numCells, np.uint32)
    lib().orc_reorder(_pb(params), _p(kv, ctypes.c_uint32), _p(pos, ctypes.c_float),
                      _p(vel, ctypes.c_float), n, _p(spos, ctypes.c_float),
                      _p(svel, ctypes.c_float), _p(cs, ctypes.c_uint32))
    return spos, svel, cs


def density(params, spos, kv, cell_start, fp64: bool = False, with_nbr: bool = False):
    spos = _f4(spos)
    kv = np.ascontiguousarray(kv, dtype=np.uint32)
    cs = np.ascontiguousarray(cell_start, dtype=np.uint32)
    n = len(spos)
    if fp64:
        d = np.empty(n, np.float64)
        pr = np.empty(n, np.float64)
        nbr = np.empty(n, np.int32)
        lib().orc_density_f64(_pb(params), _p(spos, ctypes.c_float), _p(kv, ctypes.c_uint32),
                              _p(cs, ctypes.c_uint32), n, _p(d, ctypes.c_double),
                              _p(pr, ctypes.c_double), _p(nbr, ctypes.c_int32))
        return (d, pr, nbr) if with_nbr else (d, pr)
    d = np.empty(n, np.float32)
    pr = np.empty(n, np.float32)
    lib().orc_density_f32(_pb(params), _p(spos, ctypes.c_float), _p(kv, ctypes.c_uint32),
                          _p(cs, ctypes.c_uint32), n, _p(d, ctypes.c_float),
                          _p(pr, ctypes.c_float))
    return d, pr


def force(params, spos, svel, dens, pres, kv, cell_start, fp64: bool = False):
    """New velocity in original order; fp64 also returns the per-particle
    sum of increment magnitudes (the tolerance scale)."""
    spos, svel = _f4(spos), _f4(svel)
    kv = np.ascontiguousarray(kv, dtype=np.uint32)
    cs = np.ascontiguousarray(cell_start, dtype=np.uint32)
    n = len(spos)
    if fp64:
        d = np.ascontiguousarray(dens, dtype=np.float64)
        pr = np.ascontiguousarray(pres, dtype=np.float64)
        out = np.zeros((n, 4), np.float64)
        scale = np.zeros(n, np.float64)
        lib().orc_force_f64(_pb(params), _p(spos, ctypes.c_float), _p(svel, ctypes.c_float),
                            _p(d, ctypes.c_double), _p(pr, ctypes.c_double),
                            _p(kv, ctypes.c_uint32), _p(cs, ctypes.c_uint32), n,
                            _p(out, ctypes.c_double), _p(scale, ctypes.c_double))
        return out, scale
    d = np.ascontiguousarray(dens, dtype=np.float32)
    pr = np.ascontiguousarray(pres, dtype=np.float32)
    out = np.zeros((n, 4), np.float32)
    lib().orc_force_f32(_pb(params), _p(spos, ctypes.c_float), _p(svel, ctypes.c_float),
                        _p(d, ctypes.c_float), _p(pr, ctypes.c_float), _p(kv, ctypes.c_uint32),
                        _p(cs, ctypes.c_uint32), n, _p(out, ctypes.c_float))
    return out


def force_color(params, spos, svel, dens, pres, kv, cell_start, dye):
    spos, svel = _f4(spos), _f4(svel)
    kv = np.ascontiguousarray(kv, dtype=np.uint32)
    cs = np.ascontiguousarray(cell_start, dtype=np.uint32)
    n = len(spos)
    d = np.ascontiguousarray(dens, dtype=np.float32)
    pr = np.ascontiguousarray(pres, dtype=np.float32)
    dye = np.ascontiguousarray(dye, dtype=np.float32).copy()
    out = np.zeros((n, 4), np.float32)
    clr = np.zeros((n, 4), np.float32)
    lib().orc_force_color_f32(_pb(params), _p(spos, ctypes.c_float), _p(svel, ctypes.c_float),
                              _p(d, ctypes.c_float), _p(pr, ctypes.c_float),
                              _p(kv, ctypes.c_uint32), _p(cs, ctypes.c_uint32), n,
                              _p(out, ctypes.c_float), _p(dye, ctypes.c_float),
                              _p(clr, ctypes.c_float))
    return out, dye, clr


def integrate(params, pos, vel, fp64: bool = False):
    pos, vel = _f4(pos), _f4(vel)
    n = len(pos)
    dt = np.float64 if fp64 else np.float32
    ct = ctypes.c_double if fp64 else ctypes.c_float
    npos = np.empty((n, 4), dt)
    nvel = np.empty((n, 4), dt)
    fn = lib().orc_integrate_f64 if fp64 else lib().orc_integrate_f32
    fn(_pb(params), _p(pos, ctypes.c_float), _p(vel, ctypes.c_float), n, _p(npos, ct),
       _p(nvel, ct))
    return npos, nvel


def step(params, pos, vel, steps: int = 1, threads: int = 0):
    """Whole cSPH::Update steps in single precision; returns new (pos, vel)."""
    pos = _f4(pos).copy()
    vel = _f4(vel).copy()
    rc = lib().orc_step_f32(_pb(params), _p(pos, ctypes.c_float), _p(vel, ctypes.c_float),
                            len(pos), steps, threads)
    if rc != 0:
        raise MemoryError("oracle step could not allocate its work buffers")
    return pos, vel


def step_fp64(params, pos, vel, steps: int = 1, with_density: bool = False):
    """Whole steps with the state held in double precision (orc_step_d64);
    returns new (pos, vel) as float64 arrays, and with `with_density` the
    mean density of the last step as a third item."""
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 4).copy()
    vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 4).copy()
    md = np.zeros(1, np.float64)
    rc = lib().orc_step_d64(_pb(params), _p(pos, ctypes.c_double), _p(vel, ctypes.c_double),
                            len(pos), steps, _p(md, ctypes.c_double))
    if rc != 0:
        raise MemoryError("oracle step could not allocate its work buffers")
    return (pos, vel, float(md[0])) if with_density else (pos, vel)


def threads() -> int:
    return lib().orc_threads()


def reduce(params, vel, dens=None):
    vel = _f4(vel)
    out = np.zeros(2, np.float64)
    d = None if dens is None else np.ascontiguousarray(dens, dtype=np.float32)
    lib().orc_reduce(_pb(params), _p(vel, ctypes.c_float),
                     None if d is None else _p(d, ctypes.c_float), len(vel),
                     _p(out, ctypes.c_double))
    return float(out[0]), float(out[1])


def full_stages(params, pos, vel):
    """One step as separate stages (integrate, hash, sort, reorder, density,
    force), single precision; returns every intermediate in a dict."""
    npos, nvel = integrate(params, pos, vel)
    kv = calc_hash(params, npos)
    bits = 32 if params.numCells >= 65536 else 16
    skv = sort_pairs(kv, bits)
    spos, svel, cs = reorder(params, skv, npos, nvel)
    d, pr = density(params, spos, skv, cs)
    new_vel = force(params, spos, svel, d, pr, skv, cs)
    return dict(pos=npos, vel_int=nvel, hash=kv, sorted=skv, sorted_pos=spos, sorted_vel=svel,
                cell_start=cs, density=d, pressure=pr, vel=new_vel)
