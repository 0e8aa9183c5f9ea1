"""Host API: scenes, the SPH system (the cSPH replacement) and the stage
entry points, over the C ABI.

``SPH`` mirrors the reference's ``cSPH`` (source/SPH/SPH.h:9-50): scenes from
a Scenes.xml file, ``reset`` / ``drop``-style initial states, ``set_array`` /
``get_array`` and ``update``.  Arrays are numpy arrays (host memory) or torch
CUDA tensors (device memory, passed by pointer, no copy through the host).
``stage`` exposes the reference's per-stage wrappers for code that drives
the stages itself.
"""
from __future__ import annotations

import ctypes
from typing import Iterable, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import ARRAY_POS, ARRAY_VEL, SceneInfo, SceneMotion, check, lib
from .params import SimParams

__all__ = ["Scene", "SPH", "ARRAY_POS", "ARRAY_VEL", "stage", "write_snapshot", "read_snapshot"]

SNAPSHOT_VERSION = 1


def write_snapshot(path: str, params: Sequence[SimParams], offsets, pos, vel, step: int = 0,
                   extra: Optional[dict] = None) -> None:
    """A checkpoint file (.npz): every scene's SimParams bytes, the scene
    offsets, positions and velocities in original particle order (float4),
    the caller's step count and any extra arrays of the caller (dye, emitter
    index, ...).  The reference keeps no state beyond these (its only state
    I/O is getArray / setArray, SPH_Util.cpp:44-71)."""
    raw = np.stack([np.frombuffer(p.to_bytes(), np.uint8) for p in params])
    arrays = {"extra_" + k: np.asarray(v) for k, v in (extra or {}).items()}
    for k, v in arrays.items():
        if v.dtype == object:
            raise TypeError(f"snapshot extra {k[len('extra_'):]!r}: numeric arrays only")
    np.savez(path, version=np.int64(SNAPSHOT_VERSION), params=raw, offsets=np.asarray(offsets, np.int64),
             pos=np.asarray(pos, np.float32).reshape(-1, 4), vel=np.asarray(vel, np.float32).reshape(-1, 4),
             step=np.int64(step), **arrays)


def read_snapshot(path: str) -> dict:
    """The contents of a write_snapshot file: params (list of SimParams),
    offsets, pos, vel, step, extra (dict)."""
    with np.load(path) as d:
        if int(d["version"]) != SNAPSHOT_VERSION:
            raise ValueError(f"{path}: snapshot version {int(d['version'])}, expected {SNAPSHOT_VERSION}")
        out = dict(params=[SimParams.from_bytes(row.tobytes()) for row in d["params"]],
                   offsets=[int(v) for v in d["offsets"]], pos=d["pos"].copy(), vel=d["vel"].copy(),
                   step=int(d["step"]),
                   extra={k[len("extra_"):]: d[k].copy() for k in d.files if k.startswith("extra_")})
    if out["offsets"][-1] != len(out["pos"]) or len(out["pos"]) != len(out["vel"]):
        raise ValueError(f"{path}: particle count does not match the scene offsets")
    return out


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _buf(x, dtype=np.float32, cols=4):
    """(pointer, on_device, keepalive) for a numpy array or torch tensor."""
    if _is_torch(x):
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return ctypes.c_void_p(x.data_ptr()), bool(x.is_cuda), x
    a = np.ascontiguousarray(x, dtype=dtype)
    if cols:
        a = a.reshape(-1, cols)
    return ctypes.c_void_p(a.ctypes.data), False, a


class Scene:
    """One scene: SimParams plus the init data Scene keeps beside it."""

    def __init__(self, params: SimParams, info: SceneInfo, motion: Optional[SceneMotion] = None):
        self.params = params
        self.info = info
        self.motion = motion if motion is not None else SceneMotion()

    @property
    def title(self) -> str:
        return self.info.title.decode(errors="replace")

    @classmethod
    def default(cls) -> "Scene":
        p, i = SimParams(), SceneInfo()
        check(lib().sph_scene_default(ctypes.byref(p), ctypes.byref(i)))
        return cls(p, i)

    @classmethod
    def parse(cls, xml: str) -> "Scene":
        p, i, m = SimParams(), SceneInfo(), SceneMotion()
        check(lib().sph_scene_parse(xml.encode(), ctypes.byref(p), ctypes.byref(i)))
        check(lib().sph_scene_parse_motion(xml.encode(), ctypes.byref(m)))
        return cls(p, i, m)

    @classmethod
    def load(cls, path: str, index: int) -> "Scene":
        p, i, m = SimParams(), SceneInfo(), SceneMotion()
        check(lib().sph_scene_load(path.encode(), index, ctypes.byref(p), ctypes.byref(i)))
        check(lib().sph_scene_load_motion(path.encode(), index, ctypes.byref(m)))
        return cls(p, i, m)

    @staticmethod
    def count(path: str) -> int:
        n = ctypes.c_int()
        check(lib().sph_scene_count(path.encode(), ctypes.byref(n)))
        return n.value

    @staticmethod
    def load_all(path: str) -> list["Scene"]:
        """cSPH::LoadScenes (SPH_Scenes.cpp:171-202)."""
        return [Scene.load(path, i) for i in range(Scene.count(path))]

    @staticmethod
    def default_index(path: str) -> int:
        n = ctypes.c_int()
        check(lib().sph_scene_default_index(path.encode(), ctypes.byref(n)))
        return n.value

    def reset(self, kind: int = 0, seed: int = 42):
        """cSPH::Reset (SPH_Init.cpp:23-79): (pos, vel) float32 (N, 4)."""
        n = self.params.numParticles
        pos = np.zeros((n, 4), np.float32)
        vel = np.zeros((n, 4), np.float32)
        placed = ctypes.c_uint32()
        check(lib().sph_scene_reset(ctypes.byref(self.params), ctypes.byref(self.info), kind, seed,
                                    ctypes.c_void_p(pos.ctypes.data),
                                    ctypes.c_void_p(vel.ctypes.data), ctypes.byref(placed)))
        return pos, vel

    def emitter_particles(self, k: int):
        """Particles emitter k writes in one frame (App/Update.cpp:64-91):
        (pos, vel) float32 (n, 4); empty when the emitter is off."""
        em = self.motion.emit[k]
        n = max(em.size, 0) * (em.size2 if em.size2 else max(em.size, 0))
        pos = np.zeros((max(n, 1), 4), np.float32)
        vel = np.zeros((max(n, 1), 4), np.float32)
        cnt = ctypes.c_uint32()
        check(lib().sph_emitter_particles(ctypes.byref(em), self.info.spacing,
                                          ctypes.c_void_p(pos.ctypes.data),
                                          ctypes.c_void_p(vel.ctypes.data), len(pos),
                                          ctypes.byref(cnt)))
        return pos[:cnt.value], vel[:cnt.value]

    def drop_particles(self, random: bool = False, seed: int = 1, capacity: Optional[int] = None):
        """cSPH::Drop (SPH_Init.cpp:83-117): (pos, vel) of the dropped ball."""
        r = int(self.info.dropR) + 1
        cap = (2 * r + 1) ** 3 if capacity is None else capacity
        pos = np.zeros((max(cap, 1), 4), np.float32)
        vel = np.zeros((max(cap, 1), 4), np.float32)
        cnt = ctypes.c_uint32()
        check(lib().sph_drop_particles(ctypes.byref(self.params), ctypes.byref(self.info),
                                       int(random), seed, ctypes.c_void_p(pos.ctypes.data),
                                       ctypes.c_void_p(vel.ctypes.data), cap, ctypes.byref(cnt)))
        return pos[:cnt.value], vel[:cnt.value]

    def advance(self) -> None:
        """One frame of the parameter updates (rotor angles, dye clear)."""
        check(lib().sph_scene_advance(ctypes.byref(self.params), ctypes.byref(self.motion)))


class SPH:
    """The system handle: one scene, or many independent scenes stepped
    together (``SPH([p1, p2, ...])``)."""

    def __init__(self, params, stream=None):
        L = lib()
        self._h = ctypes.c_void_p()
        if isinstance(params, SimParams):
            plist = [params]
        else:
            plist = list(params)
        arr = (SimParams * len(plist))(*plist)
        if len(plist) == 1:
            check(L.sph_create(arr, ctypes.byref(self._h)))
        else:
            check(L.sph_create_ensemble(arr, len(plist), ctypes.byref(self._h)))
        self.num_scenes = L.sph_num_scenes(self._h)
        self.n = L.sph_num_particles(self._h)
        self.num_cells = L.sph_num_cells(self._h)
        self.offsets = [L.sph_scene_offset(self._h, i) for i in range(self.num_scenes + 1)]
        if stream is not None:
            self.set_stream(stream)

    def close(self) -> None:
        if self._h:
            check(lib().sph_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream) -> None:
        """A torch.cuda.Stream, a raw cudaStream_t int, or None."""
        handle = getattr(stream, "cuda_stream", stream)
        check(lib().sph_set_stream(self._h, ctypes.c_void_p(handle or 0)))

    def params(self, scene: int = 0) -> SimParams:
        p = SimParams()
        check(lib().sph_get_params(self._h, scene, ctypes.byref(p)))
        return p

    def set_params(self, p: SimParams, scene: int = 0) -> None:
        check(lib().sph_set_params(self._h, scene, ctypes.byref(p)))

    def set_array(self, which: int, data, start: int = 0) -> None:
        """setArray (SPH_Util.cpp:59-71): float4 records from `start`."""
        ptr, dev, keep = _buf(data)
        count = keep.shape[0] if not dev else keep.numel() // 4
        check(lib().sph_set_array(self._h, which, ptr, start, count, int(dev)))

    def get_array(self, which: int, out=None):
        """getArray (SPH_Util.cpp:44-56): all particles, original order."""
        if out is None:
            out = np.empty((self.n, 4), np.float32)
        ptr, dev, keep = _buf(out)
        check(lib().sph_get_array(self._h, which, ptr, int(dev)))
        return out

    def snapshot(self, path: str, step: int = 0, extra: Optional[dict] = None) -> None:
        """Checkpoint: the scenes' current SimParams, positions and velocities
        (write_snapshot).  restore() continues the plain step bit for bit;
        the learned step restarts its density history."""
        write_snapshot(path, [self.params(k) for k in range(self.num_scenes)], self.offsets,
                       self.get_array(ARRAY_POS), self.get_array(ARRAY_VEL), step, extra)

    @classmethod
    def restore(cls, path: str, stream=None):
        """A new handle from a snapshot file: (handle, step, extra)."""
        snap = read_snapshot(path)
        ps = snap["params"]
        s = cls(ps[0] if len(ps) == 1 else ps, stream=stream)
        try:
            if list(s.offsets) != snap["offsets"]:
                raise ValueError(f"{path}: scene sizes differ from the parameters' particle counts")
            s.set_array(ARRAY_POS, snap["pos"])
            s.set_array(ARRAY_VEL, snap["vel"])
        except Exception:
            s.close()
            raise
        return s, snap["step"], snap["extra"]

    def emit(self, pos, vel, emit_id: int) -> int:
        """Writes emitted particles at the running emit index (App::emitId,
        App/Update.cpp:87-90) with setArray and returns the next index.  A
        block that would run past the last particle continues at 0 (the
        reference writes past the end of its buffers there)."""
        n, total = len(pos), self.n
        if n == 0:
            return emit_id
        if n > total or not 0 <= emit_id < total:
            raise ValueError("emit: block larger than the system or index out of range")
        first = min(n, total - emit_id)
        self.set_array(ARRAY_POS, np.ascontiguousarray(pos[:first]), start=emit_id)
        self.set_array(ARRAY_VEL, np.ascontiguousarray(vel[:first]), start=emit_id)
        if first < n:
            self.set_array(ARRAY_POS, np.ascontiguousarray(pos[first:]), start=0)
            self.set_array(ARRAY_VEL, np.ascontiguousarray(vel[first:]), start=0)
        nxt = emit_id + n
        return nxt - total if nxt >= total else nxt

    def update(self, steps: int = 1) -> None:
        """cSPH::Update (SPH_Update.cpp:12-81), `steps` times."""
        check(lib().sph_step(self._h, steps))

    def set_graph_steps(self, steps: int) -> None:
        check(lib().sph_set_graph_steps(self._h, steps))

    def set_color_output(self, clr=None, dye=None) -> None:
        """Colour (float4) and dye (float) of every following step, written
        into caller-owned device tensors of n records in original order;
        None turns the output off.  The tensors must outlive their use."""
        self._color_keep = (clr, dye)
        p = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())  # noqa: E731
        check(lib().sph_set_color_output(self._h, p(clr), p(dye)))

    def set_persistent(self, on: bool = True) -> None:
        """update(k) as one cooperative launch of k steps (same results)."""
        check(lib().sph_set_persistent(self._h, int(on)))

    # by shape (sph_set_walk_shape): threads per block, staged density walk
    WALK_THREADS = (64, 128, 256, 128, 128, 256, 128, 128, 64, 128, 64)
    WALK_STAGED = (False, False, False, True, True, True, True, False, True, True, True)
    # kernel names of the (density, force) walks by shape
    WALK_KERNELS = (("k_density", "k_force"),) * 3 + (("k_density_tile", "k_force_tile"),
                    ("k_density_pairs", "k_force_fields"), ("k_density_pairs", "k_force_fields"),
                    ("k_density_pairs", "k_force"), ("k_density", "k_force_fields"),
                    ("k_density_pairs", "k_force_fields"), ("k_density_pairs", "k_force_coop"),
                    ("k_density_pairs", "k_force_coop"))

    def set_walk_shape(self, shape: int) -> None:
        check(lib().sph_set_walk_shape(self._h, shape))

    def walk_shape(self) -> int:
        sh = ctypes.c_uint32()
        check(lib().sph_get_walk_shape(self._h, ctypes.byref(sh), None))
        return sh.value

    def autotune(self, trial_steps: int = 10):
        """Pick the fastest walk launch shape on this handle's scenes; returns
        (chosen shape, ms per step of each shape).  State is unchanged."""
        ms = (ctypes.c_float * len(self.WALK_THREADS))()
        ch = ctypes.c_uint32()
        check(lib().sph_autotune(self._h, trial_steps, ms, ctypes.byref(ch)))
        return ch.value, list(ms)

    STAGES = ("integrate_count", "scan", "scatter_ids", "place", "density", "force")

    def step_timed(self) -> dict:
        """One step with per-stage CUDA-event times (ms) on the handle's stream."""
        out = (ctypes.c_float * len(self.STAGES))()
        check(lib().sph_step_timed(self._h, out, len(self.STAGES)))
        return dict(zip(self.STAGES, list(out)))

    def cells(self):
        """(sortedHash (N,2) uint32, cellStart (C,), cellEnd (C,)) of the last step."""
        h = np.empty((self.n, 2), np.uint32)
        cs = np.empty(self.num_cells, np.uint32)
        ce = np.empty(self.num_cells, np.uint32)
        check(lib().sph_get_cells(self._h, ctypes.c_void_p(h.ctypes.data),
                                  ctypes.c_void_p(cs.ctypes.data), ctypes.c_void_p(ce.ctypes.data), 0))
        return h, cs, ce

    def fields(self):
        """(density, pressure) of the last step, sorted order."""
        d = np.empty(self.n, np.float32)
        p = np.empty(self.n, np.float32)
        check(lib().sph_get_fields(self._h, ctypes.c_void_p(d.ctypes.data),
                                   ctypes.c_void_p(p.ctypes.data), 0))
        return d, p

    def stats(self) -> np.ndarray:
        """(scenes, 4) doubles: KE, mean density, max |rho/rho0-1|, non-finite count."""
        out = (ctypes.c_double * (4 * self.num_scenes))()
        check(lib().sph_stats(self._h, out))
        return np.array(out, dtype=np.float64).reshape(self.num_scenes, 4)

    def flags(self) -> int:
        f = ctypes.c_uint32()
        check(lib().sph_flags(self._h, ctypes.byref(f)))
        return f.value


class _Stage:
    """The reference's per-stage wrappers (System.cuh, radixsort.cuh) over
    device pointers (torch CUDA tensors)."""

    @staticmethod
    def _p(t):
        if t is None:
            return ctypes.c_void_p(0)
        if not (_is_torch(t) and t.is_cuda):
            raise TypeError("stage entry points take CUDA tensors")
        return ctypes.c_void_p(t.data_ptr())

    def set_parameters(self, p: SimParams) -> None:
        check(lib().sph_setParameters(ctypes.byref(p)))

    def set_stream(self, stream) -> None:
        handle = getattr(stream, "cuda_stream", stream)
        check(lib().sph_setStageStream(ctypes.c_void_p(handle or 0)))

    def integrate(self, old_pos, new_pos, old_vel, new_vel, n: int) -> None:
        P = self._p
        check(lib().sph_integrate(P(old_pos), P(new_pos), P(old_vel), P(new_vel), n))

    def calc_hash(self, pos, particle_hash, n: int) -> None:
        check(lib().sph_calcHash(self._p(pos), self._p(particle_hash), n))

    def radix_sort(self, d0, d1, n: int, bits: int) -> None:
        check(lib().sph_RadixSort(self._p(d0), self._p(d1), n, bits))

    def reorder(self, old_pos, old_vel, sorted_pos, sorted_vel, particle_hash, cell_start,
                n: int, num_cells: int) -> None:
        P = self._p
        check(lib().sph_reorder(P(old_pos), P(old_vel), P(sorted_pos), P(sorted_vel),
                                P(particle_hash), P(cell_start), n, num_cells))

    def collide(self, sorted_pos, sorted_vel, new_vel, pressure, density, particle_hash,
                cell_start, n: int, num_cells: int, clr=None, dye=None) -> None:
        P = self._p
        check(lib().sph_collide(None, None, P(clr), P(sorted_pos), P(sorted_vel), None,
                                P(new_vel), P(pressure), P(density), P(dye), P(particle_hash),
                                P(cell_start), n, num_cells))

    def sync(self) -> None:
        check(lib().sph_threadSync())


stage = _Stage()
