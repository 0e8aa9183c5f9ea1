"""ctypes binding of libpibiti_sph.so (include/pibiti_sph.h).

The library is built in-tree by ``pibiti_gb300.csrc.build``.  There is no
fallback: if the library is missing, or the GPU path fails, callers get an
exception.
"""
from __future__ import annotations

import ctypes
import os

from .params import SimParams

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libpibiti_sph.so")

SPH_OK = 0
ERRORS = {1: "SPH_ERR_CUDA", 2: "SPH_ERR_ARG", 3: "SPH_ERR_PARAMS", 4: "SPH_ERR_UNSUPPORTED",
          5: "SPH_ERR_TIMEOUT", 6: "SPH_ERR_NOMEM", 7: "SPH_ERR_STATE", 8: "SPH_ERR_XML"}
ARRAY_POS, ARRAY_VEL = 0, 1


class SphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class SceneInfo(ctypes.Structure):
    from .params import Float3 as _F3
    _fields_ = [("title", ctypes.c_char * 64), ("chapter", ctypes.c_int32),
                ("is_default", ctypes.c_int32), ("cellSize", ctypes.c_float),
                ("initMin", _F3), ("initMax", _F3), ("initType", ctypes.c_int32),
                ("initLast", ctypes.c_int32), ("spacing", ctypes.c_float), ("dropR", ctypes.c_float),
                ("rain", ctypes.c_int32)]


NUM_EMIT = 4


class Emitter(ctypes.Structure):
    from .params import Float3 as _F3
    _fields_ = [("pos", _F3), ("rot", _F3), ("vel", ctypes.c_float), ("size", ctypes.c_int32),
                ("size2", ctypes.c_int32)]


class SceneMotion(ctypes.Structure):
    _fields_ = [("emit", Emitter * NUM_EMIT), ("rVel", ctypes.c_float), ("r2Vel", ctypes.c_float)]


_lib = None
vp = ctypes.c_void_p
u32 = ctypes.c_uint32
i32 = ctypes.c_int
P = ctypes.POINTER

# name -> argtypes (restype int unless listed in _RESTYPES)
SIGNATURES = {
    "sph_threadSync": [],
    "sph_allocateArray": [P(vp), ctypes.c_size_t],
    "sph_freeArray": [vp],
    "sph_copyFromDevice": [vp, vp, i32],
    "sph_copyToDevice": [vp, vp, i32, i32],
    "sph_setParameters": [P(SimParams)],
    "sph_setStageStream": [vp],
    "sph_integrate": [vp, vp, vp, vp, i32],
    "sph_calcHash": [vp, vp, i32],
    "sph_RadixSort": [vp, vp, u32, u32],
    "sph_RadixSort_noalloc": [vp, vp, u32, u32],
    "sph_reorder": [vp, vp, vp, vp, vp, vp, u32, u32],
    "sph_collide": [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, u32, u32],
    "sph_create": [P(SimParams), P(vp)],
    "sph_create_ensemble": [P(SimParams), u32, P(vp)],
    "sph_destroy": [vp],
    "sph_set_stream": [vp, vp],
    "sph_set_params": [vp, u32, P(SimParams)],
    "sph_get_params": [vp, u32, P(SimParams)],
    "sph_num_scenes": [vp],
    "sph_num_particles": [vp],
    "sph_scene_offset": [vp, u32],
    "sph_set_array": [vp, u32, vp, u32, u32, i32],
    "sph_get_array": [vp, u32, vp, i32],
    "sph_step": [vp, u32],
    "sph_step_timed": [vp, P(ctypes.c_float), u32],
    "sph_set_graph_steps": [vp, u32],
    "sph_set_color_output": [vp, vp, vp],
    "sph_set_persistent": [vp, i32],
    "sph_persistent_withheld": [vp, P(u32)],
    "sph_set_walk_shape": [vp, u32],
    "sph_get_walk_shape": [vp, P(u32), P(u32)],
    "sph_autotune": [vp, u32, P(ctypes.c_float), P(u32)],
    "sph_get_cells": [vp, vp, vp, vp, i32],
    "sph_get_fields": [vp, vp, vp, i32],
    "sph_num_cells": [vp],
    "sph_stats": [vp, P(ctypes.c_double)],
    "sph_flags": [vp, P(u32)],
    "sph_scene_count": [ctypes.c_char_p, P(i32)],
    "sph_scene_load": [ctypes.c_char_p, i32, P(SimParams), P(SceneInfo)],
    "sph_scene_parse": [ctypes.c_char_p, P(SimParams), P(SceneInfo)],
    "sph_scene_default": [P(SimParams), P(SceneInfo)],
    "sph_scene_default_index": [ctypes.c_char_p, P(i32)],
    "sph_scene_reset": [P(SimParams), P(SceneInfo), i32, ctypes.c_uint64, vp, vp, P(u32)],
    "sph_render_create": [i32, i32, P(vp)],
    "sph_render_destroy": [vp],
    "sph_render_frame": [vp, vp, vp, u32, vp, vp, vp, P(ctypes.c_uint64)],
    "sph_render_foam": [vp, vp, vp, vp, u32, vp, vp],
    "sph_scene_load_motion": [ctypes.c_char_p, i32, P(SceneMotion)],
    "sph_scene_parse_motion": [ctypes.c_char_p, P(SceneMotion)],
    "sph_emitter_particles": [P(Emitter), ctypes.c_float, vp, vp, u32, P(u32)],
    "sph_drop_particles": [P(SimParams), P(SceneInfo), i32, ctypes.c_uint64, vp, vp, u32, P(u32)],
    "sph_scene_advance": [P(SimParams), P(SceneMotion)],
    "sph_mlp_param_count": [],
    "sph_mlp_packed_bytes": [],
    "sph_mlp_pack": [vp, vp, vp],
    "sph_mlp_forward": [vp, vp, u32, vp, vp],
    "sph_mlp_forward_tc": [vp, vp, u32, vp, vp],
    "sph_mlp_forward_tc_withheld": [vp, vp, u32, vp, vp],
    "sph_mlp_status": [P(u32)],
    "sph_mlp_train_pass": [vp, vp, vp, u32, vp, vp, vp],
    "sph_mlp_train_pass_tc": [vp, vp, vp, u32, vp, vp, vp],
    "sph_mlp_train_pass_tc_withheld": [vp, vp, vp, u32, vp, vp, vp],
    "sph_mlp_adam": [vp, vp, vp, vp, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                     ctypes.c_float, u32, vp],
    "sph_learned_set_model": [vp, vp, vp, vp],
    "sph_learned_step": [vp, u32, u32, ctypes.c_float, P(u32)],
    "sph_features_step": [vp, u32, vp, vp],
    "sph_learned_set_options": [vp, ctypes.c_float, ctypes.c_float],
    "sph_last_error": [],
    "sph_version": [],
}
_RESTYPES = {"sph_last_error": ctypes.c_char_p, "sph_version": ctypes.c_char_p,
             "sph_num_scenes": u32, "sph_num_particles": u32, "sph_scene_offset": u32,
             "sph_num_cells": u32}


def lib() -> ctypes.CDLL:
    """Load the library (building it first if the sources are newer)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from .csrc import build as _build
            _build.build()
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing; run pibiti_gb300.csrc.build")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _lib = L
    return _lib


def last_error() -> str:
    return lib().sph_last_error().decode(errors="replace")


def check(rc: int) -> None:
    if rc != SPH_OK:
        raise SphError(rc, last_error())
