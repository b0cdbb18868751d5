"""ctypes binding of libsplat.so (include/splat.h).

The library is built in-tree (splat_gb300/libsplat.so).  There is no CPU or
PyTorch fallback: if the library cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsplat.so")

MAX_LAMBDA = 64
STATIC_HIT_MAX_RAYS = 1 << 19

OK = 0
ERR_INVALID = 1
ERR_CUDA = 2
ERR_ALLOC = 3
ERR_WORKSPACE = 4
ERR_DEVICE = 5

HITTER_BRUTE = 0
HITTER_BVH = 1
HITTER_BVH2 = 2
ACCUM_F32 = 0
ACCUM_I32 = 1
FLAG_REF_QUIRKS = 1


class SplatError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"libsplat error {code}: {msg}")
        self.code = code


class RectLight(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("dir", C.c_float * 3), ("dim1", C.c_float * 3),
                ("dim2", C.c_float * 3), ("res1", C.c_int64), ("res2", C.c_int64)]


class Material(C.Structure):
    _fields_ = [("kind", C.c_int32), ("a", C.c_float), ("b", C.c_float), ("sb", C.c_float * 3),
                ("sc", C.c_float * 3)]


class LambdaMode(C.Structure):
    _fields_ = [("mode", C.c_int32), ("n_strata", C.c_int32), ("lambda0", C.c_float), ("lambda1", C.c_float)]


class TraceParams(C.Structure):
    _fields_ = [
        ("light", RectLight), ("upscale", C.c_int64), ("lambda_mode", LambdaMode), ("seed", C.c_uint64),
        ("depth", C.c_int32), ("hitter", C.c_int32), ("material", Material), ("force_rand", C.c_float),
        ("flags", C.c_uint32), ("n_lambda", C.c_int32), ("spectrum", C.c_float * MAX_LAMBDA),
        ("map_w", C.c_int64), ("map_h", C.c_int64), ("accum", C.c_int32), ("frac_bits", C.c_int32),
        ("zero_map", C.c_int32), ("_pad", C.c_int32), ("ray_begin", C.c_int64), ("ray_end", C.c_int64),
    ]


class TraceStats(C.Structure):
    _fields_ = [("rays_per_bounce", C.c_int64 * 8), ("diffuse", C.c_int64), ("samples", C.c_int64),
                ("error", C.c_int64), ("_pad", C.c_int64)]


class SceneInfo(C.Structure):
    _fields_ = [("n_tris", C.c_int64), ("first_diffuse", C.c_int64), ("bvh_nodes", C.c_int64),
                ("bvh_leaves", C.c_int64), ("bvh_depth", C.c_int32), ("bvh_max_leaf", C.c_int32),
                ("device_bytes", C.c_int64), ("bounds_lo", C.c_float * 3), ("bounds_hi", C.c_float * 3),
                ("bvh_pad", C.c_float)]


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("look_at", C.c_float * 3), ("dir", C.c_float * 3), ("up", C.c_float * 3),
                ("right", C.c_float * 3), ("fov_half_sin", C.c_float)]


class RenderParams(C.Structure):
    _fields_ = [
        ("camera", Camera), ("height", C.c_int64), ("width", C.c_int64), ("upscale", C.c_int64),
        ("seed", C.c_uint64), ("depth", C.c_int32), ("hitter", C.c_int32), ("material", Material),
        ("force_rand", C.c_float), ("flags", C.c_uint32), ("lambda_", C.c_float), ("n_lambda", C.c_int32),
        ("spectrum", C.c_float * MAX_LAMBDA), ("retina", (C.c_float * MAX_LAMBDA) * 3),
    ]


# every symbol the header declares, with its ctypes signature
vp = C.c_void_p
i32, i64, u32, u64, f32, sz = C.c_int32, C.c_int64, C.c_uint32, C.c_uint64, C.c_float, C.c_size_t
SIGNATURES = {
    "splat_abi_version": ([], i32),
    "splat_last_error": ([], C.c_char_p),
    "splat_device_info": ([vp, vp, i32], i32),
    "splat_scene_create": ([vp, i64, i64, i32, vp, vp], i32),
    "splat_scene_destroy": ([vp], i32),
    "splat_scene_info": ([vp, C.POINTER(SceneInfo)], i32),
    "splat_scene_update": ([vp, vp, vp], i32),
    "splat_scene_tris": ([vp], vp),
    "splat_scene_errors": ([vp, i32, vp, vp], i32),
    "splat_scene_rebuild": ([vp, vp, vp], i32),
    "splat_rays_from_light": ([C.POINTER(RectLight), i64, C.POINTER(LambdaMode), u64, u32, vp, vp], i32),
    "splat_next_hit_brute": ([vp, i64, vp, i64, vp, vp, vp], i32),
    "splat_next_hit_brute_static": ([vp, i64, vp, i64, vp, vp], i32),
    "splat_next_hit": ([vp, i32, vp, i64, vp, vp, vp], i32),
    "splat_run_evolution_workspace_size": ([i64], sz),
    "splat_run_evolution": ([vp, i32, vp, i64, i32, C.POINTER(Material), f32, u64, u32, vp, vp, sz, vp], i32),
    "splat_evolve": ([vp, vp, i64, vp, vp, C.POINTER(Material), f32, u64, u32, u32, vp], i32),
    "splat_partition_workspace_size": ([i64], sz),
    "splat_partition": ([vp, i64, vp, vp, sz, vp], i32),
    "splat_continuum_light_map": ([vp, vp, i64, vp, vp, i32, i64, vp, i32, i32, i64, i64, vp], i32),
    "splat_trace_workspace_size": ([i64], sz),
    "splat_trace_forward": ([vp, C.POINTER(TraceParams), vp, vp, sz, vp, vp], i32),
    "splat_trace_forward_host": ([vp, vp, C.POINTER(TraceParams), vp, vp, vp, sz, C.POINTER(TraceStats), vp], i32),
    "splat_obj_to_ftri": ([C.c_char_p, vp, i64, C.POINTER(C.c_int64)], i32),
    "splat_camera_look_at": ([vp, vp, vp, C.c_double, C.POINTER(Camera)], i32),
    "splat_camera_rays": ([C.POINTER(Camera), i64, i64, f32, u64, vp, vp], i32),
    "splat_retina_factors": ([vp, i32, vp], i32),
    "splat_shader_create": ([i64, i64, i32, i64, i64, vp], i32),
    "splat_shader_destroy": ([vp], i32),
    "splat_shader_set_light_map": ([vp, vp, i32, i32, vp], i32),
    "splat_shader_set_skydome": ([vp, vp, vp], i32),
    "splat_continuum_shade": ([vp, vp, vp, i64, vp, vp, vp, i32, i64, i64, i64, vp, vp], i32),
    "splat_render_workspace_size": ([i64], sz),
    "splat_render_camera": ([vp, vp, C.POINTER(RenderParams), vp, vp, sz, vp], i32),
    "splat_render_camera_after": ([vp, vp, C.POINTER(RenderParams), vp, vp, sz, vp, vp], i32),
    "splat_image_accumulate": ([vp, vp, i64, i32, vp], i32),
    "splat_batch_device_bytes": ([i32, i64], sz),
    "splat_batch_create": ([i32, i64, vp], i32),
    "splat_batch_destroy": ([vp], i32),
    "splat_batch_admit": ([vp, vp, C.POINTER(TraceParams), vp, C.POINTER(C.c_int32)], i32),
    "splat_batch_tick": ([vp, vp, vp, i32, C.POINTER(C.c_int32)], i32),
    "splat_batch_release": ([vp, i32], i32),
    "splat_batch_status": ([vp, C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_int32)], i32),
    "splat_batch_capture": ([vp, vp, C.POINTER(C.c_int32)], i32),
    "splat_batch_replay": ([vp, vp, i32, vp], i32),
    "splat_server_create": ([i32, i64, i64, i32, vp], i32),
    "splat_server_destroy": ([vp], i32),
    "splat_server_submit": ([vp, vp, C.POINTER(TraceParams), vp, vp], i32),
    "splat_server_step": ([vp, vp, vp, vp], i32),
    "splat_server_poll": ([vp, i32, vp, vp, i32, vp], i32),
    "splat_server_status": ([vp, vp, vp, vp], i32),
    "splat_hit_work": ([vp, i32, vp], i32),
    "splat_set_tuning": ([i32, i32], i32),
    "splat_get_tuning": ([i32], i32),
    "splat_profile_create": ([i32, vp], i32),
    "splat_profile_attach": ([vp], i32),
    "splat_profile_read": ([vp, i32, C.POINTER(C.c_int64), C.POINTER(C.c_double)], i32),
    "splat_profile_reset": ([vp], i32),
    "splat_profile_destroy": ([vp], i32),
}

TUNE_BRUTE_BLOCKS_PER_SM = 0
TUNE_BVH_BLOCKS_PER_SM = 1
TUNE_EVOLVE_BLOCKS_PER_SM = 2
TUNE_SPLAT_BLOCKS_PER_SM = 3
TUNE_SPLAT_AGGREGATE = 4
TUNE_BVH_PACKET = 5
TUNE_SPLAT_OVERLAP = 6
TUNE_BVH_REFILL = 7
TUNE_TRACE_SPLIT = 8
TUNE_TEST_WAIT_STALL = 9
TUNE_RAY_ORDER = 10
TUNE_BRUTE_TILE = 11
TUNE_COUNT_WORK = 12
TUNE_BATCH_PERSISTENT = 13
TUNE_KEYS = 14

KERNEL_GENERATE = 0
KERNEL_HIT_BRUTE = 1
KERNEL_HIT_BVH = 2
KERNEL_EVOLVE = 3
KERNEL_AUX = 4
KERNEL_SPLAT = 5
KERNEL_BATCH = 6
KERNEL_SHADE = 7
KERNEL_ALL = 8

_lib = None
_lock = threading.Lock()


def load(build_if_missing: bool = True):
    """Load libsplat.so (building it with nvcc when it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise SplatError(ERR_INVALID, f"{LIB_PATH} is not built")
            from . import build as _build
            _build.build()
        lib = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
        return lib


def check(rc: int) -> None:
    if rc != OK:
        msg = load().splat_last_error()
        raise SplatError(rc, msg.decode() if msg else "")
