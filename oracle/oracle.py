"""ctypes wrapper of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's cpu_baseline / reference leg, always as the checker or as the
timed CPU baseline, never as part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

from splat_gb300 import types as T

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
rayp = np.ctypeslib.ndpointer(T.ADRAY, flags="C_CONTIGUOUS")


class Material(C.Structure):
    _fields_ = [("kind", C.c_int32), ("a", C.c_float), ("b", C.c_float), ("sb", C.c_float * 3), ("sc", C.c_float * 3)]


class LambdaMode(C.Structure):
    _fields_ = [("mode", C.c_int32), ("n_strata", C.c_int32), ("lambda0", C.c_float), ("lambda1", C.c_float)]


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "oracle.c")):
            build()
        L = C.CDLL(_LIB_PATH)
        vp = C.c_void_p
        L.o_philox4x32_10.argtypes = [vp, vp, vp]
        L.o_uniform.argtypes = [C.c_uint32]
        L.o_uniform.restype = C.c_float
        L.o_monotonic_u32.argtypes = [C.c_float]
        L.o_monotonic_u32.restype = C.c_uint32
        L.o_monotonic_f32.argtypes = [C.c_uint32]
        L.o_monotonic_f32.restype = C.c_float
        L.o_pack_argmin.argtypes = [C.c_float, C.c_uint32]
        L.o_pack_argmin.restype = C.c_uint64
        L.o_retrieve_arg.argtypes = [C.c_uint64]
        L.o_retrieve_arg.restype = C.c_uint32
        L.o_distance_to_plane.argtypes = [f32p, f32p, f32p, f32p]
        L.o_distance_to_plane.restype = C.c_float
        L.o_in_triangle.argtypes = [f32p, f32p, f32p, f32p]
        L.o_reflect.argtypes = [f32p, f32p, f32p]
        L.o_refract.argtypes = [f32p, f32p, C.c_float, C.c_float, f32p]
        L.o_can_refract.argtypes = [f32p, f32p, C.c_float, C.c_float]
        L.o_reflectance.argtypes = [f32p, f32p, C.c_float, C.c_float]
        L.o_reflectance.restype = C.c_float
        L.o_glass.argtypes = [C.POINTER(Material), C.c_float]
        L.o_glass.restype = C.c_float
        L.o_upres.argtypes = [C.c_int, f32p]
        L.o_fresnel_draw.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
        L.o_fresnel_draw.restype = C.c_float
        L.o_rays_from_light.argtypes = [vp, C.c_int64, C.POINTER(LambdaMode), C.c_uint64, C.c_uint32, rayp]
        L.o_next_hit.argtypes = [rayp, C.c_int64, f32p, C.c_int64, i32p, vp, C.c_int]
        L.o_evolve.argtypes = [rayp, C.c_int64, i32p, f32p, f32p, C.c_int64, C.POINTER(Material), C.c_int, C.c_int]
        L.o_run_evolution.argtypes = [rayp, C.c_int64, f32p, C.c_int64, C.c_int32, C.c_int64, C.POINTER(Material),
                                      C.c_float, C.c_uint64, C.c_int, i32p, C.c_int]
        L.o_continuum_light_map.argtypes = [rayp, C.c_int64, i32p, f32p, vp, C.c_int32, C.c_int32, vp, vp, C.c_int32,
                                            C.c_int64, C.c_int64]
        L.o_trace_forward.argtypes = [vp, C.c_int64, C.POINTER(LambdaMode), C.c_uint64, f32p, C.c_int64, C.c_int64,
                                      C.c_int32, C.POINTER(Material), C.c_float, C.c_int, vp, C.c_int32, vp, vp,
                                      C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int64, vp, vp, C.c_int]
        _lib = L
    return _lib


def _v3(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(3))


def material(m) -> Material:
    kind, a, b = m[0], m[1], m[2]
    mat = Material(kind=int(kind), a=float(a), b=float(b))
    if len(m) > 3:
        for i in range(3):
            mat.sb[i] = float(m[3][i])
            mat.sc[i] = float(m[4][i])
    return mat


def lambda_mode(lm) -> LambdaMode:
    return LambdaMode(mode=int(lm[0]), n_strata=int(lm[1]), lambda0=float(lm[2]), lambda1=float(lm[3]))


def philox(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().o_philox4x32_10(c.ctypes.data, k.ctypes.data, out.ctypes.data)
    return out


def monotonic_u32(f: float) -> int:
    return int(lib().o_monotonic_u32(float(f)))


def monotonic_f32(u: int) -> float:
    return float(lib().o_monotonic_f32(int(u)))


def pack_argmin(t: float, i: int) -> int:
    return int(lib().o_pack_argmin(float(t), int(i)))


def retrieve_arg(k: int) -> int:
    return int(lib().o_retrieve_arg(int(k)))


def distance_to_plane(o, d, pp, n) -> np.float32:
    return np.float32(lib().o_distance_to_plane(_v3(o), _v3(d), _v3(pp), _v3(n)))


def in_triangle(p, a, b, c) -> bool:
    return bool(lib().o_in_triangle(_v3(p), _v3(a), _v3(b), _v3(c)))


def reflect(v, n) -> np.ndarray:
    out = np.zeros(3, dtype=np.float32)
    lib().o_reflect(_v3(v), _v3(n), out)
    return out


def refract(v, n, n1, n2) -> np.ndarray:
    out = np.zeros(3, dtype=np.float32)
    lib().o_refract(_v3(v), _v3(n), float(n1), float(n2), out)
    return out


def can_refract(v, n, n1, n2) -> bool:
    return bool(lib().o_can_refract(_v3(v), _v3(n), float(n1), float(n2)))


def reflectance(v, n, n1, n2) -> np.float32:
    return np.float32(lib().o_reflectance(_v3(v), _v3(n), float(n1), float(n2)))


def glass(mat, lam) -> np.float32:
    m = material(mat)
    return np.float32(lib().o_glass(C.byref(m), float(lam)))


def upres(n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.float32)
    lib().o_upres(n, out)
    return out


def fresnel_draw(seed: int, ray_id: int, bounce: int) -> float:
    return float(lib().o_fresnel_draw(seed, ray_id, bounce))


def rays_from_light(light, upscale: int, lm, seed: int, light_index: int = 0) -> np.ndarray:
    n = int(light["res1"] // upscale) * int(light["res2"] // upscale)
    out = np.zeros(n, dtype=T.ADRAY)
    L = np.ascontiguousarray(light)
    lmode = lambda_mode(lm)
    lib().o_rays_from_light(L.ctypes.data, upscale, C.byref(lmode), seed, light_index, out)
    return out


def next_hit(rays: np.ndarray, tris: np.ndarray, nthreads: int = 0):
    tris = np.ascontiguousarray(tris, dtype=np.float32)
    hit = np.zeros(len(rays), dtype=np.int32)
    tt = np.zeros(len(rays), dtype=np.float32)
    lib().o_next_hit(rays, len(rays), tris, tris.shape[0], hit, tt.ctypes.data, nthreads)
    return hit, tt


def evolve(rays: np.ndarray, hit_idx, tris, rndm, first_diffuse, mat, quirks=True, nthreads=0) -> np.ndarray:
    rays = rays.copy()
    m = material(mat)
    lib().o_evolve(rays, len(rays), np.ascontiguousarray(hit_idx, np.int32), np.ascontiguousarray(tris, np.float32),
                   np.ascontiguousarray(rndm, np.float32), first_diffuse, C.byref(m), int(quirks), nthreads)
    return rays


def run_evolution(rays, tris, depth, first_diffuse, mat, force_rand=None, seed=0, quirks=True, nthreads=0):
    rays = rays.copy()
    m = material(mat)
    hit = np.zeros(len(rays), dtype=np.int32)
    fr = -1.0 if force_rand is None else float(force_rand)
    tris = np.ascontiguousarray(tris, np.float32)
    lib().o_run_evolution(rays, len(rays), tris, tris.shape[0], depth, first_diffuse, C.byref(m), fr, seed,
                          int(quirks), hit, nthreads)
    return rays, hit


def continuum_light_map(rays, hit_idx, tris, spectrum, upscale, tex_f32=None, tex_i32=None, frac_bits=16,
                        width=None, height=None):
    rays = rays.copy()
    spec = None if spectrum is None else np.ascontiguousarray(spectrum, np.float32)
    nl = 0 if spec is None else len(spec)
    tex = tex_f32 if tex_f32 is not None else tex_i32
    W, H = (tex.shape[0], tex.shape[1]) if tex is not None else (width, height)
    lib().o_continuum_light_map(rays, len(rays), np.ascontiguousarray(hit_idx, np.int32),
                                np.ascontiguousarray(tris, np.float32), None if spec is None else spec.ctypes.data, nl,
                                upscale, None if tex_f32 is None else tex_f32.ctypes.data,
                                None if tex_i32 is None else tex_i32.ctypes.data, frac_bits, W, H)
    return rays


def new_map(w, h, planes, accum):
    """Light map in the reference's column-major [w, h, planes] layout."""
    dt = np.float32 if accum == "f32" else np.int32
    return np.zeros((w, h, planes), dtype=dt, order="F")


def trace_forward(wl, ray_begin: int = 0, ray_end: Optional[int] = None, nthreads: int = 0, keep_rays: bool = False):
    """Forward trace step of a scenes.Workload over rays [ray_begin, ray_end).
    Returns (map, stats, rays-or-None)."""
    if ray_end is None:
        ray_end = wl.n_rays
    n = ray_end - ray_begin
    tris = np.ascontiguousarray(wl.tris, np.float32)
    tex = new_map(wl.map_w, wl.map_h, wl.n_planes, wl.accum)
    spec = None if wl.spectrum is None else np.ascontiguousarray(wl.spectrum, np.float32)
    stats = np.zeros(8, dtype=np.int64)
    rays = np.zeros(n, dtype=T.ADRAY) if keep_rays else None
    m = material(wl.material)
    lm = lambda_mode(wl.lambda_mode)
    L = np.ascontiguousarray(wl.light)
    fr = -1.0 if wl.force_rand is None else float(wl.force_rand)
    lib().o_trace_forward(
        L.ctypes.data, wl.upscale, C.byref(lm), wl.seed, tris, tris.shape[0], wl.first_diffuse, wl.depth,
        C.byref(m), fr, int(wl.quirks), None if spec is None else spec.ctypes.data, 0 if spec is None else len(spec),
        tex.ctypes.data if wl.accum == "f32" else None, tex.ctypes.data if wl.accum == "i32" else None,
        wl.frac_bits, wl.map_w, wl.map_h, ray_begin, ray_end, None if rays is None else rays.ctypes.data,
        stats.ctypes.data, nthreads)
    return tex, stats, rays
