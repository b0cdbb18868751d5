"""ctypes wrapper of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's cpu_baseline / reference leg, always as the correctness reference or as the
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


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("look_at", C.c_float * 3), ("dir", C.c_float * 3), ("up", C.c_float * 3),
                ("right", C.c_float * 3), ("fov_half_sin", C.c_float)]


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
        L.o_camera_look_at.argtypes = [f32p, f32p, f32p, C.c_double, C.POINTER(Camera)]
        L.o_camera_rays.argtypes = [C.POINTER(Camera), C.c_int64, C.c_int64, C.c_float, C.c_uint64, rayp]
        L.o_continuum_shade.argtypes = [rayp, C.c_int64, i32p, f32p, f32p, f32p, C.c_int32, C.c_int32, f32p,
                                        C.c_int64, C.c_int64, C.c_int64, vp, C.c_int64, C.c_int64, C.c_int64,
                                        C.c_int64, f32p, f32p]
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


# --------------------------------------------------------------------------- camera pass
def camera_look_at(pos, look_at, up, fov: float) -> Camera:
    """get_camera (src/geo.jl:183-191)."""
    cam = Camera()
    lib().o_camera_look_at(_v3(pos), _v3(look_at), _v3(up), float(fov), C.byref(cam))
    return cam


def camera_rays(cam: Camera, h: int, w: int, lam: float = 550.0, seed: int = 0) -> np.ndarray:
    """wrap_ray_gen(camera_ray) over an h x w grid (src/ray_generators.jl:18-62)."""
    out = np.zeros(h * w, dtype=T.ADRAY)
    lib().o_camera_rays(C.byref(cam), h, w, float(lam), int(seed), out)
    return out


# The reference's retina curves (src/rgb_spectrum.jl:32-91) as knots
# (nm, response); integers where the reference writes integers.
RETINA_KNOTS = (
    [(399, 0), (400, 0.0647036), (420, 0.147492), (438, 0.195683), (460, 0.162951), (466, 0), (534, 0),
     (538, 0.243127), (571, 0.798209), (593, 0.980253), (602, 0.999977), (610, 0.98481), (660, 0.375838),
     (680, 0.210109), (700, 0.11005)],
    [(399, 0), (462, 0), (467, 0.165356), (474, 0.280228), (502, 0.587139), (521, 0.829692), (534, 0.924245),
     (551, 0.910167), (572, 0.777366), (600, 0.372516), (609, 0.158767), (612, 0), (700, 0)],
    [(399, 0), (413, 0.23889), (418, 0.291473), (437, 0.437376), (456, 0.590128), (463, 0.72815), (476, 0.581812),
     (494, 0.452254), (515, 0.407615), (528, 0.299756), (536, 0), (608, 0), (611, 0.0407256), (614, 0.154091),
     (620, 0.220637), (635, 0.225269), (667, 0.116114), (700, 0.0424846)],
)


def _piecewise_tree(points):
    """The reference's `piecewise` (src/rgb_spectrum.jl:3-30) restated: a
    binary tree of comparisons `lam < x_i` over 1-based knots, leaves
    interpolating (y1 - y2) / (x1 - x2) * (lam - x1) + y1 with (x1, y1) the
    upper knot of the segment."""
    import math

    def helper(lo, hi, i):
        if hi - lo < 2:
            raise ValueError("bad")
        if hi - lo == 2:
            (x1, y1), (x2, y2) = points[hi - 1], points[lo]
            return ("leaf", x1, y1, x2, y2)
        left = helper(lo, i, int(math.ceil((lo + i) / 2)))
        right = helper(i - 1, hi, int(math.ceil((i + hi) / 2)))
        return ("node", points[i - 1][0], left, right)

    return helper(0, len(points), int(math.ceil(len(points) / 2)))


def _piecewise_eval(tree, lam, f32: bool) -> float:
    node = tree
    while node[0] == "node":
        node = node[2] if lam < node[1] else node[3]
    _, x1, y1, x2, y2 = node
    slope = (y1 - y2) / (x1 - x2)  # Python int / int -> float, float - int -> float, as Julia promotes
    d = float(np.float32(lam) - np.float32(x1)) if f32 else float(lam - x1)
    return float(slope) * d + y1


def retina_factors(spectrum) -> np.ndarray:
    """_spectrum_datastructs (src/rgb_spectrum.jl:135-149): [3, n] float32,
    each curve over its sum at 400..700 nm (a left fold)."""
    spec = np.asarray(spectrum, dtype=np.float32)
    out = np.zeros((3, len(spec)), dtype=np.float32)
    for c, knots in enumerate(RETINA_KNOTS):
        tree = _piecewise_tree(knots)
        norm = _piecewise_eval(tree, 400, False)
        for x in range(401, 701):
            norm = norm + _piecewise_eval(tree, x, False)
        for i, lam in enumerate(spec):
            out[c, i] = np.float32(_piecewise_eval(tree, np.float32(lam), True) / norm)
    return out


def continuum_shade(rays, hit_idx, tris, spectrum, retina, upscale, tex, sky, height, width):
    """continuum_shade!(ExperimentalImager2) (src/ray_imagers.jl:383-503) with
    an exact-weight model of the texture filter.  tex: float32 [w, h, planes]
    (Fortran order), sky: float32 [sw, sh, 3] or None.  Returns (rgb, tol,
    rays): rgb and tol [height, width, 3] per pixel (row, col), rays with the
    diffuse ones final-evolved."""
    rays = rays.copy()
    spec = np.ascontiguousarray(spectrum, np.float32)
    ret = np.ascontiguousarray(retina, np.float32).reshape(3, len(spec))
    texf = np.ascontiguousarray(np.asarray(tex, np.float32).ravel(order="F"))
    tw, th, tp = tex.shape
    if sky is not None:
        skyf = np.ascontiguousarray(np.asarray(sky, np.float32).ravel(order="F"))
        sw, sh = sky.shape[0], sky.shape[1]
    else:
        skyf, sw, sh = None, 0, 0
    rgb = np.zeros(height * width * 3, np.float32)
    tol = np.zeros(height * width * 3, np.float32)
    tris = np.ascontiguousarray(tris, np.float32)
    lib().o_continuum_shade(rays, len(rays), np.ascontiguousarray(hit_idx, np.int32), tris, spec, ret.ravel(),
                            len(spec), upscale, texf, tw, th, tp, None if skyf is None else skyf.ctypes.data, sw, sh,
                            height, width, rgb, tol)
    img = rgb.reshape(width, height, 3).transpose(1, 0, 2)
    tl = tol.reshape(width, height, 3).transpose(1, 0, 2)
    return img, tl, rays


def render_camera(tris, first_diffuse, cam, height, width, upscale, depth, mat, spectrum, retina, tex, sky,
                  seed=0, lam=550.0, force_rand=None, quirks=True, nthreads=0):
    """The camera pass: camera_rays -> run_evolution! -> continuum_shade!."""
    h, w = height // upscale, width // upscale
    rays = camera_rays(cam, h, w, lam, seed)
    rays, hit = run_evolution(rays, tris, depth, first_diffuse, mat, force_rand=force_rand, seed=seed,
                              quirks=quirks, nthreads=nthreads)
    return continuum_shade(rays, hit, tris, spectrum, retina, upscale, tex, sky, height, width)
