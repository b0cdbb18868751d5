"""Host-side mirror of the reference's tracer / hitter / imager call surface.

The reference dispatches on hitter and tracer types
(src/alg_types.jl:8-124): ``next_hit!(tracer, hitter, rays, n_tris)``,
``run_evolution!(hitter, tracer; depth, first_diffuse, n_tris, tris, rays,
force_rand)``, ``continuum_light_map2!(; tracer, tris, rays, spectrum, tex)``,
``rays_from_lights(lights, upscale)``.  The functions here keep those names,
argument meanings and in-place semantics, and call libsplat through its C ABI.
Device memory is torch tensors (uint8 byte buffers for the reference's
ADRay records); every call enqueues on the current torch CUDA stream.

Julia's ``!`` suffix is dropped from the names: ``next_hit``,
``run_evolution``, ``continuum_light_map2``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _lib as L
from . import types as T

BRUTE = L.HITTER_BRUTE
BVH = L.HITTER_BVH
BVH2 = L.HITTER_BVH2


def _torch():
    import torch

    return torch


def _stream() -> int:
    torch = _torch()
    return torch.cuda.current_stream().cuda_stream


def _ptr(t) -> int:
    return 0 if t is None else int(t.data_ptr())


def _material(m) -> L.Material:
    mat = L.Material(kind=int(m[0]), a=float(m[1]), b=float(m[2]))
    if len(m) > 3:
        for i in range(3):
            mat.sb[i] = float(m[3][i])
            mat.sc[i] = float(m[4][i])
    return mat


def _light(rec) -> L.RectLight:
    li = L.RectLight()
    for f in ("center", "dir", "dim1", "dim2"):
        arr = getattr(li, f)
        for i in range(3):
            arr[i] = float(rec[f][i])
    li.res1 = int(rec["res1"])
    li.res2 = int(rec["res2"])
    return li


def _lmode(lm) -> L.LambdaMode:
    return L.LambdaMode(mode=int(lm[0]), n_strata=int(lm[1]), lambda0=float(lm[2]), lambda1=float(lm[3]))


class Scene:
    """Resident scene: FTri array, hoisted hit records and (optionally) the
    BVH.  The analogue of building n_tris plus a DPBVHitter / ExperimentalHitter6
    (src/tracer.jl:313, src/alg_types.jl:53-90)."""

    def __init__(self, tris: np.ndarray, first_diffuse: int, bvh: bool = True):
        lib = L.load()
        self.tris_host = np.ascontiguousarray(tris, dtype=np.float32)
        assert self.tris_host.ndim == 3 and self.tris_host.shape[1:] == (10, 3)
        self.n_tris = int(self.tris_host.shape[0])
        self.first_diffuse = int(first_diffuse)
        self.has_bvh = bool(bvh)
        h = C.c_void_p()
        L.check(lib.splat_scene_create(self.tris_host.ctypes.data, self.n_tris, self.first_diffuse, int(bvh),
                                       _stream(), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        if self._h is None:
            raise L.SplatError(L.ERR_INVALID, "scene is closed")
        return self._h

    def info(self) -> dict:
        inf = L.SceneInfo()
        L.check(L.load().splat_scene_info(self.handle, C.byref(inf)))
        return {f: (list(getattr(inf, f)) if f.startswith("bounds") else getattr(inf, f)) for f, _ in inf._fields_}

    def update(self, d_tris) -> None:
        """Per-frame geometry upload (repack + BVH refit) from a device FTri tensor."""
        L.check(L.load().splat_scene_update(self.handle, _ptr(d_tris), _stream()))

    def rebuild(self, d_tris=None) -> None:
        """Per-frame geometry upload with the BVH rebuilt on the GPU."""
        L.check(L.load().splat_scene_rebuild(self.handle, _ptr(d_tris), _stream()))

    def errors(self, reset: bool = True) -> int:
        """The device error word (16: a hit index outside 1..n_tris); syncs."""
        out = C.c_int32(0)
        L.check(L.load().splat_scene_errors(self.handle, int(reset), C.byref(out), _stream()))
        return int(out.value)

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            L.load().splat_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# rays
# ---------------------------------------------------------------------------
def rays_to_device(rays: np.ndarray):
    torch = _torch()
    assert rays.dtype == T.ADRAY
    return torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8)).cuda()


def rays_to_host(d_rays) -> np.ndarray:
    return d_rays.cpu().numpy().view(T.ADRAY).copy()


def n_rays_of(d_rays) -> int:
    return d_rays.numel() // T.ADRAY.itemsize


def rays_from_light(light, upscale: int = 1, lambda_mode=(T.LAMBDA_FIXED, 1, 550.0, 550.0), seed: int = 0,
                    light_index: int = 0):
    """rays_from_light (src/ray_generators.jl:64-97): a device ADRay buffer."""
    torch = _torch()
    n = int(light["res1"] // upscale) * int(light["res2"] // upscale)
    out = torch.empty(n * T.ADRAY.itemsize, dtype=torch.uint8, device="cuda")
    li, lm = _light(light), _lmode(lambda_mode)
    L.check(L.load().splat_rays_from_light(C.byref(li), int(upscale), C.byref(lm), int(seed), int(light_index),
                                           _ptr(out), _stream()))
    return out


def rays_from_lights(lights: Sequence, upscale: int = 1, lambda_mode=(T.LAMBDA_FIXED, 1, 550.0, 550.0),
                     seed: int = 0):
    """rays_from_lights (src/ray_generators.jl:99-113): the lights' rays concatenated."""
    torch = _torch()
    parts = [rays_from_light(l, upscale, lambda_mode, seed, i) for i, l in enumerate(lights)]
    return parts[0] if len(parts) == 1 else torch.cat(parts)


# ---------------------------------------------------------------------------
# hitters
# ---------------------------------------------------------------------------
def n_tris_array(tris: np.ndarray):
    """The reference's n_tris = tuple.(1:T, tri_from_ftri.(tris)) as a device
    buffer of Tuple{Int32,Tri} records (52 bytes)."""
    torch = _torch()
    tris = np.ascontiguousarray(tris, dtype=np.float32)
    rec = np.zeros((tris.shape[0], 13), dtype=np.float32)
    rec[:, 0] = np.arange(1, tris.shape[0] + 1, dtype=np.int32).view(np.float32)
    rec[:, 1:] = tris[:, :4, :].reshape(-1, 12)
    return torch.from_numpy(rec.view(np.uint8).reshape(-1)).cuda()


def next_hit_brute(d_rays, d_n_tris, tmp=None):
    """next_hit!(tracer, ::ExperimentalHitter6, rays, n_tris) (src/hitters.jl:205-226).
    Returns (hit_idx, tmp) with tmp the packed (t, index) argmin words."""
    torch = _torch()
    n = n_rays_of(d_rays)
    nt = d_n_tris.numel() // 52
    if tmp is None:
        tmp = torch.empty(n, dtype=torch.int64, device="cuda")
    hit = torch.empty(n, dtype=torch.int32, device="cuda")
    L.check(L.load().splat_next_hit_brute(_ptr(d_rays), n, _ptr(d_n_tris), nt, _ptr(tmp), _ptr(hit), _stream()))
    return hit, tmp


def next_hit(scene: Scene, hitter: int, d_rays, with_t: bool = False):
    """next_hit! with a resident scene; hitter BRUTE or BVH."""
    torch = _torch()
    n = n_rays_of(d_rays)
    hit = torch.empty(n, dtype=torch.int32, device="cuda")
    t = torch.empty(n, dtype=torch.float32, device="cuda") if with_t else None
    L.check(L.load().splat_next_hit(scene.handle, int(hitter), _ptr(d_rays), n, _ptr(hit), _ptr(t), _stream()))
    return (hit, t) if with_t else hit


def run_evolution(hitter: int, scene: Scene, d_rays, depth: int, material, force_rand: Optional[float] = None,
                  seed: int = 0, quirks: bool = True, workspace=None):
    """run_evolution! (src/tracer.jl:233-282): evolves d_rays in place and
    returns the realigned hit indices."""
    torch = _torch()
    lib = L.load()
    n = n_rays_of(d_rays)
    need = int(lib.splat_run_evolution_workspace_size(n))
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(need, dtype=torch.uint8, device="cuda")
    hit = torch.empty(n, dtype=torch.int32, device="cuda")
    mat = _material(material)
    fr = -1.0 if force_rand is None else float(force_rand)
    L.check(lib.splat_run_evolution(scene.handle, int(hitter), _ptr(d_rays), n, int(depth), C.byref(mat), fr,
                                    int(seed), L.FLAG_REF_QUIRKS if quirks else 0, _ptr(hit), _ptr(workspace),
                                    workspace.numel(), _stream()))
    return hit


def evolve(scene: Scene, d_rays, hit_idx, material, rndm=None, force_rand: Optional[float] = None, seed: int = 0,
           bounce: int = 1, quirks: bool = True):
    """One `rays .= evolve_ray.(rays, hit_idx, tri_view, rndm, first_diffuse)`
    (src/tracer.jl:181-201, 246-256) in place; rndm is a device float32
    array of per-ray Fresnel draws, or None for force_rand / Philox(seed)."""
    n = n_rays_of(d_rays)
    mat = _material(material)
    fr = -1.0 if force_rand is None else float(force_rand)
    L.check(L.load().splat_evolve(scene.handle, _ptr(d_rays), n, _ptr(hit_idx), _ptr(rndm), C.byref(mat), fr,
                                  int(seed), int(bounce), L.FLAG_REF_QUIRKS if quirks else 0, _stream()))
    return d_rays


def partition(d_rays, workspace=None):
    """partition!(rays, ray_swap; by = status != ACTIVE) (src/partition.jl:122-132):
    ACTIVE rays to the front in place; returns the device int64 count."""
    torch = _torch()
    lib = L.load()
    n = n_rays_of(d_rays)
    need = int(lib.splat_partition_workspace_size(n))
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(need, dtype=torch.uint8, device="cuda")
    count = torch.empty(1, dtype=torch.int64, device="cuda")
    L.check(lib.splat_partition(_ptr(d_rays), n, _ptr(count), _ptr(workspace), workspace.numel(), _stream()))
    return count


def new_light_map(w: int, h: int, planes: int, accum: str = "f32"):
    """Light map [w, h, planes] in the reference's column-major order; the
    returned tensor has shape (planes, h, w) over the same memory."""
    torch = _torch()
    dt = torch.float32 if accum == "f32" else torch.int32
    return torch.zeros((planes, h, w), dtype=dt, device="cuda")


def continuum_light_map2(scene: Scene, d_rays, hit_idx, spectrum, upscale: int, tex, frac_bits: int = 16):
    """continuum_light_map2! (src/ray_imagers.jl:142-165): final_evolution of
    the diffuse rays in place, then the splat into tex."""
    torch = _torch()
    n = n_rays_of(d_rays)
    spec = None if spectrum is None else np.ascontiguousarray(spectrum, dtype=np.float32)
    nl = 0 if spec is None else len(spec)
    accum = L.ACCUM_F32 if tex.dtype == torch.float32 else L.ACCUM_I32
    planes, h, w = tex.shape
    L.check(L.load().splat_continuum_light_map(
        scene.handle, _ptr(d_rays), n, _ptr(hit_idx), None if spec is None else spec.ctypes.data, nl, int(upscale),
        _ptr(tex), accum, int(frac_bits), int(w), int(h), _stream()))
    return tex


# ---------------------------------------------------------------------------
# fused trace step
# ---------------------------------------------------------------------------
def trace_params(wl, ray_begin: int = 0, ray_end: int = 0, zero_map: bool = True) -> L.TraceParams:
    """splat_trace_params_t of a scenes.Workload."""
    P = L.TraceParams()
    P.light = _light(wl.light)
    P.upscale = int(wl.upscale)
    P.lambda_mode = _lmode(wl.lambda_mode)
    P.seed = int(wl.seed)
    P.depth = int(wl.depth)
    P.hitter = {"bvh": BVH, "bvh2": BVH2, "brute": BRUTE}[wl.hitter]
    P.material = _material(wl.material)
    P.force_rand = -1.0 if wl.force_rand is None else float(wl.force_rand)
    P.flags = L.FLAG_REF_QUIRKS if wl.quirks else 0
    if wl.spectrum is None:
        P.n_lambda = 0
    else:
        spec = np.asarray(wl.spectrum, dtype=np.float32)
        P.n_lambda = len(spec)
        for i, v in enumerate(spec):
            P.spectrum[i] = float(v)
    P.map_w = int(wl.map_w)
    P.map_h = int(wl.map_h)
    P.accum = L.ACCUM_I32 if wl.accum == "i32" else L.ACCUM_F32
    P.frac_bits = int(wl.frac_bits)
    P.zero_map = 1 if zero_map else 0
    P.ray_begin = int(ray_begin)
    P.ray_end = int(ray_end)
    return P


@dataclass
class StepResult:
    tex: object
    stats: dict


class TraceStep:
    """One forward trace step of a workload with everything resident: scene,
    light map, workspace and stats live on the device and are reused."""

    def __init__(self, wl, scene: Optional[Scene] = None, ray_begin: int = 0, ray_end: int = 0):
        torch = _torch()
        self.wl = wl
        self.scene = scene if scene is not None else Scene(wl.tris, wl.first_diffuse, bvh=(wl.hitter != "brute"))
        self.params = trace_params(wl, ray_begin, ray_end)
        n_grid = wl.n_rays
        re = n_grid if ray_end <= 0 or ray_end > n_grid else ray_end
        self.n = re - ray_begin
        lib = L.load()
        self.ws = torch.empty(int(lib.splat_trace_workspace_size(self.n)), dtype=torch.uint8, device="cuda")
        self.tex = new_light_map(wl.map_w, wl.map_h, wl.n_planes, wl.accum)
        self.d_stats = torch.zeros(16, dtype=torch.int64, device="cuda")

    def run(self, stream: Optional[int] = None):
        lib = L.load()
        L.check(lib.splat_trace_forward(self.scene.handle, C.byref(self.params), _ptr(self.tex), _ptr(self.ws),
                                        self.ws.numel(), _ptr(self.d_stats), _stream() if stream is None else stream))
        return self.tex

    def stats(self) -> dict:
        s = self.d_stats.cpu().numpy()
        return {"rays_per_bounce": [int(x) for x in s[: self.wl.depth]], "diffuse": int(s[8]),
                "samples": int(s[9]), "error": int(s[10])}

    def run_host(self, host_tris: Optional[np.ndarray], host_map: np.ndarray, stream: Optional[int] = None) -> dict:
        """The step through the host-buffer entry point: uploads host_tris
        (if given), traces, downloads the map into host_map."""
        lib = L.load()
        st = L.TraceStats()
        L.check(lib.splat_trace_forward_host(
            self.scene.handle, None if host_tris is None else host_tris.ctypes.data, C.byref(self.params),
            host_map.ctypes.data, _ptr(self.tex), _ptr(self.ws), self.ws.numel(), C.byref(st),
            _stream() if stream is None else stream))
        return {"rays_per_bounce": list(st.rays_per_bounce)[: self.wl.depth]}


def trace_forward(wl, scene: Optional[Scene] = None, ray_begin: int = 0, ray_end: int = 0):
    """Forward half of trace! (src/tracer.jl:317-342) for a workload: returns
    (light map tensor (planes, h, w), stats)."""
    step = TraceStep(wl, scene, ray_begin, ray_end)
    tex = step.run()
    _torch().cuda.synchronize()
    return StepResult(tex, step.stats())


# ---------------------------------------------------------------------------
# camera pass: the backward half of trace! (src/tracer.jl:345-378)
# ---------------------------------------------------------------------------
def camera_look_at(pos, look_at, up, fov: float) -> L.Camera:
    """get_camera (src/geo.jl:183-191); fov in radians."""
    cam = L.Camera()
    f = lambda v: (C.c_float * 3)(*[float(x) for x in v])  # noqa: E731
    L.check(L.load().splat_camera_look_at(f(pos), f(look_at), f(up), float(fov), C.byref(cam)))
    return cam


def camera_rays(cam: L.Camera, height: int, width: int, lam: float = 550.0, seed: int = 0):
    """wrap_ray_gen(camera_ray) (src/ray_generators.jl:18-62) over a
    height x width grid: a device ADRay buffer in pixel order."""
    torch = _torch()
    out = torch.empty(int(height) * int(width) * T.ADRAY.itemsize, dtype=torch.uint8, device="cuda")
    L.check(L.load().splat_camera_rays(C.byref(cam), int(height), int(width), float(lam), int(seed), _ptr(out),
                                       _stream()))
    return out


def retina_factors(spectrum) -> np.ndarray:
    """_spectrum_datastructs (src/rgb_spectrum.jl:135-149): [3, n] float32."""
    spec = np.ascontiguousarray(spectrum, dtype=np.float32)
    out = np.zeros((3, len(spec)), dtype=np.float32)
    L.check(L.load().splat_retina_factors(spec.ctypes.data, len(spec), out.ctypes.data))
    return out


def new_image(height: int, width: int):
    """RGB image, column-major pixels (the reference's RGBf array): a
    (width, height, 3) float32 tensor; image(t) gives [row, col, channel]."""
    return _torch().zeros((int(width), int(height), 3), dtype=_torch().float32, device="cuda")


def image(rgb) -> np.ndarray:
    return rgb.cpu().numpy().transpose(1, 0, 2)


class Shader:
    """The light map and skydome as linear-filtered 3-D textures (the
    reference's CuTexture objects), device arrays reused across frames."""

    def __init__(self, map_w: int, map_h: int, planes: int, sky_w: int = 0, sky_h: int = 0):
        h = C.c_void_p()
        L.check(L.load().splat_shader_create(int(map_w), int(map_h), int(planes), int(sky_w), int(sky_h), C.byref(h)))
        self._h = h
        self.map_w, self.map_h, self.planes = int(map_w), int(map_h), int(planes)

    @property
    def handle(self):
        if self._h is None:
            raise L.SplatError(L.ERR_INVALID, "shader is closed")
        return self._h

    def set_light_map(self, tex, frac_bits: int = 16) -> None:
        """tex: a light map tensor (planes, h, w) from new_light_map."""
        torch = _torch()
        accum = L.ACCUM_F32 if tex.dtype == torch.float32 else L.ACCUM_I32
        assert tuple(tex.shape) == (self.planes, self.map_h, self.map_w)
        L.check(L.load().splat_shader_set_light_map(self.handle, _ptr(tex), accum, int(frac_bits), _stream()))

    def set_skydome(self, sky) -> None:
        """sky: float32 tensor (3, sky_h, sky_w) = the reference's [w, h, 3]."""
        L.check(L.load().splat_shader_set_skydome(self.handle, _ptr(sky.contiguous()), _stream()))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            L.load().splat_shader_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def continuum_shade(scene: Scene, shader: Shader, d_rays, hit_idx, spectrum, retina, upscale: int, height: int,
                    width: int, rgb=None):
    """continuum_shade!(ExperimentalImager2) (src/ray_imagers.jl:441-503) on
    rays after run_evolution: returns the (width, height, 3) image tensor."""
    spec = np.ascontiguousarray(spectrum, dtype=np.float32)
    ret = np.ascontiguousarray(retina, dtype=np.float32).reshape(3, len(spec))
    if rgb is None:
        rgb = new_image(height, width)
    L.check(L.load().splat_continuum_shade(scene.handle, shader.handle, _ptr(d_rays), n_rays_of(d_rays),
                                           _ptr(hit_idx), spec.ctypes.data, ret.ctypes.data, len(spec),
                                           int(upscale), int(height), int(width), _ptr(rgb), _stream()))
    return rgb


def render_params(cam: L.Camera, height: int, width: int, upscale: int, depth: int, material, spectrum,
                  hitter: str = "bvh", seed: int = 0, force_rand: Optional[float] = None, quirks: bool = True,
                  lam: float = 550.0) -> L.RenderParams:
    P = L.RenderParams()
    P.camera = cam
    P.height, P.width, P.upscale = int(height), int(width), int(upscale)
    P.seed = int(seed)
    P.depth = int(depth)
    P.hitter = {"bvh": BVH, "bvh2": BVH2, "brute": BRUTE}[hitter]
    P.material = _material(material)
    P.force_rand = -1.0 if force_rand is None else float(force_rand)
    P.flags = L.FLAG_REF_QUIRKS if quirks else 0
    P.lambda_ = float(lam)
    spec = np.asarray(spectrum, dtype=np.float32)
    ret = retina_factors(spec)
    P.n_lambda = len(spec)
    for i, v in enumerate(spec):
        P.spectrum[i] = float(v)
        for c in range(3):
            P.retina[c][i] = float(ret[c, i])
    return P


class CameraPass:
    """The fused camera pass (splat_render_camera) with its workspace and
    image resident."""

    def __init__(self, scene: Scene, shader: Shader, params: L.RenderParams):
        torch = _torch()
        self.scene, self.shader, self.params = scene, shader, params
        n = (params.height // params.upscale) * (params.width // params.upscale)
        self.ws = torch.empty(int(L.load().splat_render_workspace_size(n)), dtype=torch.uint8, device="cuda")
        self.rgb = new_image(params.height, params.width)

    def run(self, stream: Optional[int] = None, map_ready=None):
        """Enqueue the pass; with map_ready (a torch.cuda.Event) the shading
        waits for it while the camera rays' bounce loop does not."""
        st = _stream() if stream is None else stream
        if map_ready is None:
            L.check(L.load().splat_render_camera(self.scene.handle, self.shader.handle, C.byref(self.params),
                                                 _ptr(self.rgb), _ptr(self.ws), self.ws.numel(), st))
        else:
            L.check(L.load().splat_render_camera_after(self.scene.handle, self.shader.handle, C.byref(self.params),
                                                       _ptr(self.rgb), _ptr(self.ws), self.ws.numel(), st,
                                                       map_ready.cuda_event))
        return self.rgb


_GOLDEN = 0x9E3779B97F4A7C15
_ITER = 0xBF58476D1CE4E5B9
_CAMERA_SALT = 0xD1B54A32D192ED03
_M64 = (1 << 64) - 1


def forward_seed(seed: int, light: int, iteration: int) -> int:
    """Philox key of light `light` (0-based) in iteration `iteration` (1-based)
    of a frame: the workload's own seed for light 0 of iteration 1."""
    return (int(seed) + light * _GOLDEN + (iteration - 1) * _ITER) & _M64


def camera_seed(seed: int, iteration: int) -> int:
    return ((int(seed) ^ _CAMERA_SALT) + (iteration - 1) * _ITER) & _M64


class Renderer:
    """trace! (src/tracer.jl:287-388): per iteration, the forward step of every
    light into the light map (onto a base map, the reference's tex_f()), the
    map into the shader's texture, the camera pass, and the running average of
    the iterations' images.  Light i of iteration k draws with
    forward_seed(seed, i, k); the camera pass with camera_seed(seed, k)."""

    def __init__(self, wl, cam: L.Camera, height: int, width: int, upscale: int = 2, lights: Optional[Sequence] = None,
                 sky=None, base_map=None, iterations: int = 1, scene: Optional[Scene] = None,
                 camera_depth: Optional[int] = None, camera_hitter: Optional[str] = None):
        torch = _torch()
        if wl.spectrum is None:
            raise ValueError("rendering needs a spectrum (one light-map plane per wavelength)")
        self.wl = wl
        self.step = TraceStep(wl, scene)
        self.scene = self.step.scene
        self.lights = list(lights) if lights is not None else [wl.light]
        n_max = max(int(li["res1"] // wl.upscale) * int(li["res2"] // wl.upscale) for li in self.lights)
        if n_max > self.step.n:
            self.step.ws = torch.empty(int(L.load().splat_trace_workspace_size(n_max)), dtype=torch.uint8,
                                       device="cuda")
            self.step.n = n_max
        self.iterations = int(iterations)
        sw, sh = (0, 0) if sky is None else (int(sky.shape[2]), int(sky.shape[1]))
        self.shader = Shader(wl.map_w, wl.map_h, wl.n_planes, sw, sh)
        if sky is not None:
            self.shader.set_skydome(sky)
        self.base = base_map
        self.params = render_params(cam, height, width, upscale, camera_depth or wl.depth, wl.material, wl.spectrum,
                                    camera_hitter or wl.hitter, camera_seed(wl.seed, 1), wl.force_rand, wl.quirks)
        self.camera = CameraPass(self.scene, self.shader, self.params)
        self.out = new_image(height, width)
        self.n_values = self.out.numel()
        self._torch = torch

    def forward(self, iteration: int = 1):
        P = self.step.params
        for i, light in enumerate(self.lights):
            P.light = _light(light)
            P.seed = forward_seed(self.wl.seed, i, iteration)
            first = i == 0
            if first and self.base is not None:
                self.step.tex.copy_(self.base)
            P.zero_map = 1 if first and self.base is None else 0
            self.step.run()
        return self.step.tex

    def run(self):
        """Enqueue the frame on the current stream.  The camera pass runs on a
        second stream: its bounce loop overlaps the forward step, and its
        shading waits for the light map; the current stream waits for the
        image at the end, so the frame is ordered like a one-stream call."""
        lib = L.load()
        torch = self._torch
        main = torch.cuda.current_stream()
        if not hasattr(self, "_cam_stream"):
            self._cam_stream = torch.cuda.Stream()
            self._map_ready = torch.cuda.Event()
            self._shaded = torch.cuda.Event()
        cam = self._cam_stream
        cam.wait_stream(main)  # inputs enqueued before the frame (geometry, base map) are in place
        for k in range(1, self.iterations + 1):
            self.forward(k)
            if k > 1:
                main.wait_event(self._shaded)  # the previous iteration's shading has read the texture
            self.shader.set_light_map(self.step.tex, self.wl.frac_bits)
            self._map_ready.record(main)
            self.params.seed = camera_seed(self.wl.seed, k)
            rgb = self.camera.run(cam.cuda_stream, self._map_ready)
            L.check(lib.splat_image_accumulate(_ptr(self.out), _ptr(rgb), self.n_values, k, cam.cuda_stream))
            self._shaded.record(cam)
        main.wait_event(self._shaded)
        return self.out
