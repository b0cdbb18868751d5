"""The camera pass on the GPU against the oracle.

Camera rays and the rays after run_evolution are bit-exact.  Shading goes
through the hardware texture filter (as the reference's CuTexture does),
whose 8-bit fractional weights the oracle models with exact weights plus a
per-value bound (|gpu - oracle| <= tol, tol from the texels' spread), so
images are compared within that bound; the fused form equals the plugin
composition bit for bit."""
import numpy as np
import pytest

from helpers import assert_rays_equal, small_scene
from oracle import oracle as O
from splat_gb300 import scenes as S
from splat_gb300 import types as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


SPEC = np.arange(400, 701, 25, dtype=np.float32)  # 13 planes, the reference's 400:25:700


def _tex(w=64, h=48, planes=len(SPEC), seed=4):
    rng = np.random.default_rng(seed)
    base = rng.uniform(0.0, 30.0, size=(w // 8 + 1, h // 8 + 1, planes))
    # smooth-ish: bilinear upsample of a coarse grid, plus fine noise
    xi = np.linspace(0, w // 8, w)
    yi = np.linspace(0, h // 8, h)
    X0, Y0 = np.floor(xi).astype(int), np.floor(yi).astype(int)
    X1, Y1 = np.minimum(X0 + 1, w // 8), np.minimum(Y0 + 1, h // 8)
    fx, fy = (xi - X0)[:, None, None], (yi - Y0)[None, :, None]
    t = ((1 - fx) * (1 - fy) * base[X0][:, Y0] + fx * (1 - fy) * base[X1][:, Y0] + (1 - fx) * fy * base[X0][:, Y1]
         + fx * fy * base[X1][:, Y1])
    t = t + rng.uniform(0, 1.0, size=t.shape)
    return np.asfortranarray(t.astype(np.float32))


def _dev_map(torch, tex):
    return torch.from_numpy(np.ascontiguousarray(tex.transpose(2, 1, 0))).cuda()


def _dev_sky(torch, sky):
    return torch.from_numpy(np.ascontiguousarray(sky.transpose(2, 1, 0))).cuda()


def _check_image(got, ref, tol, what):
    finite = np.isfinite(tol)
    diff = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    both_nan = np.isnan(got) & np.isnan(ref)
    bad = finite & ~both_nan & ~(diff <= tol + 1e-7)
    assert not bad.any(), (f"{what}: {bad.sum()} values outside tolerance, e.g. {np.argwhere(bad)[:4]}: "
                           f"{got[bad][:4]} vs {ref[bad][:4]} (tol {tol[bad][:4]})")
    assert finite.mean() > 0.99


@pytest.fixture(scope="module")
def setup(torch_cuda):
    from splat_gb300 import tracer

    tris, fd = small_scene(3, 0.04)
    scene = tracer.Scene(tris, fd, bvh=True)
    cam = S.realtime_camera()
    ccam = tracer.camera_look_at(cam["pos"], cam["look_at"], cam["up"], cam["fov"])
    ocam = O.camera_look_at(cam["pos"], cam["look_at"], cam["up"], cam["fov"])
    assert bytes(ccam) == bytes(ocam)
    tex = _tex()
    sky = S.gradient_sky(40, 24)
    shader = tracer.Shader(tex.shape[0], tex.shape[1], tex.shape[2], sky.shape[0], sky.shape[1])
    shader.set_light_map(_dev_map(torch_cuda, tex))
    shader.set_skydome(_dev_sky(torch_cuda, sky))
    return dict(tris=tris, fd=fd, scene=scene, cam=ccam, ocam=ocam, tex=tex, sky=sky, shader=shader)


def test_camera_rays_match_oracle(setup):
    from splat_gb300 import tracer

    for h, w, seed in [(36, 64, 3), (17, 5, 11)]:
        got = tracer.rays_to_host(tracer.camera_rays(setup["cam"], h, w, 550.0, seed))
        assert_rays_equal(got, O.camera_rays(setup["ocam"], h, w, 550.0, seed), f"camera rays {h}x{w}")


@pytest.mark.parametrize("upscale,force_rand", [(2, None), (1, 0.0), (3, 1.0)])
def test_plugin_camera_pass_matches_oracle(setup, upscale, force_rand):
    """camera_rays -> run_evolution! -> continuum_shade! (the reference's
    backward half) against the oracle: rays bit-exact, image within the
    texture-filter bound."""
    from splat_gb300 import tracer

    height, width, depth, seed = 48 * upscale, 60 * upscale, 4, 21
    h, w = height // upscale, width // upscale
    mat = S.CAUCHY_GLASS
    ret = tracer.retina_factors(SPEC)
    d_rays = tracer.camera_rays(setup["cam"], h, w, 550.0, seed)
    hit = tracer.run_evolution(tracer.BVH, setup["scene"], d_rays, depth, mat, force_rand=force_rand, seed=seed)
    rgb = tracer.continuum_shade(setup["scene"], setup["shader"], d_rays, hit, SPEC, ret, upscale, height, width)
    got_img = tracer.image(rgb)
    got_rays = tracer.rays_to_host(d_rays)
    ref_img, tol, ref_rays = O.render_camera(setup["tris"], setup["fd"], setup["ocam"], height, width, upscale, depth,
                                             mat, SPEC, ret, setup["tex"], setup["sky"], seed=seed,
                                             force_rand=force_rand)
    assert_rays_equal(got_rays, ref_rays, "rays after run_evolution + final_evolution")
    st = got_rays["status"]
    assert (st == T.STATUS_DIFFUSE).sum() > 0 and (st == T.STATUS_INFINITY).sum() > 0
    _check_image(got_img, ref_img, tol, f"image upscale {upscale}")


def test_fused_camera_pass_equals_plugin_composition(setup, torch_cuda):
    from splat_gb300 import tracer

    height, width, upscale, depth, seed = 96, 128, 2, 4, 5
    P = tracer.render_params(setup["cam"], height, width, upscale, depth, S.CAUCHY_GLASS, SPEC, "bvh", seed)
    fused = tracer.image(tracer.CameraPass(setup["scene"], setup["shader"], P).run())
    d_rays = tracer.camera_rays(setup["cam"], height // upscale, width // upscale, 550.0, seed)
    hit = tracer.run_evolution(tracer.BVH, setup["scene"], d_rays, depth, S.CAUCHY_GLASS, seed=seed)
    plug = tracer.image(tracer.continuum_shade(setup["scene"], setup["shader"], d_rays, hit, SPEC,
                                               tracer.retina_factors(SPEC), upscale, height, width))
    assert np.array_equal(fused.view(np.uint32), plug.view(np.uint32))
    for hitter in ("brute", "bvh2"):
        P2 = tracer.render_params(setup["cam"], height, width, upscale, depth, S.CAUCHY_GLASS, SPEC, hitter, seed)
        other = tracer.image(tracer.CameraPass(setup["scene"], setup["shader"], P2).run())
        assert np.array_equal(fused.view(np.uint32), other.view(np.uint32)), hitter
    assert fused.max() > 0


def test_int32_light_map_shades_like_its_float_value(setup, torch_cuda):
    """An int32 fixed-point map in the shader equals the float map holding
    value / 2^frac_bits."""
    from splat_gb300 import tracer

    tex = setup["tex"]
    fixed = np.round(tex.astype(np.float64) * 65536).astype(np.int32)
    asfloat = (fixed.astype(np.float32) * np.float32(2.0 ** -16)).astype(np.float32)
    imgs = []
    for m, fb in ((fixed, 16), (np.asfortranarray(asfloat), 16)):
        sh = tracer.Shader(tex.shape[0], tex.shape[1], tex.shape[2])
        sh.set_light_map(_dev_map(torch_cuda, np.asfortranarray(m)), fb)
        P = tracer.render_params(setup["cam"], 64, 64, 2, 3, S.CAUCHY_GLASS, SPEC, "bvh", 9)
        imgs.append(tracer.image(tracer.CameraPass(setup["scene"], sh, P).run()))
    assert np.array_equal(imgs[0].view(np.uint32), imgs[1].view(np.uint32))


def test_renderer_iterations_average(setup, torch_cuda):
    """trace!'s iterations_per_frame: the running average of per-iteration
    images (first copied, then out (k-1)/k + rgb/k), each iteration with its
    own draws; and multiple lights accumulate into one map."""
    from splat_gb300 import tracer

    wl = S.realtime(light=S.scaled_light(S.realtime().light, 128), tris=setup["tris"], first_diffuse=setup["fd"],
                    spectrum=SPEC, lambda_mode=(T.LAMBDA_STRATIFIED, len(SPEC), 400.0, 700.0), map_w=64, map_h=48)
    cam = setup["cam"]
    lights = [wl.light, S.hemisphere_light(7, 128, 1.1)]
    r = tracer.Renderer(wl, cam, 64, 80, 2, lights=lights, iterations=3, scene=setup["scene"])
    out = tracer.image(r.run()).astype(np.float32)
    singles = []
    for k in (1, 2, 3):
        r1 = tracer.Renderer(wl, cam, 64, 80, 2, lights=lights, iterations=1, scene=setup["scene"])
        r1.forward(k)
        r1.shader.set_light_map(r1.step.tex, wl.frac_bits)
        r1.params.seed = tracer.camera_seed(wl.seed, k)
        singles.append(tracer.image(r1.camera.run()).astype(np.float32))
    acc = singles[0].copy()
    for k in (2, 3):
        acc = (acc * np.float32(k - 1)) / np.float32(k) + singles[k - 1] / np.float32(k)
    assert np.array_equal(out.view(np.uint32), acc.view(np.uint32))
    assert not np.array_equal(singles[0], singles[1])
    # two lights: the map is the sum of the lights' maps (int32, exact)
    m2 = r.forward(1).cpu().numpy().astype(np.int64)
    one = tracer.TraceStep(wl, setup["scene"])
    one.params.seed = tracer.forward_seed(wl.seed, 0, 1)
    a = one.run().cpu().numpy().astype(np.int64)
    one.params.light = tracer._light(lights[1])
    one.params.seed = tracer.forward_seed(wl.seed, 1, 1)
    b = one.run().cpu().numpy().astype(np.int64)
    assert np.array_equal(m2, a + b)
