"""rays_from_light, run_evolution! and continuum_light_map2! through the C ABI
against the CPU restatement (src/ray_generators.jl:64-97,
src/tracer.jl:181-282, src/ray_imagers.jl:4-165)."""
import numpy as np
import pytest

from helpers import assert_rays_equal, rel_l1, small_scene
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


LAMBDA_MODES = [(T.LAMBDA_FIXED, 1, 550.0, 550.0), (T.LAMBDA_UNIFORM, 1, 400.0, 700.0),
                (T.LAMBDA_STRATIFIED, 5, 400.0, 700.0)]


@pytest.mark.parametrize("lm", LAMBDA_MODES)
@pytest.mark.parametrize("upscale", [1, 2])
def test_rays_from_light(torch_cuda, lm, upscale):
    from splat_gb300 import tracer

    light = S.hemisphere_light(3, 48, 1.1)
    got = tracer.rays_to_host(tracer.rays_from_light(light, upscale, lm, seed=99))
    ref = O.rays_from_light(light, upscale, lm, seed=99)
    assert_rays_equal(got, ref, "rays_from_light")


MATERIALS = [(T.MATERIAL_LINEAR_REF, 0.0, 0.0), S.CAUCHY_GLASS,
             (T.MATERIAL_SELLMEIER, 0.0, 0.0, (1.03961212, 0.231792344, 1.01046945),
              (0.00600069867, 0.0200179144, 103.560653))]


@pytest.mark.parametrize("hitter", ["brute", "bvh"])
@pytest.mark.parametrize("quirks", [True, False])
@pytest.mark.parametrize("force_rand", [None, 0.0, 1.0])
def test_run_evolution(torch_cuda, hitter, quirks, force_rand):
    from splat_gb300 import tracer

    tris, fd = small_scene(3, 0.05)
    scene = tracer.Scene(tris, fd, bvh=True)
    light = S.hemisphere_light(1, 40, 1.05)
    rays = O.rays_from_light(light, 1, (T.LAMBDA_UNIFORM, 1, 400.0, 700.0), seed=5)
    mat = S.CAUCHY_GLASS
    d = tracer.rays_to_device(rays)
    h = tracer.BVH if hitter == "bvh" else tracer.BRUTE
    hit = tracer.run_evolution(h, scene, d, 4, mat, force_rand, seed=21, quirks=quirks)
    got = tracer.rays_to_host(d)
    ref, ref_hit = O.run_evolution(rays, tris, 4, fd, mat, force_rand, seed=21, quirks=quirks)
    assert_rays_equal(got, ref, "run_evolution")
    assert np.array_equal(hit.cpu().numpy(), ref_hit)
    st = np.bincount(ref["status"], minlength=3)
    assert st[T.STATUS_DIFFUSE] > 100


@pytest.mark.parametrize("mat", MATERIALS, ids=["linear", "cauchy", "sellmeier"])
def test_run_evolution_materials(torch_cuda, mat):
    from splat_gb300 import tracer

    tris, fd = small_scene(3)
    scene = tracer.Scene(tris, fd, bvh=False)
    light = S.hemisphere_light(2, 32, 1.05)
    rays = O.rays_from_light(light, 1, (T.LAMBDA_STRATIFIED, 4, 400.0, 700.0), seed=8)
    d = tracer.rays_to_device(rays)
    hit = tracer.run_evolution(tracer.BRUTE, scene, d, 3, mat, None, seed=4)
    ref, ref_hit = O.run_evolution(rays, tris, 3, fd, mat, None, seed=4)
    assert_rays_equal(tracer.rays_to_host(d), ref, "materials")
    assert np.array_equal(hit.cpu().numpy(), ref_hit)


@pytest.mark.parametrize("accum", ["i32", "f32"])
@pytest.mark.parametrize("spectrum,upscale", [(None, 1), (S.stratified_spectrum(6), 1), (S.stratified_spectrum(3), 2)])
def test_continuum_light_map2(torch_cuda, accum, spectrum, upscale):
    from splat_gb300 import tracer

    tris, fd = small_scene(3, 0.05)
    scene = tracer.Scene(tris, fd, bvh=True)
    light = S.hemisphere_light(1, 48, 1.05)
    rays = O.rays_from_light(light, upscale, (T.LAMBDA_UNIFORM, 1, 400.0, 700.0), seed=3)
    ev, hit = O.run_evolution(rays, tris, 3, fd, S.CAUCHY_GLASS, None, seed=6)
    planes = 1 if spectrum is None else len(spectrum)
    ref_tex = O.new_map(64, 48, planes, accum)
    kw = {"tex_f32": ref_tex} if accum == "f32" else {"tex_i32": ref_tex}
    ref_rays = O.continuum_light_map(ev, hit, tris, spectrum, upscale, **kw)
    d = tracer.rays_to_device(ev)
    dh = torch_cuda.from_numpy(hit).cuda()
    tex = tracer.new_light_map(64, 48, planes, accum)
    tracer.continuum_light_map2(scene, d, dh, spectrum, upscale, tex)
    assert_rays_equal(tracer.rays_to_host(d), ref_rays, "final_evolution")
    got = tex.cpu().numpy().ravel()
    ref = ref_tex.ravel(order="F")
    assert ref.sum() > 0
    if accum == "i32":
        assert np.array_equal(got, ref)
    else:
        assert rel_l1(got, ref) <= 1e-5
