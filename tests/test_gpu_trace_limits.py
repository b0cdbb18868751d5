"""The fused trace step at the limits of its parameters and on degenerate
scenes, against the oracle: depth 8, 64 spectrum planes, 16 x 16
sub-samples, every ray missing, a scene without glass, one-ray ranges at
both ends of the light grid, brute force at depth 8."""
import numpy as np
import pytest

from helpers import rel_l1
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


SELLMEIER = (T.MATERIAL_SELLMEIER, 0.0, 0.0, (1.03961212, 0.231792344, 1.01046945),
             (0.00600069867, 0.0200179144, 103.560653))


def _small(**kw):
    tris, fd = S.assemble(S.sphere_tris(3, noise_amp=0.05), S.floor_tris(-1.5, 4.0))
    w = S.Workload(name="limits", tris=tris, first_diffuse=fd, light=S.hemisphere_light(4, 64, 1.05), depth=4,
                   material=S.CAUCHY_GLASS, map_w=64, map_h=48, accum="i32", spectrum=S.stratified_spectrum(4),
                   lambda_mode=(T.LAMBDA_UNIFORM, 1, 400.0, 700.0), hitter="bvh", seed=21)
    return w.with_(**kw) if kw else w


def _run(wl, ray_begin=0, ray_end=0):
    from splat_gb300 import tracer

    scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    r = tracer.trace_forward(wl, scene=scene, ray_begin=ray_begin, ray_end=ray_end)
    return r.tex.cpu().numpy().ravel(), r.stats


def _check(wl, ray_begin=0, ray_end=None):
    got, st = _run(wl, ray_begin, 0 if ray_end is None else ray_end)
    ref, ref_st, _ = O.trace_forward(wl, ray_begin, ray_end)
    k = min(wl.depth, 6)  # the oracle counts the first six bounces; the map covers the rest
    assert st["rays_per_bounce"][:k] == [int(x) for x in ref_st[:k]]
    ref = ref.ravel(order="F")
    if wl.accum == "i32":
        bad = np.nonzero(got != ref)[0]
        assert bad.size == 0, f"{bad.size} texels differ"
    else:
        assert rel_l1(got, ref) <= 1e-5
    return got, st


@pytest.mark.parametrize("hitter", ["bvh", "brute"])
def test_depth_8_sellmeier(torch_cuda, hitter):
    got, st = _check(_small(depth=8, material=SELLMEIER, quirks=False, hitter=hitter))
    assert st["rays_per_bounce"][7] > 0 and got.sum() > 0


@pytest.mark.parametrize("accum", ["i32", "f32"])
def test_64_planes(torch_cuda, accum):
    wl = _small(spectrum=S.stratified_spectrum(64), accum=accum, light=S.hemisphere_light(4, 48, 1.05))
    got, _ = _check(wl)
    assert got.reshape(64, -1).sum(axis=1).min() > 0  # every plane received samples


def test_16x16_subsamples(torch_cuda):
    wl = _small(upscale=16, light=S.hemisphere_light(4, 256, 1.05), spectrum=S.stratified_spectrum(2))
    assert wl.n_rays == 256
    got, _ = _check(wl)
    assert got.sum() > 0


def test_every_ray_misses(torch_cuda):
    light = T.rect_light((0.0, 3.0, 0.0), (0.0, 1.0, 0.0), (1.0, 0.0, 0.0), (0.0, 0.0, 1.0), 32, 32)
    wl = _small(light=light)
    got, st = _check(wl)
    assert st["rays_per_bounce"] == [1024, 0, 0, 0] and got.sum() == 0 and st["diffuse"] == 0


def test_scene_without_glass(torch_cuda):
    tris, fd = S.assemble(np.zeros((0, 10, 3), np.float32), S.floor_tris(-1.5, 4.0))
    assert fd == 2
    wl = _small(tris=tris, first_diffuse=fd)
    got, st = _check(wl)
    assert st["rays_per_bounce"][1] == 0 and st["diffuse"] > 0 and got.sum() > 0


@pytest.mark.parametrize("where", ["first", "last"])
def test_one_ray_ranges(torch_cuda, where):
    wl = _small(light=S.hemisphere_light(4, 256, 1.05))
    n = wl.n_rays
    lo = 0 if where == "first" else n - 1
    _check(wl, lo, lo + 1)
