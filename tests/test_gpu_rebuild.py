"""GPU BVH rebuild (splat_scene_rebuild, linear BVH): after a rebuild, with
the same, moved or deformed geometry, every hitter returns the oracle's
brute-force hits bit for bit; tiny and degenerate scenes (one triangle, a
handful, all centroids equal) too; the fused trace step on a rebuilt scene
gives the host-built BVH's map exactly."""
import numpy as np
import pytest

from helpers import random_rays, small_scene
from oracle import oracle as O
from splat_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _hits(tracer, scene, hitter, rays):
    d = tracer.rays_to_device(rays)
    hit, t = tracer.next_hit(scene, hitter, d, with_t=True)
    return hit.cpu().numpy(), t.cpu().numpy()


def _check_all(tracer, scene, tris, rays, what):
    o_hit, o_t = O.next_hit(rays, tris)
    for hitter in (tracer.BRUTE, tracer.BVH, tracer.BVH2):
        hit, t = _hits(tracer, scene, hitter, rays)
        assert np.array_equal(hit, o_hit), f"{what}: hitter {hitter}, {np.count_nonzero(hit != o_hit)} differ"
        assert np.array_equal(t.view(np.uint32), o_t.view(np.uint32)), f"{what}: hitter {hitter} t"
    assert (o_hit > 1).sum() > 0


def _renormal(t):
    a, b = t[:, 1] - t[:, 2], t[:, 2] - t[:, 3]
    t[:, 0] = np.cross(a, b)
    return t


@pytest.mark.parametrize("bvh", [True, False])
def test_rebuild_equals_brute_force_after_deformation(torch_cuda, bvh):
    """A scene built with (or without) a host BVH, rebuilt on the GPU three
    times: unchanged, moved + jittered, then a different shape of the same
    triangle count."""
    import torch

    from splat_gb300 import tracer

    tris, fd = small_scene(3, 0.05)
    scene = tracer.Scene(tris, fd, bvh=bvh)
    rays = random_rays(6000, 21, tris.shape[0])
    scene.rebuild()
    _check_all(tracer, scene, tris, rays, "rebuilt in place")
    rng = np.random.default_rng(5)
    moved = tris.copy()
    moved[1:fd - 1, 1:4] += np.float32(0.3)
    moved[1:fd - 1, 1:4] *= (1 + 0.08 * rng.uniform(-1, 1, size=(fd - 2, 3, 1))).astype(np.float32)
    moved = _renormal(moved)
    scene.rebuild(torch.from_numpy(moved.reshape(-1)).cuda())
    _check_all(tracer, scene, moved, rays, "moved + jittered")
    other, _ = small_scene(3, 0.3)
    other[fd - 1:] = moved[fd - 1:]
    other = _renormal(other)
    scene.update(torch.from_numpy(other.reshape(-1)).cuda())  # after a rebuild, update rebuilds
    _check_all(tracer, scene, other, rays, "reshaped through update")


@pytest.mark.parametrize("n_glass", [1, 2, 3, 4, 5, 17])
def test_rebuild_tiny_scenes(torch_cuda, n_glass):
    from splat_gb300 import tracer

    full, _ = small_scene(2)
    glass = full[1:1 + n_glass]
    tris, fd = S.assemble(glass, np.zeros((0, 10, 3), np.float32))
    scene = tracer.Scene(tris, fd, bvh=False)
    scene.rebuild()
    rays = random_rays(3000, 3 + n_glass, tris.shape[0], aim=0.95)
    o_hit, o_t = O.next_hit(rays, tris)
    for hitter in (tracer.BVH, tracer.BVH2):
        hit, t = _hits(tracer, scene, hitter, rays)
        assert np.array_equal(hit, o_hit) and np.array_equal(t.view(np.uint32), o_t.view(np.uint32))


def test_rebuild_with_coincident_centroids(torch_cuda):
    """Every triangle shares one centroid (all Morton codes equal): the tree
    falls back on the sorted positions."""
    from splat_gb300 import tracer

    rng = np.random.default_rng(9)
    n = 300
    P = rng.normal(size=(n, 3, 3)).astype(np.float32)
    P -= P.mean(axis=1, keepdims=True)
    P[:, 0] = -(P[:, 1] + P[:, 2])  # box centre stays near the origin; nudge to equal centroids below
    lo, hi = P.min(axis=1), P.max(axis=1)
    P -= ((lo + hi) / 2)[:, None, :]
    N = np.zeros_like(P)
    N[:, :, 2] = 1
    tris, fd = S.assemble(S.ftri_records(P, N, np.zeros_like(P)), np.zeros((0, 10, 3), np.float32))
    scene = tracer.Scene(tris, fd, bvh=False)
    scene.rebuild()
    rays = random_rays(3000, 13, tris.shape[0], aim=0.9)
    o_hit, o_t = O.next_hit(rays, tris)
    for hitter in (tracer.BVH, tracer.BVH2):
        hit, t = _hits(tracer, scene, hitter, rays)
        assert np.array_equal(hit, o_hit) and np.array_equal(t.view(np.uint32), o_t.view(np.uint32))


def test_trace_on_rebuilt_scene_equals_host_bvh(torch_cuda):
    from splat_gb300 import tracer

    wl = S.realtime(light=S.scaled_light(S.realtime().light, 512))
    host = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    gpu = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    gpu.rebuild()
    a = tracer.trace_forward(wl, scene=host)
    b = tracer.trace_forward(wl, scene=gpu)
    assert a.stats == b.stats
    assert np.array_equal(a.tex.cpu().numpy(), b.tex.cpu().numpy())
    c = tracer.trace_forward(wl.with_(hitter="bvh2"), scene=gpu)
    assert np.array_equal(a.tex.cpu().numpy(), c.tex.cpu().numpy())


def test_moving_water_surface(torch_cuda):
    """The reference's ripples scene (src/procedural_assets.jl:20-73) animated:
    each frame's surface uploaded and the BVH rebuilt on the GPU; a sampled ray
    range of every frame equals the oracle on that frame's geometry."""
    from splat_gb300 import tracer

    wl0 = S.ripples_scene(0.0)
    scene = tracer.Scene(wl0.tris, wl0.first_diffuse, bvh=True)
    n = wl0.n_rays
    lo = n // 4 + 300  # a range of the light grid above the part of the water over the square
    for t in (0.05, 0.1, 0.15):
        wl = S.ripples_scene(t)
        scene.rebuild(torch_cuda.from_numpy(np.ascontiguousarray(wl.tris).reshape(-1)).cuda())
        r = tracer.trace_forward(wl, scene=scene, ray_begin=lo, ray_end=lo + 1400)
        ref, ref_st, _ = O.trace_forward(wl, lo, lo + 1400)
        assert r.stats["rays_per_bounce"] == [int(x) for x in ref_st[: wl.depth]] and ref_st[1] > 0
        assert np.array_equal(r.tex.cpu().numpy().ravel(), ref.ravel(order="F")) and ref.sum() > 0
