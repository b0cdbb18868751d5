"""Hitters on the GPU against the CPU restatement of the reference's
next_hit! (src/hitters.jl:24-30): hit index and binary32 hit distance must be
bit-identical; BVH must equal brute force bit for bit."""
import numpy as np
import pytest

from helpers import assert_rays_equal, random_rays, small_scene
from oracle import oracle as O

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


@pytest.mark.parametrize("subdiv,noise", [(2, 0.0), (3, 0.05)])
def test_brute_and_bvh_match_oracle(torch_cuda, subdiv, noise):
    from splat_gb300 import tracer

    tris, fd = small_scene(subdiv, noise)
    scene = tracer.Scene(tris, fd, bvh=True)
    rays = random_rays(4000, 11 + subdiv, tris.shape[0])
    o_hit, o_t = O.next_hit(rays, tris)
    assert (o_hit > 1).sum() > 1000, "test rays should mostly hit"
    for hitter in (tracer.BRUTE, tracer.BVH, tracer.BVH2):
        hit, t = _hits(tracer, scene, hitter, rays)
        assert np.array_equal(hit, o_hit), f"hitter {hitter}: {np.nonzero(hit != o_hit)[0][:10]}"
        assert np.array_equal(t.view(np.uint32), o_t.view(np.uint32)), f"hitter {hitter}: t bits differ"


@pytest.mark.parametrize("tile", [32, 128])
def test_brute_tile_sizes_match_oracle(torch_cuda, tile):
    """The brute-force hitter with 32 and 128 hit records per ring stage
    (SPLAT_TUNE_BRUTE_TILE) against the oracle, bit for bit."""
    from splat_gb300 import _lib as L
    from splat_gb300 import tracer

    lib = L.load()
    old = lib.splat_get_tuning(L.TUNE_BRUTE_TILE)
    tris, fd = small_scene(3, 0.05)
    scene = tracer.Scene(tris, fd, bvh=False)
    rays = random_rays(5000, 17, tris.shape[0])
    o_hit, o_t = O.next_hit(rays, tris)
    try:
        L.check(lib.splat_set_tuning(L.TUNE_BRUTE_TILE, tile))
        hit, t = _hits(tracer, scene, tracer.BRUTE, rays)
    finally:
        L.check(lib.splat_set_tuning(L.TUNE_BRUTE_TILE, old))
    assert np.array_equal(hit, o_hit)
    assert np.array_equal(t.view(np.uint32), o_t.view(np.uint32))


def test_ntris_dropin_matches_oracle(torch_cuda):
    from splat_gb300 import tracer

    tris, fd = small_scene(3)
    rays = random_rays(3000, 5, tris.shape[0])
    o_hit, o_t = O.next_hit(rays, tris)
    hit, tmp = tracer.next_hit_brute(tracer.rays_to_device(rays), tracer.n_tris_array(tris))
    assert np.array_equal(hit.cpu().numpy(), o_hit)
    packed = tmp.cpu().numpy().view(np.uint64)
    # the packed words decode to the hit distance (src/atomic_argmin.jl:423-431)
    dec = np.array([O.monotonic_f32(int(k >> np.uint64(32))) for k in packed[:500]], dtype=np.float32)
    assert np.array_equal(dec.view(np.uint32), o_t[:500].view(np.uint32))


def test_bvh_equals_brute_large_scene(torch_cuda):
    """81,920-triangle displaced icosphere: BVH == brute on 2^16 rays."""
    from splat_gb300 import scenes as S
    from splat_gb300 import tracer

    wl = S.realtime()
    scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    rays = random_rays(1 << 16, 3, wl.n_tris)
    hb, tb = _hits(tracer, scene, tracer.BRUTE, rays)
    for hitter in (tracer.BVH, tracer.BVH2):
        hv, tv = _hits(tracer, scene, hitter, rays)
        assert np.array_equal(hb, hv)
        assert np.array_equal(tb.view(np.uint32), tv.view(np.uint32))
    sample = np.arange(0, 1 << 16, 97)
    o_hit, o_t = O.next_hit(rays[sample], wl.tris)
    assert np.array_equal(hb[sample], o_hit)


def test_edge_cases(torch_cuda):
    from splat_gb300 import tracer
    from splat_gb300 import types as T

    tris, fd = small_scene(1)
    scene = tracer.Scene(tris, fd, bvh=True)
    rays = random_rays(64, 9, tris.shape[0])
    rays["dir"][0] = 0.0  # zero direction: NaN t, miss
    rays["pos"][1] = np.nan  # NaN origin: miss
    rays["dir"][2] = [0.0, -1.0, 0.0]  # axis-aligned
    rays["pos"][2] = [0.0, 5.0, 0.0]
    o_hit, o_t = O.next_hit(rays, tris)
    for hitter in (tracer.BRUTE, tracer.BVH, tracer.BVH2):
        hit, t = _hits(tracer, scene, hitter, rays)
        assert np.array_equal(hit, o_hit)
    assert o_hit[0] == 1 and o_hit[1] == 1 and o_hit[2] > 1
    # empty ray list
    empty = np.zeros(0, dtype=T.ADRAY)
    import torch

    d = torch.zeros(0, dtype=torch.uint8, device="cuda")
    assert tracer.next_hit(scene, tracer.BRUTE, d).numel() == 0
    # a scene with only the sentinel: everything misses
    only = tracer.Scene(tris[:1], 2, bvh=True)
    for hitter in (tracer.BRUTE, tracer.BVH, tracer.BVH2):
        hit, t = _hits(tracer, only, hitter, rays)
        assert (hit == 1).all() and np.isinf(t).all()
    # one real triangle
    one = tracer.Scene(tris[:2], 3, bvh=True)
    o1, _ = O.next_hit(rays, tris[:2])
    for hitter in (tracer.BRUTE, tracer.BVH, tracer.BVH2):
        hit, _ = _hits(tracer, one, hitter, rays)
        assert np.array_equal(hit, o1)
    del empty


def test_degenerate_geometry_matches_oracle(torch_cuda):
    """Rays starting on triangle planes (num = 0), running parallel to them
    (den = 0), coincident cube faces (exact ties) and grazing hits: brute and
    BVH both equal the oracle."""
    from splat_gb300 import scenes as S
    from splat_gb300 import tracer
    from splat_gb300 import types as T

    tris, fd = S.assemble(S.menger_tris(2, 2.0, rotation_seed=None), S.box_tris(3.0))
    scene = tracer.Scene(tris, fd, bvh=True)
    rng = np.random.default_rng(17)
    n = 6000
    rays = np.zeros(n, dtype=T.ADRAY)
    grid = np.round(rng.uniform(-1, 1, size=(n, 3)) * 9) / 9  # on the sponge's cube planes
    d = rng.normal(size=(n, 3))
    axis = rng.integers(0, 3, size=n)
    par = rng.uniform(size=n) < 0.3
    d[par, axis[par]] = 0.0  # parallel to a family of planes
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["pos"] = grid.astype(np.float32)
    rays["dir"] = d.astype(np.float32)
    rays["ignore_tri"] = np.where(rng.uniform(size=n) < 0.5, rng.integers(2, tris.shape[0] + 1, size=n), 1)
    rays["status"] = T.STATUS_ACTIVE
    o_hit, o_t = O.next_hit(rays, tris)
    for hitter in (tracer.BRUTE, tracer.BVH, tracer.BVH2):
        hit, t = _hits(tracer, scene, hitter, rays)
        bad = np.nonzero(hit != o_hit)[0]
        assert bad.size == 0, f"hitter {hitter}: {bad[:10]} {hit[bad[:5]]} vs {o_hit[bad[:5]]}"
        assert np.array_equal(t.view(np.uint32), o_t.view(np.uint32))
    assert (o_hit > 1).mean() > 0.5


def test_refit_after_geometry_change(torch_cuda):
    """splat_scene_update with moved and deformed triangles: after the repack
    and the bottom-up refit both BVHs still return the brute-force result."""
    import torch

    from splat_gb300 import tracer

    tris, fd = small_scene(3, 0.05)
    scene = tracer.Scene(tris, fd, bvh=True)
    moved = tris.copy()
    rng = np.random.default_rng(5)
    moved[1:fd - 1, 1:4] += np.float32(0.3)  # translate the sphere ...
    moved[1:fd - 1, 1:4] *= (1 + 0.05 * rng.uniform(-1, 1, size=(fd - 2, 3, 1))).astype(np.float32)  # ... and jitter it
    a, b = moved[:, 1] - moved[:, 2], moved[:, 2] - moved[:, 3]
    moved[:, 0] = np.cross(a, b)
    scene.update(torch.from_numpy(moved.reshape(-1)).cuda())
    rays = random_rays(5000, 8, tris.shape[0])
    o_hit, o_t = O.next_hit(rays, moved)
    for hitter in (tracer.BRUTE, tracer.BVH, tracer.BVH2):
        hit, t = _hits(tracer, scene, hitter, rays)
        assert np.array_equal(hit, o_hit), f"hitter {hitter}"
        assert np.array_equal(t.view(np.uint32), o_t.view(np.uint32))


def test_packet_traversal_matches_oracle(torch_cuda):
    """The warp-packet four-wide traversal (SPLAT_TUNE_BVH_PACKET = 2) gives
    the oracle's hits bit for bit on coherent and incoherent rays, through
    the plugin entry and the fused step."""
    from splat_gb300 import _lib as L
    from splat_gb300 import scenes as S
    from splat_gb300 import tracer

    lib = L.load()
    old = lib.splat_get_tuning(L.TUNE_BVH_PACKET)
    tris, fd = small_scene(3, 0.05)
    scene = tracer.Scene(tris, fd, bvh=True)
    light = S.hemisphere_light(2, 96, 1.05)
    coherent = O.rays_from_light(light, 1, (0, 1, 550.0, 550.0), 3)
    incoherent = random_rays(5000, 17, tris.shape[0])
    try:
        L.check(lib.splat_set_tuning(L.TUNE_BVH_PACKET, 2))
        for rays in (coherent, incoherent, incoherent[:37]):
            o_hit, o_t = O.next_hit(rays, tris)
            hit, t = _hits(tracer, scene, tracer.BVH, rays)
            assert np.array_equal(hit, o_hit) and np.array_equal(t.view(np.uint32), o_t.view(np.uint32))
        scene.rebuild()
        hit, t = _hits(tracer, scene, tracer.BVH, incoherent)
        o_hit, o_t = O.next_hit(incoherent, tris)
        assert np.array_equal(hit, o_hit)
        wl = S.realtime(light=S.scaled_light(S.realtime().light, 384))
        sc = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
        maps = []
        for mode in range(6):
            L.check(lib.splat_set_tuning(L.TUNE_BVH_PACKET, mode))
            maps.append(tracer.trace_forward(wl, scene=sc).tex.cpu().numpy())
        assert all(np.array_equal(maps[0], m) for m in maps[1:]) and maps[0].sum() > 0
        L.check(lib.splat_set_tuning(L.TUNE_BVH_PACKET, 5))
        hit, t = _hits(tracer, scene, tracer.BVH, incoherent)
        assert np.array_equal(hit, o_hit)
    finally:
        L.check(lib.splat_set_tuning(L.TUNE_BVH_PACKET, old))


def test_refill_traversal_matches_oracle(torch_cuda):
    """The per-ray four-wide traversal with finished lanes refilled from the
    work counter (SPLAT_TUNE_BVH_REFILL) at several thresholds: run_evolution!
    bit for bit against the oracle, and the fused step's map identical to the
    one without refills."""
    from splat_gb300 import _lib as L
    from splat_gb300 import scenes as S
    from splat_gb300 import tracer
    from splat_gb300 import types as T

    lib = L.load()
    old = lib.splat_get_tuning(L.TUNE_BVH_REFILL)
    tris, fd = small_scene(3, 0.05)
    scene = tracer.Scene(tris, fd, bvh=True)
    rays = O.rays_from_light(S.hemisphere_light(1, 48, 1.05), 1, (T.LAMBDA_UNIFORM, 1, 400.0, 700.0), seed=9)
    ref, ref_hit = O.run_evolution(rays, tris, 4, fd, S.CAUCHY_GLASS, None, seed=3)
    wl = S.realtime(light=S.scaled_light(S.realtime().light, 384))
    sc = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    try:
        L.check(lib.splat_set_tuning(L.TUNE_BVH_REFILL, 0))
        base = tracer.trace_forward(wl, scene=sc).tex.cpu().numpy()
        for m in (1, 7, 32):
            L.check(lib.splat_set_tuning(L.TUNE_BVH_REFILL, m))
            d = tracer.rays_to_device(rays)
            hit = tracer.run_evolution(tracer.BVH, scene, d, 4, S.CAUCHY_GLASS, None, seed=3)
            assert_rays_equal(tracer.rays_to_host(d), ref, f"refill {m}")
            assert np.array_equal(hit.cpu().numpy(), ref_hit)
            got = tracer.trace_forward(wl, scene=sc).tex.cpu().numpy()
            assert np.array_equal(got, base) and base.sum() > 0
    finally:
        L.check(lib.splat_set_tuning(L.TUNE_BVH_REFILL, old))
    assert scene.errors() == 0 and sc.errors() == 0
