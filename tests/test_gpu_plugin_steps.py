"""The reference-granularity plugin steps through the C ABI: one
`evolve_ray` broadcast (src/tracer.jl:181-201, called at :246-256) and
`partition!` (src/partition.jl:122-132, called at src/tracer.jl:263),
against the CPU restatement; and the experimental tracer's bounce loop
(src/tracer.jl:233-282) composed from those calls."""
import numpy as np
import pytest
from numpy.lib import recfunctions as rfn

from helpers import assert_rays_equal, optics_scenario, small_scene
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


def _sorted_rows(rays: np.ndarray):
    """Row order of rays by the bytes of their fields (a canonical order for
    multisets; padding bytes left out)."""
    packed = rfn.repack_fields(rays)
    b = np.ascontiguousarray(packed).view(np.uint8).reshape(len(rays), packed.dtype.itemsize)
    return np.lexsort(b.T[::-1])


@pytest.mark.parametrize("quirks", [True, False])
@pytest.mark.parametrize("draws", ["array", "seed", "force0", "force1"])
def test_evolve_matches_oracle(torch_cuda, quirks, draws):
    from splat_gb300 import tracer

    tris, fd = small_scene(3, 0.05)
    scene = tracer.Scene(tris, fd, bvh=True)
    rays = O.rays_from_light(S.hemisphere_light(1, 40, 1.05), 1, (T.LAMBDA_UNIFORM, 1, 400.0, 700.0), seed=12)
    mat = S.CAUCHY_GLASS
    rng = np.random.default_rng(3)
    d = tracer.rays_to_device(rays)
    ref = rays
    for bounce in (1, 2, 3):
        hit, _ = O.next_hit(ref, tris)
        n = len(ref)
        if draws == "array":
            rndm = rng.uniform(size=n).astype(np.float32)
            kw = {"rndm": torch_cuda.from_numpy(rndm).cuda()}
        elif draws == "seed":
            rndm = np.array([O.fresnel_draw(77, k, bounce) for k in range(n)], dtype=np.float32)
            kw = {"seed": 77}
        else:
            fr = 0.0 if draws == "force0" else 1.0
            rndm = np.full(n, fr, dtype=np.float32)
            kw = {"force_rand": fr}
        tracer.evolve(scene, d, torch_cuda.from_numpy(hit).cuda(), mat, bounce=bounce, quirks=quirks, **kw)
        ref = O.evolve(ref, hit, tris, rndm, fd, mat, quirks=quirks)
        assert_rays_equal(tracer.rays_to_host(d), ref, f"evolve bounce {bounce}")
    st = np.bincount(ref["status"], minlength=3)
    assert st[T.STATUS_DIFFUSE] > 50


def test_evolve_bad_hit_index_is_reported(torch_cuda):
    from splat_gb300 import tracer

    tris, fd = small_scene(2)
    scene = tracer.Scene(tris, fd, bvh=False)
    rays = O.rays_from_light(S.hemisphere_light(1, 8, 1.05), 1, (T.LAMBDA_FIXED, 1, 550.0, 550.0), seed=1)
    hit, _ = O.next_hit(rays, tris)
    hit[3] = len(tris) + 5
    d = tracer.rays_to_device(rays)
    assert scene.errors() == 0
    tracer.evolve(scene, d, torch_cuda.from_numpy(hit).cuda(), S.CAUCHY_GLASS, force_rand=0.5)
    assert scene.errors() & 16
    assert scene.errors() == 0


@pytest.mark.parametrize("n,p_active", [(0, 0.5), (1, 1.0), (1, 0.0), (257, 0.5), (5000, 0.0), (5000, 1.0),
                                        (100_003, 0.3), (1 << 20, 0.9)])
def test_partition(torch_cuda, n, p_active):
    from splat_gb300 import tracer
    from helpers import random_rays

    rays = random_rays(n, seed=n + 7, n_tris=100) if n else np.zeros(0, dtype=T.ADRAY)
    rng = np.random.default_rng(n)
    if n:
        rays["status"] = np.where(rng.uniform(size=n) < p_active, T.STATUS_ACTIVE,
                                  rng.choice([T.STATUS_DIFFUSE, T.STATUS_INFINITY], size=n))
    d = tracer.rays_to_device(rays) if n else torch_cuda.zeros(0, dtype=torch_cuda.uint8, device="cuda")
    count = int(tracer.partition(d).item())
    got = tracer.rays_to_host(d)
    n_act = int((rays["status"] == T.STATUS_ACTIVE).sum())
    assert count == n_act
    assert (got["status"][:count] == T.STATUS_ACTIVE).all()
    assert (got["status"][count:] != T.STATUS_ACTIVE).all()
    # a permutation of the input
    assert_rays_equal(got[_sorted_rows(got)], rays[_sorted_rows(rays)], "partition")


def test_partition_workspace_checked(torch_cuda):
    from splat_gb300 import _lib as L
    from splat_gb300 import tracer
    from helpers import random_rays

    d = tracer.rays_to_device(random_rays(1000, 1, 10))
    lib = L.load()
    need = int(lib.splat_partition_workspace_size(1000))
    ws = torch_cuda.empty(need - 1, dtype=torch_cuda.uint8, device="cuda")
    cnt = torch_cuda.empty(1, dtype=torch_cuda.int64, device="cuda")
    rc = lib.splat_partition(d.data_ptr(), 1000, cnt.data_ptr(), ws.data_ptr(), need - 1, None)
    assert rc == L.ERR_WORKSPACE


@pytest.mark.parametrize("hitter", ["brute", "bvh"])
@pytest.mark.parametrize("force_rand", [0.0, 1.0])
def test_experimental_loop_composed_from_plugin_steps(torch_cuda, hitter, force_rand):
    """depth x {next_hit!, evolve_ray., partition!, cap to a multiple of 512}
    and the final realigning hit, each a separate libsplat call, give the
    oracle's run_evolution! result as a multiset of (ray, hit) pairs."""
    from splat_gb300 import tracer

    tris, fd = small_scene(3, 0.05)
    scene = tracer.Scene(tris, fd, bvh=True)
    rays = O.rays_from_light(S.hemisphere_light(1, 64, 1.05), 1, (T.LAMBDA_UNIFORM, 1, 400.0, 700.0), seed=4)
    mat = S.CAUCHY_GLASS
    h = tracer.BVH if hitter == "bvh" else tracer.BRUTE
    sz = T.ADRAY.itemsize
    d = tracer.rays_to_device(rays)
    n = len(rays)
    cap = n
    for bounce in range(1, 5):
        view = d[: cap * sz]
        hit = tracer.next_hit(scene, h, view)
        tracer.evolve(scene, view, hit, mat, force_rand=force_rand, bounce=bounce)
        count = int(tracer.partition(view).item())
        cap = min(n, -(-count // 512) * 512) if count else 0
        if cap == 0:
            break
    hit = tracer.next_hit(scene, h, d).cpu().numpy()
    got = tracer.rays_to_host(d)
    ref, ref_hit = O.run_evolution(rays, tris, 4, fd, mat, force_rand)
    ig, ir = _sorted_rows(got), _sorted_rows(ref)
    assert_rays_equal(got[ig], ref[ir], "composed loop")
    assert np.array_equal(hit[ig], ref_hit[ir])


def test_empty_inputs_are_no_ops(torch_cuda):
    """Every plugin entry point accepts zero rays and leaves its outputs
    alone; depth 0 run_evolution! only realigns the hits."""
    from splat_gb300 import tracer

    tris, fd = small_scene(2)
    scene = tracer.Scene(tris, fd, bvh=True)
    empty = torch_cuda.zeros(0, dtype=torch_cuda.uint8, device="cuda")
    assert tracer.next_hit(scene, tracer.BVH, empty).numel() == 0
    assert tracer.next_hit(scene, tracer.BRUTE, empty).numel() == 0
    hit = torch_cuda.zeros(0, dtype=torch_cuda.int32, device="cuda")
    tracer.evolve(scene, empty, hit, S.CAUCHY_GLASS, force_rand=0.5)
    assert tracer.run_evolution(tracer.BVH, scene, empty, 3, S.CAUCHY_GLASS, 0.5).numel() == 0
    tex = tracer.new_light_map(8, 8, 2, "i32")
    tracer.continuum_light_map2(scene, empty, hit, S.stratified_spectrum(2), 1, tex)
    assert int(tex.sum()) == 0
    assert int(tracer.partition(empty).item()) == 0
    rays = O.rays_from_light(S.hemisphere_light(1, 16, 1.05), 1, (T.LAMBDA_FIXED, 1, 550.0, 550.0), seed=2)
    d = tracer.rays_to_device(rays)
    h0 = tracer.run_evolution(tracer.BVH, scene, d, 0, S.CAUCHY_GLASS, 0.5)
    o_hit, _ = O.next_hit(rays, tris)
    assert np.array_equal(h0.cpu().numpy(), o_hit)
    assert_rays_equal(tracer.rays_to_host(d), rays, "depth 0")
    assert scene.errors() == 0


def test_evolve_reference_optics_scenario(torch_cuda):
    """test/optics.jl:1-18 (evolve_ray(adr, 1, t, 1.0f0, 2) on the reference's
    one ray and one triangle, from the committed fixture) through
    splat_evolve: the ray and all its partials equal the oracle's."""
    from splat_gb300 import tracer

    rays, tris, hit, rndm, fd, mat = optics_scenario()
    scene = tracer.Scene(tris, fd, bvh=False)
    d = tracer.rays_to_device(rays)
    tracer.evolve(scene, d, torch_cuda.from_numpy(hit).cuda(), mat, rndm=torch_cuda.from_numpy(rndm).cuda())
    ref = O.evolve(rays, hit, tris, rndm, fd, mat)
    assert_rays_equal(tracer.rays_to_host(d), ref, "optics.jl scenario")
    assert ref[0]["status"] == T.STATUS_ACTIVE and not ref[0]["in_medium"]
    assert scene.errors() == 0
