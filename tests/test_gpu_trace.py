"""The fused forward trace step (splat_trace_forward) against the CPU
restatement of the forward half of trace! (src/tracer.jl:317-342).

Small and sampled cases compare whole light maps with the oracle
(fixed-point maps bit-exact, float maps within 1e-5 relative L1).  At the
benchmark sizes, size-independent properties: brute force == BVH, run-to-run
identity of fixed-point maps, and linearity (the map of all rays equals the
sum of the maps of disjoint ray ranges), plus oracle checks of sampled ranges."""
import numpy as np
import pytest

from helpers import rel_l1
from oracle import oracle as O
from splat_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _gpu(wl, ray_begin=0, ray_end=0, scene=None):
    from splat_gb300 import tracer

    r = tracer.trace_forward(wl, scene=scene, ray_begin=ray_begin, ray_end=ray_end)
    return r.tex.cpu().numpy().ravel(), r.stats


def _cmp(wl, got, ref_tex):
    ref = ref_tex.ravel(order="F")
    if wl.accum == "i32":
        bad = np.nonzero(got != ref)[0]
        assert bad.size == 0, f"{bad.size} texels differ, first {bad[:8]}: {got[bad[:8]]} vs {ref[bad[:8]]}"
    else:
        assert rel_l1(got, ref) <= 1e-5


@pytest.mark.parametrize("accum", ["f32", "i32"])
@pytest.mark.parametrize("hitter", ["brute", "bvh"])
def test_plain_small_reduced(torch_cuda, accum, hitter):
    wl = S.plain_small(light=S.scaled_light(S.plain_small().light, 96), accum=accum, hitter=hitter)
    got, st = _gpu(wl)
    ref_tex, ref_st, _ = O.trace_forward(wl)
    assert st["rays_per_bounce"] == [int(x) for x in ref_st[: wl.depth]]
    assert st["diffuse"] == int(ref_st[6]) and st["samples"] == int(ref_st[7])
    _cmp(wl, got, ref_tex)


@pytest.mark.parametrize("force_rand,quirks", [(0.0, True), (1.0, True), (None, False)])
def test_plain_small_variants(torch_cuda, force_rand, quirks):
    wl = S.plain_small(light=S.scaled_light(S.plain_small().light, 64), accum="i32", force_rand=force_rand,
                       quirks=quirks, material=(0, 0.0, 0.0))
    got, st = _gpu(wl)
    ref_tex, ref_st, _ = O.trace_forward(wl)
    assert st["rays_per_bounce"] == [int(x) for x in ref_st[: wl.depth]]
    _cmp(wl, got, ref_tex)


def test_plain_small_full_size(torch_cuda):
    """The 2^16-ray, 20,480-triangle brute-force workload at full size."""
    wl = S.plain_small()
    got, st = _gpu(wl)
    ref_tex, ref_st, _ = O.trace_forward(wl)
    assert st["rays_per_bounce"] == [int(x) for x in ref_st[: wl.depth]]
    _cmp(wl, got, ref_tex)
    wl_i = wl.with_(accum="i32")
    got_i, _ = _gpu(wl_i)
    ref_i, _, _ = O.trace_forward(wl_i)
    _cmp(wl_i, got_i, ref_i)


@pytest.mark.parametrize("make", [S.realtime, S.menger], ids=["realtime", "menger"])
def test_sampled_ranges_match_oracle(torch_cuda, make):
    """Full-size workloads, disjoint ray ranges in the middle of the light
    grid traced alone, each compared with the oracle."""
    from splat_gb300 import tracer

    wl = make()
    scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    n = wl.n_rays
    h = int(wl.light["res1"]) // wl.upscale
    centres = [n // 2 + h // 2 - 600, n // 3 + h // 3]
    if make is S.menger:
        # the occlusion-heavy sponge: three more ranges across the grid
        centres += [n // 4 + (3 * h) // 8, (5 * n) // 8 + (5 * h) // 8, (3 * n) // 4 + h // 4]
    for c in centres:
        got, st = _gpu(wl, c, c + 1200, scene=scene)
        ref_tex, ref_st, _ = O.trace_forward(wl, c, c + 1200)
        assert st["rays_per_bounce"] == [int(x) for x in ref_st[: wl.depth]]
        assert ref_st[1] > 0, "the sample should reach the glass"
        _cmp(wl, got, ref_tex)


def test_realtime_full_size_properties(torch_cuda):
    """2^20 rays / 81,922 triangles: BVH == brute force, run-to-run identity,
    and linearity over disjoint ray ranges (int32 accumulation)."""
    from splat_gb300 import tracer

    wl = S.realtime()
    scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    a, sa = _gpu(wl, scene=scene)
    b, sb = _gpu(wl, scene=scene)
    assert np.array_equal(a, b) and sa == sb
    for other in ("brute", "bvh2"):
        c, sc = _gpu(wl.with_(hitter=other), scene=scene)
        assert np.array_equal(a, c) and sa["rays_per_bounce"] == sc["rays_per_bounce"]
    n = wl.n_rays
    cuts = [0, n // 3, n // 2 + 17, n]
    parts = sum(_gpu(wl, lo, hi, scene=scene)[0].astype(np.int64) for lo, hi in zip(cuts[:-1], cuts[1:]))
    assert np.array_equal(parts, a.astype(np.int64))
    assert sa["diffuse"] > n // 2 and a.sum() > 0


def test_menger_full_size_properties(torch_cuda):
    """2^22 rays / 96,013 triangles, depth 6 (the occlusion-heavy sponge):
    four-wide BVH == binary BVH == brute force at full size, run-to-run
    identity, and linearity over disjoint ray ranges (int32)."""
    from splat_gb300 import tracer

    wl = S.menger()
    scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    a, sa = _gpu(wl, scene=scene)
    b, sb = _gpu(wl, scene=scene)
    assert np.array_equal(a, b) and sa == sb
    for other in ("bvh2", "brute"):
        c, sc = _gpu(wl.with_(hitter=other), scene=scene)
        assert np.array_equal(a, c) and sa["rays_per_bounce"] == sc["rays_per_bounce"], other
    n = wl.n_rays
    cuts = [0, n // 5, n // 2 + 31, n - 4096, n]
    parts = sum(_gpu(wl, lo, hi, scene=scene)[0].astype(np.int64) for lo, hi in zip(cuts[:-1], cuts[1:]))
    assert np.array_equal(parts, a.astype(np.int64))
    assert sa["rays_per_bounce"][5] > n // 2 and a.sum() > 0


@pytest.mark.parametrize("make", [S.menger, S.realtime], ids=["menger", "realtime"])
@pytest.mark.parametrize("bits,packet", [(16, 1), (20, 1), (20, 2), (12, 4), (20, 5)])
def test_ray_order_keeps_every_map(torch_cuda, make, bits, packet):
    """Secondary rays traced in sorted order (SPLAT_TUNE_RAY_ORDER: octant,
    BVH position of the triangle left) and the packet forms over them give
    the compaction-order step's int32 map and statistics bit for bit, on a
    2^18-ray range of the full-size workload; one small range also against
    the oracle."""
    from splat_gb300 import _lib as L
    from splat_gb300 import tracer

    lib = L.load()
    keys = (L.TUNE_RAY_ORDER, L.TUNE_BVH_PACKET)
    old = [lib.splat_get_tuning(k) for k in keys]
    wl = make()
    scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    n = wl.n_rays
    lo, hi = n // 2 - (1 << 17), n // 2 + (1 << 17)
    try:
        L.check(lib.splat_set_tuning(L.TUNE_RAY_ORDER, 0))
        L.check(lib.splat_set_tuning(L.TUNE_BVH_PACKET, 1))
        ref, sref = _gpu(wl, lo, hi, scene=scene)
        L.check(lib.splat_set_tuning(L.TUNE_RAY_ORDER, bits))
        L.check(lib.splat_set_tuning(L.TUNE_BVH_PACKET, packet))
        got, sg = _gpu(wl, lo, hi, scene=scene)
        c = n // 2 + 300
        small, ss = _gpu(wl, c, c + 1000, scene=scene)
    finally:
        for k, v in zip(keys, old):
            L.check(lib.splat_set_tuning(k, v))
    assert sg == sref and np.array_equal(got, ref) and ref.sum() > 0
    ref_tex, ref_st, _ = O.trace_forward(wl, c, c + 1000)
    assert ss["rays_per_bounce"] == [int(x) for x in ref_st[: wl.depth]]
    _cmp(wl, small, ref_tex)


def test_host_entry_point_matches_device(torch_cuda):
    """splat_trace_forward_host (host triangles in, host map out, scene
    repack + BVH refit in between) equals the resident-scene step."""
    from splat_gb300 import tracer

    wl = S.realtime(light=S.scaled_light(S.realtime().light, 512))
    step = tracer.TraceStep(wl)
    dev = step.run().cpu().numpy().ravel()
    host_map = np.zeros(dev.shape, dtype=np.int32)
    st = step.run_host(np.ascontiguousarray(wl.tris), host_map)
    assert np.array_equal(host_map, dev)
    assert st["rays_per_bounce"] == step.stats()["rays_per_bounce"]


@pytest.mark.parametrize("accum", ["i32", "f32"])
def test_splat_aggregation_matches_direct_atomics(torch_cuda, accum):
    """The splat's shared-memory texel table (tuning knob) against direct map
    atomics: int32 maps bit-identical, float maps within 1e-5 relative L1;
    the reduced workload also against the oracle."""
    from splat_gb300 import _lib as L
    from splat_gb300 import tracer

    lib = L.load()
    old = lib.splat_get_tuning(L.TUNE_SPLAT_AGGREGATE)
    wl = S.realtime(light=S.scaled_light(S.realtime().light, 384), accum=accum)
    scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    try:
        L.check(lib.splat_set_tuning(L.TUNE_SPLAT_AGGREGATE, 1))
        agg, sa = _gpu(wl, scene=scene)
        L.check(lib.splat_set_tuning(L.TUNE_SPLAT_AGGREGATE, 0))
        direct, sd = _gpu(wl, scene=scene)
    finally:
        L.check(lib.splat_set_tuning(L.TUNE_SPLAT_AGGREGATE, old))
    assert sa == sd and agg.sum() > 0
    if accum == "i32":
        assert np.array_equal(agg, direct)
    else:
        assert rel_l1(agg, direct) <= 1e-5
    n = wl.n_rays
    h = int(wl.light["res1"]) // wl.upscale
    lo = n // 2 + h // 2 - 500
    L.check(lib.splat_set_tuning(L.TUNE_SPLAT_AGGREGATE, 1))
    try:
        got, st = _gpu(wl, lo, lo + 1000, scene=scene)
    finally:
        L.check(lib.splat_set_tuning(L.TUNE_SPLAT_AGGREGATE, old))
    ref_tex, ref_st, _ = O.trace_forward(wl, lo, lo + 1000)
    assert st["rays_per_bounce"] == [int(x) for x in ref_st[: wl.depth]]
    _cmp(wl, got, ref_tex)


@pytest.mark.parametrize("accum", ["i32", "f32"])
@pytest.mark.parametrize("overlap", [1, 2])
def test_splat_overlap_matches_single_splat(torch_cuda, accum, overlap):
    """Queue segments splatted on a side stream while later bounces trace
    (tuning knob) against one splat after the last bounce: int32 maps
    bit-identical, float maps within 1e-5 relative L1, same statistics; the
    reduced workload also against the oracle."""
    from splat_gb300 import _lib as L
    from splat_gb300 import tracer

    lib = L.load()
    old = lib.splat_get_tuning(L.TUNE_SPLAT_OVERLAP)
    wl = S.realtime(light=S.scaled_light(S.realtime().light, 384), accum=accum)
    scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    try:
        L.check(lib.splat_set_tuning(L.TUNE_SPLAT_OVERLAP, overlap))
        seg, ss = _gpu(wl, scene=scene)
        L.check(lib.splat_set_tuning(L.TUNE_SPLAT_OVERLAP, 0))
        one, so = _gpu(wl, scene=scene)
        n = wl.n_rays
        h = int(wl.light["res1"]) // wl.upscale
        lo = n // 2 + h // 2 - 500
        L.check(lib.splat_set_tuning(L.TUNE_SPLAT_OVERLAP, overlap))
        got, st = _gpu(wl, lo, lo + 1000, scene=scene)
    finally:
        L.check(lib.splat_set_tuning(L.TUNE_SPLAT_OVERLAP, old))
    assert ss == so and one.sum() > 0
    if accum == "i32":
        assert np.array_equal(seg, one)
    else:
        assert rel_l1(seg, one) <= 1e-5
    ref_tex, ref_st, _ = O.trace_forward(wl, lo, lo + 1000)
    assert st["rays_per_bounce"] == [int(x) for x in ref_st[: wl.depth]]
    _cmp(wl, got, ref_tex)


def test_many_caller_streams(torch_cuda):
    """The fused step on more caller streams than the library keeps side
    streams for (the least recently used are recycled): every map equals the
    one on the default stream."""
    from splat_gb300 import tracer

    wl = S.realtime(light=S.scaled_light(S.realtime().light, 256))
    scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    ref = tracer.trace_forward(wl, scene=scene).tex.clone()
    streams = [torch_cuda.cuda.Stream() for _ in range(40)]
    outs = []
    for s in streams:
        with torch_cuda.cuda.stream(s):
            outs.append(tracer.trace_forward(wl, scene=scene).tex)
    torch_cuda.cuda.synchronize()
    assert ref.sum() > 0 and all(torch_cuda.equal(o, ref) for o in outs)


@pytest.mark.parametrize("accum", ["i32", "f32"])
def test_ray_ranges_on_concurrent_streams(torch_cuda, accum):
    """The fused step as 2, 3 and 4 ray ranges traced on concurrent streams
    (SPLAT_TUNE_TRACE_SPLIT) against one range: int32 maps and statistics
    identical, float maps within 1e-5 relative L1; the host entry point's
    statistics (now accumulated on the device) match."""
    from splat_gb300 import _lib as L
    from splat_gb300 import tracer

    lib = L.load()
    old = lib.splat_get_tuning(L.TUNE_TRACE_SPLIT)
    wl = S.realtime(light=S.scaled_light(S.realtime().light, 800), accum=accum)  # 160,000 rays, over 2^17
    scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    try:
        L.check(lib.splat_set_tuning(L.TUNE_TRACE_SPLIT, 1))
        one, s1 = _gpu(wl, scene=scene)
        for parts in (2, 3, 4):
            L.check(lib.splat_set_tuning(L.TUNE_TRACE_SPLIT, parts))
            got, sg = _gpu(wl, scene=scene)
            assert sg == s1, (parts, sg, s1)
            if accum == "i32":
                assert np.array_equal(got, one), parts
            else:
                assert rel_l1(got, one) <= 1e-5
            step = tracer.TraceStep(wl, scene)
            host_map = np.zeros(got.shape, dtype=got.dtype)
            st = step.run_host(np.ascontiguousarray(wl.tris), host_map)
            assert st["rays_per_bounce"] == s1["rays_per_bounce"]
    finally:
        L.check(lib.splat_set_tuning(L.TUNE_TRACE_SPLIT, old))
    assert one.sum() > 0


@pytest.mark.parametrize("res1,res2", [(37, 53), (24, 100), (9, 70), (5, 33)])
def test_tiled_first_bounce_on_odd_grids(torch_cuda, res1, res2):
    """The first bounce's packets and evolve take a light grid in 8 x 4
    tiles of groups of 16 columns; rows past the last multiple of 8, and
    columns past the last full group, follow in order.  On grids of every
    such shape, with packets on every bounce and whole or column-straddling
    ray ranges, the int32 map and the per-bounce counts equal the oracle's."""
    from splat_gb300 import _lib as L

    lib = L.load()
    base = S.plain_small()
    light = base.light.copy()
    light["res1"], light["res2"] = res1, res2
    wl = S.plain_small(light=light, accum="i32", hitter="bvh")
    old = lib.splat_get_tuning(L.TUNE_BVH_PACKET)
    try:
        L.check(lib.splat_set_tuning(L.TUNE_BVH_PACKET, 2))
        n = res1 * res2
        for rb, re in ((0, 0), (res1 + 3, n - 5), (2 * res1, n)):
            got, st = _gpu(wl, ray_begin=rb, ray_end=re)
            ref_tex, ref_st, _ = O.trace_forward(wl, ray_begin=rb, ray_end=re if re else n)
            assert st["rays_per_bounce"] == [int(x) for x in ref_st[: wl.depth]], (rb, re)
            _cmp(wl, got, ref_tex)
    finally:
        L.check(lib.splat_set_tuning(L.TUNE_BVH_PACKET, old))


def test_counted_traversal_work_matches_the_frame(torch_cuda):
    """The counting kernels (SPLAT_TUNE_COUNT_WORK) trace the same rays as
    the plain ones -- same map, same statistics -- and count every traced
    ray once per bounce; splat_hit_work reads and clears the counters."""
    import ctypes as C

    from splat_gb300 import _lib as L
    from splat_gb300 import tracer

    lib = L.load()
    wl = S.menger(light=S.scaled_light(S.menger().light, 256))
    scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
    ref, sref = _gpu(wl, scene=scene)
    work = (C.c_int64 * 4)()
    stream = torch_cuda.cuda.current_stream().cuda_stream
    L.check(lib.splat_hit_work(work, 1, stream))
    old = lib.splat_get_tuning(L.TUNE_COUNT_WORK)
    try:
        L.check(lib.splat_set_tuning(L.TUNE_COUNT_WORK, 1))
        got, sg = _gpu(wl, scene=scene)
    finally:
        L.check(lib.splat_set_tuning(L.TUNE_COUNT_WORK, old))
    L.check(lib.splat_hit_work(work, 1, stream))
    nodes, pre, full, rays = (int(work[i]) for i in range(4))
    assert np.array_equal(got, ref) and sg == sref
    assert rays == sum(sref["rays_per_bounce"])
    assert nodes > rays and pre >= full > 0
    L.check(lib.splat_hit_work(work, 0, stream))
    assert all(int(work[i]) == 0 for i in range(4))  # cleared by the previous read
