"""Serving loop on the GPU: requests arriving while others are in flight
overlap on the device, and each result equals the same frame rendered
alone (int32 maps, bit-exact)."""
import numpy as np
import pytest

from splat_gb300 import scenes as S
from splat_gb300 import types as T

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("split", [1 << 30, 1000], ids=["whole", "split"])
def test_served_results_equal_alone(split):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from splat_gb300 import serve, tracer

    scenes = {0: S.assemble(S.sphere_tris(3, noise_amp=0.05), S.floor_tris(-1.5, 4.0)),
              1: S.assemble(S.menger_tris(2, 2.0, rotation_seed=9), S.box_tris(3.0))}
    pool = serve.ScenePool(lambda sid: scenes[sid], 8 << 30)
    srv = serve.Server(pool, 8 << 30, max_items=16, max_pool_rays=1 << 20, split_min_rays=split)
    rng = np.random.default_rng(3)
    for rid in range(24):
        sid = rid % 2
        tris, fd = scenes[sid]
        res = int(rng.integers(60, 200))
        light = (S.hemisphere_light(rid, res, 1.1) if sid == 0 else
                 T.rect_light((0.0, 2.6, 0.0), (0.0, -1.0, 0.0), (1.3, 0, 0), (0, 0, 1.3), res, res))
        planes = int(rng.integers(1, 9))
        wl = S.Workload(name=f"r{rid}", tris=tris, first_diffuse=fd, light=light, depth=int(rng.integers(2, 7)),
                        spectrum=S.stratified_spectrum(planes), lambda_mode=(T.LAMBDA_STRATIFIED, planes, 400.0, 700.0),
                        material=S.CAUCHY_GLASS, map_w=int(rng.integers(32, 129)), map_h=64, accum="i32",
                        hitter="bvh", seed=500 + rid)
        srv.submit(serve.Request(arrival=0.002 * rid, rid=rid, scene_id=sid, wl=wl))
    srv.drain()
    assert len(srv.done) == 24
    lat = srv.latencies()
    assert np.all(lat > 0)
    overlapped = sum(1 for r in srv.done if r.done_at > r.arrival + 0.0)  # all completed after arrival
    assert overlapped == 24
    for r in srv.done:
        alone = tracer.trace_forward(r.wl, scene=pool.resident[r.scene_id]).tex
        assert torch.equal(r.tex, alone), f"request {r.rid} differs from its alone result"


def test_served_maps_delivered_then_released():
    """With on_done, each completed request is delivered once (here: its map
    copied to the host), the server keeps no map of its own afterwards, and
    every delivered map equals the frame rendered alone."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from splat_gb300 import serve, tracer

    scenes = {0: S.assemble(S.sphere_tris(3, noise_amp=0.05), S.floor_tris(-1.5, 4.0))}
    pool = serve.ScenePool(lambda sid: scenes[sid], 8 << 30)
    delivered = {}

    def deliver(req):
        assert req.rid not in delivered
        delivered[req.rid] = req.tex.cpu()

    srv = serve.Server(pool, 8 << 30, max_items=16, max_pool_rays=1 << 20, on_done=deliver)
    tris, fd = scenes[0]
    wls = []
    for rid in range(12):
        wl = S.Workload(name=f"d{rid}", tris=tris, first_diffuse=fd, light=S.hemisphere_light(rid, 64 + 8 * rid, 1.1),
                        depth=3, spectrum=S.stratified_spectrum(4), lambda_mode=(T.LAMBDA_STRATIFIED, 4, 400.0, 700.0),
                        material=S.CAUCHY_GLASS, map_w=96, map_h=64, accum="i32", hitter="bvh", seed=900 + rid)
        wls.append(wl)
        srv.submit(serve.Request(arrival=0.001 * rid, rid=rid, scene_id=0, wl=wl))
    srv.drain()
    assert sorted(delivered) == list(range(12))
    assert len(srv.done) == 12 and all(r.tex is None for r in srv.done)
    assert srv.map_bytes_in_use == 0
    for rid, wl in enumerate(wls):
        alone = tracer.trace_forward(wl, scene=pool.resident[0]).tex.cpu()
        assert torch.equal(delivered[rid], alone), f"request {rid} differs from its alone result"


def test_native_server_budget_and_order():
    """splat_server_* directly: with a map budget that holds one request's map
    at a time, requests still complete, one after another, in arrival order,
    each equal to its alone result; a map larger than the budget is refused
    at submission."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctypes as C

    from splat_gb300 import _lib as L
    from splat_gb300 import tracer

    lib = L.load()
    tris, fd = S.assemble(S.sphere_tris(3, noise_amp=0.05), S.floor_tris(-1.5, 4.0))
    scene = tracer.Scene(tris, fd, bvh=True)
    wls = [S.Workload(name=f"q{i}", tris=tris, first_diffuse=fd, light=S.hemisphere_light(i, 96, 1.1), depth=3,
                      spectrum=S.stratified_spectrum(4), lambda_mode=(T.LAMBDA_STRATIFIED, 4, 400.0, 700.0),
                      material=S.CAUCHY_GLASS, map_w=64, map_h=64, accum="i32", hitter="bvh", seed=90 + i)
           for i in range(5)]
    one_map = 64 * 64 * 4 * 4
    h = C.c_void_p()
    L.check(lib.splat_server_create(8, 1 << 20, one_map, 2, C.byref(h)))
    try:
        stream = torch.cuda.current_stream().cuda_stream
        texs, ids = [], []
        for wl in wls:
            tex = tracer.new_light_map(wl.map_w, wl.map_h, wl.n_planes, wl.accum)
            P = tracer.trace_params(wl)
            rid = C.c_int64()
            L.check(lib.splat_server_submit(h, scene.handle, C.byref(P), tex.data_ptr(), C.byref(rid)))
            texs.append(tex)
            ids.append(rid.value)
        big = wls[0].with_(map_w=128)
        P = tracer.trace_params(big)
        rid = C.c_int64()
        assert lib.splat_server_submit(h, scene.handle, C.byref(P), texs[0].data_ptr(), C.byref(rid)) == L.ERR_WORKSPACE
        order = []
        buf, ms = (C.c_int64 * 16)(), (C.c_double * 16)()
        for _ in range(1000):
            fl, q, n = C.c_int32(), C.c_int32(), C.c_int32()
            L.check(lib.splat_server_step(h, stream, C.byref(fl), C.byref(q)))
            assert fl.value <= 1  # one map in flight at a time
            # nothing ticking: wait for the completions that hold the budget
            L.check(lib.splat_server_poll(h, int(fl.value == 0), buf, ms, 16, C.byref(n)))
            order += [buf[i] for i in range(n.value)]
            if len(order) == len(wls):
                break
        assert order == ids
        for wl, tex in zip(wls, texs):
            assert torch.equal(tex, tracer.trace_forward(wl, scene=scene).tex)
    finally:
        lib.splat_server_destroy(h)
