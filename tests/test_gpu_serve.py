"""Serving loop on the GPU: requests arriving while others are in flight
overlap on the device, and each result equals the same frame rendered
alone (int32 maps, bit-exact)."""
import numpy as np
import pytest

from splat_gb300 import scenes as S
from splat_gb300 import types as T

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from splat_gb300 import serve, tracer

    scenes = {0: S.assemble(S.sphere_tris(3, noise_amp=0.05), S.floor_tris(-1.5, 4.0)),
              1: S.assemble(S.menger_tris(2, 2.0, rotation_seed=9), S.box_tris(3.0))}
    pool = serve.ScenePool(lambda sid: scenes[sid], 8 << 30)
    srv = serve.Server(pool, 8 << 30, max_items=16, max_pool_rays=1 << 20)
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
