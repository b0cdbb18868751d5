"""The autotuner on the GPU: the batch engine's brute-force vs BVH sweep
runs, and whatever the tuner chooses (a hitter per frame from the
crossover, the batch engine's launch shapes, the plain step's knobs) every
int32 light map stays the map of the frame traced alone, bit for bit."""
import numpy as np
import pytest

from splat_gb300 import scenes as S
from splat_gb300 import types as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(autouse=True)
def tmp_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("SPLAT_TUNE_CACHE", str(tmp_path / "tuning.json"))


@pytest.fixture()
def restore_knobs(torch_cuda):
    from splat_gb300 import autotune as A

    from splat_gb300 import _lib as L

    old = {**A.get_knobs(), **A.get_knobs({L.TUNE_BATCH_PERSISTENT: (0,)})}
    yield
    A.set_knobs(old)


def _frames():
    from splat_gb300 import tracer

    out = []
    for i, (sub, res) in enumerate([(1, 64), (2, 96), (3, 80), (4, 120)]):
        tris, fd = S.assemble(S.sphere_tris(sub, noise_amp=0.05, noise_seed=i), S.floor_tris(-1.5, 4.0))
        wl = S.Workload(name=f"t{i}", tris=tris, first_diffuse=fd, light=S.hemisphere_light(i, res, 1.1), depth=3,
                        spectrum=S.stratified_spectrum(4), lambda_mode=(T.LAMBDA_STRATIFIED, 4, 400.0, 700.0),
                        material=S.CAUCHY_GLASS, map_w=64, map_h=48, accum="i32", hitter="bvh", seed=40 + i)
        out.append((tracer.Scene(wl.tris, wl.first_diffuse, bvh=True), wl))
    return out


def test_crossover_sweep_runs_and_caches(torch_cuda):
    from splat_gb300 import autotune as A

    r = A.batch_crossover(sizes=(32, 512), n_rays=1 << 12, reps=1)
    assert [row["n_tris"] for row in r["rows"]] == [32, 512]
    assert all(row["ms"]["brute"] > 0 and row["ms"]["bvh"] > 0 for row in r["rows"])
    assert r["crossover_tris"] in (32, 512, 513)
    assert A.batch_crossover(sizes=(32, 512), n_rays=1 << 12, reps=1) == r  # from the cache


def test_tuned_hitters_and_batch_knobs_keep_every_map(torch_cuda, restore_knobs):
    from splat_gb300 import autotune as A
    from splat_gb300 import batch, tracer

    fr = _frames()
    scenes = [sc for sc, _ in fr]
    wls = [wl for _, wl in fr]
    cross = sorted(w.n_tris for w in wls)[2]  # the two smallest frames by brute force
    maps = [tracer.new_light_map(w.map_w, w.map_h, w.n_planes, w.accum) for w in wls]
    lanes = batch.Lanes(2, wls, scenes, maps, crossover_tris=cross)
    assert lanes.hitters == ["brute", "brute", "bvh", "bvh"]
    seeds = [w.seed for w in wls]
    tuned = A.tune_batch(lanes, seeds, reps=1, use_cache=False)
    from splat_gb300 import _lib as L

    assert set(tuned["knobs"]) == {str(k) for k in A.BATCH_KNOB_CHOICES} | {str(L.TUNE_BATCH_PERSISTENT)}
    lanes.replay(seeds)
    for (sc, wl), m in zip(fr, maps):
        alone = tracer.trace_forward(wl, scene=sc).tex
        assert torch_cuda.equal(m, alone), wl.name


def test_tuned_step_knobs_keep_the_map(torch_cuda, restore_knobs):
    from splat_gb300 import autotune as A
    from splat_gb300 import tracer

    sc, wl = _frames()[3]
    ref = tracer.trace_forward(wl, scene=sc).tex.clone()
    step = tracer.TraceStep(wl, sc)
    r = A.tune_knobs(step, reps=1, use_cache=False)
    assert set(r["knobs"]) == {str(k) for k in A.KNOB_CHOICES}
    assert torch_cuda.equal(tracer.trace_forward(wl, scene=sc).tex, ref)


def test_server_with_crossover_equals_alone(torch_cuda):
    from splat_gb300 import serve, tracer

    scenes = {0: S.assemble(S.sphere_tris(1, noise_amp=0.05), S.floor_tris(-1.5, 4.0)),
              1: S.assemble(S.sphere_tris(4, noise_amp=0.05), S.floor_tris(-1.5, 4.0))}
    pool = serve.ScenePool(lambda sid: scenes[sid], 4 << 30)
    srv = serve.Server(pool, 4 << 30, max_items=8, max_pool_rays=1 << 18, crossover_tris=1000)
    for rid in range(8):
        sid = rid % 2
        tris, fd = scenes[sid]
        wl = S.Workload(name=f"q{rid}", tris=tris, first_diffuse=fd, light=S.hemisphere_light(rid, 72, 1.1),
                        depth=3, spectrum=S.stratified_spectrum(2), lambda_mode=(T.LAMBDA_STRATIFIED, 2, 400.0, 700.0),
                        material=S.CAUCHY_GLASS, map_w=40, map_h=40, accum="i32", hitter="bvh", seed=900 + rid)
        srv.submit(serve.Request(arrival=0.001 * rid, rid=rid, scene_id=sid, wl=wl))
    srv.drain()
    assert srv.hitter_counts == {"brute": 4, "bvh": 4}
    for r in srv.done:
        alone = tracer.trace_forward(r.wl.with_(hitter="bvh"), scene=pool.resident[r.scene_id]).tex
        assert torch_cuda.equal(r.tex, alone), r.rid
