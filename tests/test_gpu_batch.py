"""Batch engine (splat_batch_*): frames of different scenes, ray counts,
depths, spectra, map sizes and hitters traced together must each give the
frame splat_trace_forward gives alone -- bit-exact for int32 maps, within
1e-5 relative L1 for float maps (float atomics add in another order) --
whether they start together, join while others are in flight, or run as a
replayed CUDA graph with new seeds."""
import numpy as np
import pytest

from helpers import rel_l1
from splat_gb300 import scenes as S
from splat_gb300 import types as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def frames(torch_cuda):
    """(scene, workload) pairs of very different shapes."""
    from splat_gb300 import tracer

    out = []
    tris, fd = S.assemble(S.sphere_tris(2), S.floor_tris(-1.5, 4.0))
    small = S.Workload(name="s", tris=tris, first_diffuse=fd, light=S.hemisphere_light(3, 80, 1.05), depth=3,
                       material=S.CAUCHY_GLASS, map_w=48, map_h=40, accum="i32", spectrum=S.stratified_spectrum(3),
                       lambda_mode=(T.LAMBDA_UNIFORM, 1, 400.0, 700.0), hitter="brute", seed=11)
    out.append((tracer.Scene(small.tris, small.first_diffuse, bvh=True), small))
    out.append((out[0][0], small.with_(hitter="bvh", depth=2, seed=12, quirks=False, map_w=64)))
    rt = S.realtime(light=S.scaled_light(S.realtime().light, 384))
    out.append((tracer.Scene(rt.tris, rt.first_diffuse, bvh=True), rt))
    mg = S.menger(light=S.scaled_light(S.menger().light, 160))
    out.append((tracer.Scene(mg.tris, mg.first_diffuse, bvh=True), mg))
    ps = S.plain_small(light=S.scaled_light(S.plain_small().light, 120))
    out.append((tracer.Scene(ps.tris, ps.first_diffuse, bvh=True), ps))  # float map, own wavelength
    sell = (T.MATERIAL_SELLMEIER, 0.0, 0.0, (1.03961212, 0.231792344, 1.01046945),
            (0.00600069867, 0.0200179144, 103.560653))
    out.append((out[2][0], rt.with_(material=sell, depth=5, seed=99, light=S.scaled_light(rt.light, 200))))
    return out


def _alone(scene, wl, seed=None):
    from splat_gb300 import tracer

    w = wl if seed is None else wl.with_(seed=seed)
    return tracer.trace_forward(w, scene=scene).tex.cpu().numpy()


def _check(wl, got, ref, what):
    if wl.accum == "i32":
        bad = np.count_nonzero(got != ref)
        assert bad == 0, f"{what}: {bad} texels differ"
    else:
        assert rel_l1(got, ref) <= 1e-5, what
    assert ref.sum() > 0, what


@pytest.fixture()
def knobs(torch_cuda):
    """Sets tuning knobs for one test and puts the old values back."""
    from splat_gb300 import _lib as L

    lib = L.load()
    saved = {}

    def set_(key, value):
        if key not in saved:
            saved[key] = lib.splat_get_tuning(key)
        L.check(lib.splat_set_tuning(key, value))

    yield set_
    for key, value in saved.items():
        L.check(lib.splat_set_tuning(key, value))


# the batch hit kernel's traversal forms (SPLAT_TUNE_BVH_PACKET): the default
# (packets on first-bounce warps of one item), none, every warp of one item,
# and per warp by ray spread; with and without the rays of every tick
# grouped by (item, BVH position of the triangle left, octant) first
@pytest.mark.parametrize("packet,order", [(None, 0), (0, 0), (2, 0), (5, 0), (0, 20), (2, 20), (5, 20)])
def test_batch_equals_single_frames(frames, knobs, packet, order):
    from splat_gb300 import _lib as L
    from splat_gb300 import batch, tracer

    b = batch.Batch(16, 1 << 21)
    texs = []
    for sc, wl in frames:
        tex = tracer.new_light_map(wl.map_w, wl.map_h, wl.n_planes, wl.accum)
        b.admit(sc, wl, tex)
        texs.append(tex)
    if packet is not None:
        knobs(L.TUNE_BVH_PACKET, packet)
    knobs(L.TUNE_RAY_ORDER, order)
    done = b.run()
    assert sorted(done) == list(range(len(frames)))
    for i, ((sc, wl), tex) in enumerate(zip(frames, texs)):
        _check(wl, tex.cpu().numpy(), _alone(sc, wl), f"frame {i}")
    for s in done:
        b.release(s)
    assert b.status()["in_flight"] == 0


@pytest.mark.parametrize("order", [0, 20])
def test_frames_joining_while_others_run(frames, knobs, order):
    """Continuous batching: frames admitted at different ticks overlap on the
    device and each still equals its alone result (with the ray order, the
    items' key ranges are reassigned at every admission while rays are in
    flight)."""
    from splat_gb300 import _lib as L
    from splat_gb300 import batch, tracer

    knobs(L.TUNE_RAY_ORDER, order)
    knobs(L.TUNE_BVH_PACKET, 5 if order else 1)
    b = batch.Batch(8, 1 << 21)
    plan = {0: [3, 0], 1: [2], 2: [1, 5], 4: [4]}
    texs, done = {}, []
    tick = 0
    while tick <= 4 or b.status()["in_flight"] > 0:
        for i in plan.get(tick, []):
            sc, wl = frames[i]
            texs[i] = (b.admit(sc, wl, tracer.new_light_map(wl.map_w, wl.map_h, wl.n_planes, wl.accum)), i)
            texs[i] = (texs[i][0], b.items[texs[i][0]][2])
        assert b.status()["in_flight"] > 0 or tick > 4
        done += b.tick()
        tick += 1
    assert len(done) == 6
    for i, (slot, tex) in texs.items():
        sc, wl = frames[i]
        _check(wl, tex.cpu().numpy(), _alone(sc, wl), f"frame {i} joined late")


@pytest.mark.parametrize("order", [0, 20])
def test_graph_capture_and_replay_with_new_seeds(frames, knobs, order):
    from splat_gb300 import _lib as L
    from splat_gb300 import batch, tracer

    knobs(L.TUNE_RAY_ORDER, order)
    b = batch.Batch(8, 1 << 21)
    sel = [0, 2, 3]
    texs = []
    for i in sel:
        sc, wl = frames[i]
        tex = tracer.new_light_map(wl.map_w, wl.map_h, wl.n_planes, wl.accum)
        b.admit(sc, wl, tex)
        texs.append(tex)
    n_ticks = b.capture()
    assert n_ticks == max(frames[i][1].depth for i in sel)
    for seeds in ([101, 202, 303], [7, 8, 9]):
        b.replay(seeds)
        for s, i in enumerate(sel):
            sc, wl = frames[i]
            _check(wl, texs[s].cpu().numpy(), _alone(sc, wl, seeds[s]), f"replay frame {i} seed {seeds[s]}")


def test_admission_respects_the_pool(frames):
    from splat_gb300 import batch, tracer

    sc, wl = frames[2]  # 192^2 = 36,864 rays
    b = batch.Batch(4, 50000)
    t1 = tracer.new_light_map(wl.map_w, wl.map_h, wl.n_planes, wl.accum)
    s1 = b.admit(sc, wl, t1)
    with pytest.raises(batch.PoolFull):
        b.admit(sc, wl, tracer.new_light_map(wl.map_w, wl.map_h, wl.n_planes, wl.accum))
    assert b.run() == [s1]
    b.release(s1)
    t2 = tracer.new_light_map(wl.map_w, wl.map_h, wl.n_planes, wl.accum)
    b.admit(sc, wl.with_(seed=5), t2)
    b.run()
    _check(wl, t1.cpu().numpy(), _alone(sc, wl), "first")
    _check(wl, t2.cpu().numpy(), _alone(sc, wl, 5), "second")


def test_lanes_replay_concurrently_and_equal_alone(frames):
    """Frames dealt to two engines whose graphs replay concurrently on two
    streams: every map equals the frame's alone result, pass after pass."""
    from splat_gb300 import batch, tracer

    scenes = [sc for sc, _ in frames]
    wls = [wl for _, wl in frames]
    maps = [tracer.new_light_map(w.map_w, w.map_h, w.n_planes, w.accum) for w in wls]
    lanes = batch.Lanes(2, wls, scenes, maps)
    assert sorted(i for m in lanes.members for i in m) == list(range(len(wls)))
    lanes.capture()
    for k in range(2):
        seeds = [w.seed + 7 * k for w in wls]
        lanes.replay(seeds)
        for i, (sc, wl) in enumerate(frames):
            _check(wl, maps[i].cpu().numpy(), _alone(sc, wl, seeds[i]), f"frame {i} pass {k}")


@pytest.mark.parametrize("n_lanes", [1, 2])
def test_persistent_pass_equals_alone(frames, n_lanes):
    """The captured pass as one persistent cooperative launch per engine
    (SPLAT_TUNE_BATCH_PERSISTENT; grid-wide waits between reserve, generate,
    traversal + the previous tick's splat, evolve): every map equals the
    frame's alone result, pass after pass, and re-capturing tick by tick
    gives the same maps again."""
    from splat_gb300 import batch, tracer

    scenes = [sc for sc, _ in frames]
    wls = [wl for _, wl in frames]
    maps = [tracer.new_light_map(w.map_w, w.map_h, w.n_planes, w.accum) for w in wls]
    lanes = batch.Lanes(n_lanes, wls, scenes, maps)
    n_ticks = lanes.persistent(True)
    assert n_ticks == max(w.depth for w in wls)
    for k in range(2):
        seeds = [w.seed + 11 * k for w in wls]
        lanes.replay(seeds)
        for i, (sc, wl) in enumerate(frames):
            _check(wl, maps[i].cpu().numpy(), _alone(sc, wl, seeds[i]), f"frame {i} pass {k}")
    lanes.persistent(False)
    lanes.replay([w.seed for w in wls])
    for i, (sc, wl) in enumerate(frames):
        _check(wl, maps[i].cpu().numpy(), _alone(sc, wl), f"frame {i} tick by tick")
