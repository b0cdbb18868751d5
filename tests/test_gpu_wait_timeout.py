"""The failure path of the brute-force hitter's bounded mbarrier waits, made
to run out on purpose and on the host's say-so: the test-only knob
SPLAT_TUNE_TEST_WAIT_STALL makes the wait for one tile of every block poll a
barrier that nothing completes, 64 times.  Each block then sets error bit 1,
drains its copies still in flight (their barriers do complete) and returns.
Checked: the call returns, the error word reaches splat_trace_stats_t.error
and the host entry point's SPLAT_ERR_DEVICE, and once the scene's error word
is cleared the next call on the same stream is exact against the oracle.
Nothing here traps, faults or waits without a bound."""
import numpy as np
import pytest

from oracle import oracle as O
from splat_gb300 import _lib as L
from splat_gb300 import scenes as S
from splat_gb300 import types as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _workload():
    tris, fd = S.assemble(S.sphere_tris(3, noise_amp=0.05), S.floor_tris(-1.5, 4.0))
    return S.Workload(name="stalled-wait", tris=tris, first_diffuse=fd, light=S.hemisphere_light(4, 64, 1.05),
                      depth=3, material=S.CAUCHY_GLASS, map_w=64, map_h=48, accum="i32",
                      spectrum=S.stratified_spectrum(4), lambda_mode=(T.LAMBDA_UNIFORM, 1, 400.0, 700.0),
                      hitter="brute", seed=33)


# stall on the first tile (no copy consumed yet) and on the third (copies of
# later tiles in flight, which the drain must wait for)
@pytest.mark.parametrize("stall", [1, 3])
def test_stalled_wait_reports_and_the_stream_recovers(torch_cuda, stall):
    torch = torch_cuda
    from splat_gb300 import tracer

    lib = L.load()
    wl = _workload()
    scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=False)
    step = tracer.TraceStep(wl, scene)
    host_map = np.zeros(step.tex.numel(), dtype=np.int32)
    old = lib.splat_get_tuning(L.TUNE_TEST_WAIT_STALL)
    try:
        L.check(lib.splat_set_tuning(L.TUNE_TEST_WAIT_STALL, stall))
        # device entry point: the statistics carry the error word
        step.run()
        torch.cuda.synchronize()
        assert step.stats()["error"] & 1
        assert scene.errors(reset=True) & 1
        # host entry point: the same word as SPLAT_ERR_DEVICE
        with pytest.raises(L.SplatError) as ei:
            step.run_host(None, host_map)
        assert ei.value.code == L.ERR_DEVICE
        assert "kernel error word" in str(ei.value)
    finally:
        L.check(lib.splat_set_tuning(L.TUNE_TEST_WAIT_STALL, old))
    assert scene.errors(reset=True) & 1
    # the context and the stream are usable: the same step is now exact
    res = tracer.trace_forward(wl, scene=scene)
    assert res.stats["error"] == 0
    ref, ref_st, _ = O.trace_forward(wl)
    assert res.stats["rays_per_bounce"] == [int(x) for x in ref_st[: wl.depth]]
    got = res.tex.cpu().numpy().ravel()
    assert np.array_equal(got, ref.ravel(order="F"))
    step.run_host(None, host_map)
    assert np.array_equal(host_map, ref.ravel(order="F"))
