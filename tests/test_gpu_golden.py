"""The fused trace step (splat_trace_forward) against the committed golden
values of the oracle (tests/golden/oracle_trace.json): rays per bounce,
diffuse rays, splat samples and the SHA-256 of the int32 light map, for
both hitters (their results are identical bit for bit).  No oracle runs
here: the CUDA path is checked against the committed fixture alone."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_oracle_golden as G  # noqa: E402

FIXTURE = json.load(open(os.path.join(HERE, "golden", "oracle_trace.json"), encoding="utf-8"))

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("hitter", ["as_built", "other"])
@pytest.mark.parametrize("case", FIXTURE["cases"], ids=lambda c: c["name"])
def test_trace_matches_golden(case, hitter):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from splat_gb300 import tracer

    wl, b, e = G.workload(case)
    if hitter == "other":
        wl = wl.with_(hitter="brute" if wl.hitter != "brute" else "bvh")
    r = tracer.trace_forward(wl, ray_begin=b, ray_end=e)
    flat = r.tex.cpu().numpy().ravel()
    want = case["expect"]
    assert r.stats["error"] == 0
    assert r.stats["rays_per_bounce"] == want["rays_per_bounce"]
    assert r.stats["diffuse"] == want["diffuse"] and r.stats["samples"] == want["samples"]
    assert int(flat.astype(np.int64).sum()) == want["map_sum"]
    assert int((flat != 0).sum()) == want["nonzero_texels"]
    assert G.digest(flat) == want["map_sha256"]
