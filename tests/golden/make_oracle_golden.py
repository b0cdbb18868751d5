"""Writes oracle_trace.json: the oracle's forward trace step on fixed cases
of the three workloads, reduced to what a parity check needs -- rays per
bounce, diffuse rays, splat samples and a SHA-256 of the int32 light map
(column-major [w, h, planes], little-endian).  The GPU tests compare the
CUDA path with these committed values without running the oracle; a CPU
test re-runs the oracle on the cheap cases and compares, so a change in
the restatement shows.

Usage: python tests/golden/make_oracle_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "oracle_trace.json")

# name, workload constructor, keyword overrides, light grid scaled to this
# side (0: as built), ray range [begin, end) (end 0: all rays); cheap cases
# are re-run by the CPU tests
CASES = [
    {"name": "plain_small_96_brute", "make": "plain_small", "light_side": 96, "kw": {"accum": "i32", "hitter": "brute"},
     "begin": 0, "end": 0, "cheap": True},
    {"name": "plain_small_64_linear_force1", "make": "plain_small", "light_side": 64,
     "kw": {"accum": "i32", "force_rand": 1.0, "material": [0, 0.0, 0.0]}, "begin": 0, "end": 0, "cheap": True},
    {"name": "plain_small_64_noquirks", "make": "plain_small", "light_side": 64,
     "kw": {"accum": "i32", "quirks": False, "material": [0, 0.0, 0.0]}, "begin": 0, "end": 0, "cheap": True},
    {"name": "plain_small_full", "make": "plain_small", "light_side": 0, "kw": {"accum": "i32"}, "begin": 0, "end": 0,
     "cheap": False},
    {"name": "realtime_mid_1200", "make": "realtime", "light_side": 0, "kw": {}, "begin": "mid", "end": 1200,
     "cheap": True},
    {"name": "realtime_third_1200", "make": "realtime", "light_side": 0, "kw": {}, "begin": "third", "end": 1200,
     "cheap": True},
    {"name": "menger_mid_1200", "make": "menger", "light_side": 0, "kw": {}, "begin": "mid", "end": 1200,
     "cheap": True},
    {"name": "menger_third_1200", "make": "menger", "light_side": 0, "kw": {}, "begin": "third", "end": 1200,
     "cheap": True},
]


_BASE = {}


def _base(make: str):
    """The workload as its constructor builds it (geometry built once)."""
    if make not in _BASE:
        if ROOT not in sys.path:
            sys.path.insert(0, ROOT)
        from splat_gb300 import scenes as S

        _BASE[make] = getattr(S, make)()
    return _BASE[make]


def workload(case):
    """(workload, ray_begin, ray_end) of a case; ray_end 0 means all rays."""
    from splat_gb300 import scenes as S

    base = _base(case["make"])
    kw = dict(case["kw"])
    if "material" in kw:
        kw["material"] = tuple(kw["material"])
    if case["light_side"]:
        kw["light"] = S.scaled_light(base.light, case["light_side"])
    wl = base.with_(**kw) if kw else base
    begin, count = case["begin"], case["end"]
    if begin == 0 and count == 0:
        return wl, 0, 0
    n = wl.n_rays
    h = int(wl.light["res1"]) // wl.upscale
    c = n // 2 + h // 2 - 600 if begin == "mid" else n // 3 + h // 3
    return wl, c, c + count


def digest(tex_column_major) -> str:
    import numpy as np

    return hashlib.sha256(np.ascontiguousarray(tex_column_major, dtype="<i4").tobytes()).hexdigest()


def run_oracle(case) -> dict:
    from oracle import oracle as O

    wl, b, e = workload(case)
    tex, st, _ = O.trace_forward(wl, b, e if e else None)
    flat = tex.ravel(order="F")
    return {"rays_per_bounce": [int(x) for x in st[: wl.depth]], "diffuse": int(st[6]), "samples": int(st[7]),
            "map_sha256": digest(flat), "map_sum": int(flat.astype("int64").sum()),
            "nonzero_texels": int((flat != 0).sum())}


def main() -> None:
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from oracle import oracle as O

    O.build()
    out = {"note": "oracle forward trace step; int32 maps (scale 2^16), column-major, little-endian", "cases": []}
    for case in CASES:
        out["cases"].append({**case, "expect": run_oracle(case)})
        print(case["name"], out["cases"][-1]["expect"]["rays_per_bounce"], flush=True)
    with open(OUT, "w", encoding="utf-8") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
