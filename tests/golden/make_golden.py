"""Writes reference_tests.json: the inputs and expected values of the
reference's own unit tests, read as text from its test files.

  test/geo.jl:10-15   reflect axis cases      reflect(v, n) ≈ want
  test/geo.jl:18-22   reflect regression      ‖reflect(d0, n) - d1‖ < 1e-6
  test/geo.jl:24-29   distance_to_plane sign symmetries (o, d, p, n)
  test/optics.jl:1-18 evolve_ray(adr, 1, t, 1.0f0, 2) on one ray and one
                      triangle (the file asserts nothing; the scenario is
                      kept so the restatement and the kernels run it)

The test files use the stale constructor names V3 (now R3) and a 9-field
ADRay (pos, dpos/dλ, dir, ddir/dλ, in_medium, ignore_tri, dest, λ, status);
the fixture records the values, not the constructors.

Usage: python tests/golden/make_golden.py [reference root]
(the reference checkout: the argument, else the REFERENCE_ROOT environment
variable; one of them is required).
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "reference_tests.json")

NUM = r"-?\d+(?:\.\d+)?(?:[eE]-?\d+)?(?:f0)?"
V3 = rf"V3\(\s*({NUM})\s*,\s*({NUM})\s*,\s*({NUM})\s*\)"


def _num(s: str) -> float:
    return float(s[:-2] if s.endswith("f0") else s)


def _vec(groups) -> list:
    return [_num(g) for g in groups]


def parse_geo(text: str) -> dict:
    reflect = []
    for m in re.finditer(rf"@test reflect\({V3},\s*{V3}\)\s*≈\s*{V3}", text):
        g = m.groups()
        reflect.append({"v": _vec(g[0:3]), "n": _vec(g[3:6]), "want": _vec(g[6:9])})
    assigns = {}
    for m in re.finditer(rf"^(\w+)\s*=\s*{V3}", text, re.M):
        assigns[m.group(1)] = _vec(m.groups()[1:4])
    tol = re.search(r"@test norm\(reflect\(d0, n\) - d1\) < (\S+)", text)
    regression = {"d0": assigns["d0"], "n": assigns["n"], "d1": assigns["d1"], "tol": float(tol.group(1))}
    dist = []
    for m in re.finditer(rf"distance_to_plane\({V3},\s*{V3}(\s*\*\s*-1)?,\s*{V3},\s*{V3}(\s*\*\s*-1)?\)", text):
        g = m.groups()
        d = _vec(g[3:6])
        n = _vec(g[10:13])
        if g[6]:
            d = [-x for x in d]
        if g[13]:
            n = [-x for x in n]
        dist.append({"o": _vec(g[0:3]), "d": d, "p": _vec(g[7:10]), "n": n})
    # the two @test lines each compare a pair: (0, 1) normal sign, (2, 3) direction sign
    return {"reflect_axis_cases": reflect, "reflect_regression": regression,
            "distance_to_plane": {"normal_sign_pair": dist[0:2], "direction_sign_pair": dist[2:4]}}


def parse_optics(text: str) -> dict:
    m = re.search(rf"adr = ADRay\(\s*{V3},\s*zero\(V3\),\s*{V3},\s*zero\(V3\),\s*(true|false),\s*({NUM}),\s*"
                  rf"({NUM}),\s*({NUM}),\s*RAY_STATUS_(\w+)\)", text)
    g = m.groups()
    ray = {"pos": _vec(g[0:3]), "dp_dl": [0.0, 0.0, 0.0], "dir": _vec(g[3:6]), "dd_dl": [0.0, 0.0, 0.0],
           "in_medium": g[6] == "true", "ignore_tri": int(_num(g[7])), "dest": int(_num(g[8])),
           "lam": _num(g[9]), "status": g[10]}
    verts = {k: _vec(re.search(rf"^{k} = {V3}", text, re.M).groups()) for k in ("a", "b", "c")}
    call = re.search(rf"evolve_ray\(adr, Int32\((\d+)\), t, ({NUM}), (\d+)\)", text)
    return {"ray": ray, "tri_vertices": verts,
            "tri": "FTri(n, a, b, c, n, n, n, 0, 0, 0) with n = normalize(cross(a - b, b - c))",
            "hit_index": int(call.group(1)), "rndm": _num(call.group(2)), "first_diffuse": int(call.group(3))}


def generate(root: str) -> dict:
    with open(os.path.join(root, "test", "geo.jl"), encoding="utf-8") as f:
        geo = parse_geo(f.read())
    with open(os.path.join(root, "test", "optics.jl"), encoding="utf-8") as f:
        optics = parse_optics(f.read())
    return {"source": {"geo": "test/geo.jl", "optics": "test/optics.jl"}, "geo": geo, "optics_evolve": optics}


def main() -> None:
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py <reference root> (or set REFERENCE_ROOT)")
    data = generate(root)
    with open(OUT, "w", encoding="utf-8") as f:
        json.dump(data, f, indent=1)
        f.write("\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
