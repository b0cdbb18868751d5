"""Shared test inputs and comparisons."""
from __future__ import annotations

import json
import os

import numpy as np

from splat_gb300 import scenes as S
from splat_gb300 import types as T

FLOAT_FIELDS = ["pos", "dp_dl", "dp_dx", "dp_dy", "dir", "dd_dl", "dd_dx", "dd_dy", "lam", "x", "y"]


def small_scene(subdiv: int = 2, noise: float = 0.0):
    return S.assemble(S.sphere_tris(subdiv, noise_amp=noise), S.floor_tris(-1.5, 4.0))


def random_rays(n: int, seed: int, n_tris: int, aim: float = 0.7) -> np.ndarray:
    """Rays around a unit sphere: a fraction aimed at it, the rest random;
    random ignore_tri values (some real triangle indices)."""
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, dtype=T.ADRAY)
    o = rng.normal(size=(n, 3))
    o = 3.0 * o / np.linalg.norm(o, axis=1, keepdims=True)
    d = rng.normal(size=(n, 3))
    aimed = rng.uniform(size=n) < aim
    tgt = rng.uniform(-0.8, 0.8, size=(n, 3))
    d[aimed] = tgt[aimed] - o[aimed]
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["pos"] = o.astype(np.float32)
    rays["dir"] = d.astype(np.float32)
    rays["dp_dx"] = rng.normal(scale=0.01, size=(n, 3)).astype(np.float32)
    rays["dp_dy"] = rng.normal(scale=0.01, size=(n, 3)).astype(np.float32)
    rays["lam"] = rng.uniform(400, 700, size=n).astype(np.float32)
    rays["x"] = rng.uniform(1, 64, size=n).astype(np.float32)
    rays["y"] = rng.uniform(1, 64, size=n).astype(np.float32)
    rays["ignore_tri"] = np.where(rng.uniform(size=n) < 0.3, rng.integers(1, n_tris + 1, size=n), 1)
    rays["status"] = T.STATUS_ACTIVE
    return rays


def float_equal(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Elementwise numeric equality with NaN == NaN (signed zeros equal)."""
    return (a == b) | (np.isnan(a) & np.isnan(b))


def assert_rays_equal(got: np.ndarray, ref: np.ndarray, what: str = "rays"):
    assert got.shape == ref.shape
    for f in ["status", "ignore_tri", "in_medium", "dest"]:
        bad = got[f] != ref[f]
        assert not bad.any(), f"{what}: field {f} differs at {np.nonzero(bad)[0][:10]}"
    for f in FLOAT_FIELDS:
        eq = float_equal(got[f], ref[f])
        if eq.ndim > 1:
            eq = eq.all(axis=1)
        assert eq.all(), (f"{what}: field {f} differs at {np.nonzero(~eq)[0][:10]}: "
                          f"{got[f][~eq][:3]} vs {ref[f][~eq][:3]}")


def rel_l1(a: np.ndarray, b: np.ndarray) -> float:
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


# The reference's own test vectors (tests/golden/make_golden.py).
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_tests.json"), encoding="utf-8"))


def optics_scenario():
    """The test/optics.jl ray and triangle as ADRay / FTri records."""
    g = GOLDEN["optics_evolve"]
    r = g["ray"]
    rays = T.empty_rays(1)
    rays["pos"][0], rays["dir"][0] = r["pos"], r["dir"]
    rays["dp_dl"][0], rays["dd_dl"][0] = r["dp_dl"], r["dd_dl"]
    rays["in_medium"][0] = 1 if r["in_medium"] else 0
    rays["ignore_tri"][0], rays["dest"][0], rays["lam"][0] = r["ignore_tri"], r["dest"], r["lam"]
    rays["status"][0] = {"ACTIVE": T.STATUS_ACTIVE, "DIFFUSE": T.STATUS_DIFFUSE, "INFINITY": T.STATUS_INFINITY}[r["status"]]
    a, b, c = (np.asarray(g["tri_vertices"][k], np.float32) for k in ("a", "b", "c"))
    n = np.cross(a - b, b - c).astype(np.float32)
    n = (n * np.float32(1.0 / np.sqrt(np.float32(np.dot(n, n))))).astype(np.float32)
    tri = np.zeros((1, 10, 3), np.float32)
    tri[0, 0], tri[0, 1], tri[0, 2], tri[0, 3] = n, a, b, c
    tri[0, 4] = tri[0, 5] = tri[0, 6] = n
    hit = np.array([g["hit_index"]], np.int32)
    rndm = np.array([g["rndm"]], np.float32)
    return rays, tri, hit, rndm, g["first_diffuse"], (T.MATERIAL_LINEAR_REF, 0.0, 0.0)
