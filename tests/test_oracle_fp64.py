"""The oracle's binary32 results against binary64 re-evaluations (CPU only;
the GPU path equals the oracle bit for bit, see the gpu tests):

- hit distance: the binary32 t of the chosen triangle against the same
  distance_to_plane (src/geo.jl:433-443) evaluated in binary64, and the
  chosen triangle against a binary64 nearest-hit search;
- ray-differential Jacobians: the forward-mode partials that evolve_ray
  (src/tracer.jl:118-179) writes, with the reference's derivative quirks
  switched off, against central finite differences of a binary64 primal of
  the same bounce (distance_to_plane, next_p, optical_normal
  src/geo.jl:202-258, refract / reflect src/geo.jl:481-561, glass
  src/material.jl:1-13) over the expanded ray family.

The binary64 restatements here are independent of the oracle's code: plain
numpy, written from the reference's formulas."""
import numpy as np
import pytest

from helpers import random_rays, small_scene
from oracle import oracle as O
from splat_gb300 import scenes as S
from splat_gb300 import types as T

SELLMEIER = (T.MATERIAL_SELLMEIER, 0.0, 0.0, (1.03961212, 0.231792344, 1.01046945),
             (0.00600069867, 0.0200179144, 103.560653))


def _nrm(v):
    return v / np.linalg.norm(v)


def _glass(mat, lam):
    if mat[0] == T.MATERIAL_CAUCHY:
        lu = lam * 1e-3
        return mat[1] + mat[2] / (lu * lu)
    if mat[0] == T.MATERIAL_SELLMEIER:
        l2 = (lam * 1e-3) ** 2
        return np.sqrt(1.0 + sum(mat[3][i] * l2 / (l2 - mat[4][i]) for i in range(3)))
    return (1.4 - 1.3) / (700.0 - 400.0) * (lam - 400.0) + 1.3


def _refract(v, n, n1, n2):
    n = _nrm(n)
    if v @ n > 0:
        n = -n
    c1 = _nrm(v) @ n
    s2 = n1 / n2 * np.sqrt(1.0 - c1 * c1)
    return _nrm(v * (n1 / n2) + n * ((n1 / n2) * c1 - np.sqrt(1.0 - s2 * s2)))


def _reflect(v, n):
    n = _nrm(n)
    return v - 2.0 * (n @ v) * n


def _bounce64(R, tri, mat, refracts, lam, x, y):
    """Position on the hit and new direction of the ray family member at
    (lam, x, y), in binary64."""
    f = lambda k: R[k].astype(np.float64)
    dl, dx, dy = lam - float(R["lam"]), x - float(R["x"]), y - float(R["y"])
    o = f("pos") + f("dp_dl") * dl + f("dp_dx") * dx + f("dp_dy") * dy
    d = f("dir") + f("dd_dl") * dl + f("dd_dx") * dx + f("dd_dy") * dy
    nt, a, b, c, na, nb, nc = (tri[i].astype(np.float64) for i in range(7))
    p = o + d * ((nt @ a - nt @ o) / (nt @ d))
    N = np.cross(b - a, c - a)
    u = N @ np.cross(c - b, p - b) / (N @ N)
    v = N @ np.cross(a - c, p - c) / (N @ N)
    nn = _nrm(na * u + nb * v + nc * (1.0 - u - v))
    n1, n2 = (_glass(mat, lam), 1.0) if R["in_medium"] else (1.0, _glass(mat, lam))
    return p, (_refract(d, nn, n1, n2) if refracts else _reflect(d, nn))


def _t64(ray, tri):
    o, d = ray["pos"].astype(np.float64), ray["dir"].astype(np.float64)
    n, a = tri[0].astype(np.float64), tri[1].astype(np.float64)
    return (n @ a - n @ o) / (n @ d)


def test_hit_distance_against_binary64():
    tris, _ = small_scene(3, 0.05)
    rays = random_rays(3000, 41, tris.shape[0])
    hit, t32 = O.next_hit(rays, tris)
    sel = np.nonzero(hit > 1)[0]
    assert sel.size > 1000
    rel = np.array([abs(float(t32[k]) - _t64(rays[k], tris[hit[k] - 1])) / abs(_t64(rays[k], tris[hit[k] - 1]))
                    for k in sel])
    # binary32 distance_to_plane: a few ulps, more where n.o nearly cancels n.v1
    assert np.median(rel) < 1e-6 and np.percentile(rel, 99) < 1e-4, (np.median(rel), np.percentile(rel, 99))
    # the binary64 nearest hit over all triangles picks the same triangle for
    # all but near-ties (two candidates within 1e-5 relative of each other)
    o = rays["pos"][sel].astype(np.float64)
    d = rays["dir"][sel].astype(np.float64)
    nt, a, b, c = (tris[1:, i].astype(np.float64) for i in range(4))
    t = ((nt * a).sum(1)[None, :] - o @ nt.T) / (d @ nt.T)
    p = o[:, None, :] + d[:, None, :] * t[:, :, None]
    v0, v1, v2 = c - a, b - a, p - a[None]
    d00, d01, d11 = (v0 * v0).sum(1), (v0 * v1).sum(1), (v1 * v1).sum(1)
    d02, d12 = (v2 * v0[None]).sum(2), (v2 * v1[None]).sum(2)
    inv = 1.0 / (d00 * d11 - d01 * d01)
    uu, vv = (d11 * d02 - d01 * d12) * inv, (d00 * d12 - d01 * d02) * inv
    ok = (uu >= 0) & (vv >= 0) & (uu + vv < 1) & (t > 0)
    ok &= np.arange(1, tris.shape[0])[None, :] + 1 != rays["ignore_tri"][sel][:, None]
    t = np.where(ok, t, np.inf)
    best = t.argmin(1) + 2
    same = best == hit[sel]
    for k in np.nonzero(~same)[0]:
        t1, t2 = t[k, hit[sel][k] - 2], t[k, best[k] - 2]
        assert abs(t1 - t2) <= 1e-5 * abs(t2) or not np.isfinite(t1), (k, t1, t2)
    assert same.mean() > 0.99


@pytest.mark.parametrize("mat", [S.CAUCHY_GLASS, SELLMEIER], ids=["cauchy", "sellmeier"])
@pytest.mark.parametrize("force", [0.0, 1.0], ids=["reflect", "refract"])
def test_jacobians_against_finite_differences(mat, force):
    tris, fd = small_scene(3, 0.05)
    cur = O.rays_from_light(S.hemisphere_light(1, 48, 1.05), 1, (T.LAMBDA_UNIFORM, 1, 400.0, 700.0), seed=5)
    checked = 0
    for bounce in (1, 2):
        hit, _ = O.next_hit(cur, tris)
        out = O.evolve(cur, hit, tris, np.full(len(cur), force, np.float32), fd, mat, quirks=False)
        sel = np.nonzero((out["status"] == T.STATUS_ACTIVE) & (cur["status"] == T.STATUS_ACTIVE))[0]
        errs = []
        for k in sel[:150]:
            R, tri = cur[k], tris[hit[k] - 1]
            refracts = out["in_medium"][k] != cur["in_medium"][k]
            base = [float(R["lam"]), float(R["x"]), float(R["y"])]
            for i, h, pk, dk in ((0, 1e-3, "dp_dl", "dd_dl"), (1, 1e-4, "dp_dx", "dd_dx"), (2, 1e-4, "dp_dy", "dd_dy")):
                up, dn = list(base), list(base)
                up[i] += h
                dn[i] -= h
                (p1, d1), (p0, d0) = _bounce64(R, tri, mat, refracts, *up), _bounce64(R, tri, mat, refracts, *dn)
                fdp, fdd = (p1 - p0) / (2 * h), (d1 - d0) / (2 * h)
                errs.append(np.linalg.norm(out[pk][k] - fdp) / max(np.linalg.norm(fdp), 1e-6))
                errs.append(np.linalg.norm(out[dk][k] - fdd) / max(np.linalg.norm(fdd), 1e-6))
        if errs:
            e = np.array(errs)
            assert np.median(e) < 1e-5 and np.percentile(e, 99) < 1e-2, (bounce, np.median(e), e.max())
            checked += len(errs)
        cur = out
    assert checked > 600
