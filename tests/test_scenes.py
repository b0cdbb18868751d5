"""Procedural workloads: sizes the benchmarks are quoted on and the
reference's scene conventions (sentinel first, glass then diffuse)."""
import numpy as np

from splat_gb300 import scenes as S
from splat_gb300 import types as T


def test_icosphere_counts():
    for k, (v, f) in {5: (10242, 20480), 6: (40962, 81920)}.items():
        V, F = S.icosphere(k)
        assert V.shape[0] == v and F.shape[0] == f
        np.testing.assert_allclose(np.linalg.norm(V, axis=1), 1.0, rtol=1e-12)


def test_menger_counts():
    assert len(S.menger_cubes(1)) == 20
    assert len(S.menger_cubes(3)) == 8000
    assert S.menger_tris(3).shape == (96000, 10, 3)
    R = S.random_quaternion_matrix(4)
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-12)
    assert abs(np.linalg.det(R) - 1) < 1e-12


def test_workload_conventions():
    for make, n_tris, n_rays in [(S.plain_small, 20483, 1 << 16), (S.realtime, 81923, 1 << 20),
                                 (S.menger, 96013, 1 << 22)]:
        wl = make()
        assert wl.tris.dtype == np.float32 and wl.tris.shape == (n_tris, 10, 3)
        assert not wl.tris[0].any(), "reference index 1 is the zero sentinel"
        assert wl.n_rays == n_rays
        assert 2 <= wl.first_diffuse <= n_tris
        # FTri normal is cross(v1 - v2, v2 - v3) of the stored vertices
        t = wl.tris[1:200].astype(np.float64)
        n = np.cross(t[:, 1] - t[:, 2], t[:, 2] - t[:, 3])
        np.testing.assert_allclose(wl.tris[1:200, 0], n, rtol=1e-5, atol=1e-9)
    wl = S.realtime()
    assert wl.n_planes == 16 and wl.upscale == 2 and wl.accum == "i32" and wl.hitter == "bvh"
    fl = wl.tris[wl.first_diffuse - 1:]
    assert fl.shape[0] == 2 and (fl[:, 7:10, :2] >= 0).all() and (fl[:, 7:10, :2] <= 1).all()


def test_light_is_seeded_and_in_upper_hemisphere():
    a = S.hemisphere_light(1, 256, 1.05)
    b = S.hemisphere_light(1, 256, 1.05)
    assert a.tobytes() == b.tobytes()
    assert a["dir"][1] < 0  # shines down from the upper hemisphere
    assert abs(np.dot(a["dir"], a["dim1"])) < 1e-6 and abs(np.dot(a["dir"], a["dim2"])) < 1e-6


def test_spectrum():
    s = S.stratified_spectrum(16)
    assert s.dtype == np.float32 and len(s) == 16
    assert abs(s[0] - (400 + 300 / 32)) < 1e-4 and abs(s[-1] - (700 - 300 / 32)) < 1e-4
    assert T.upres(2).tolist() == [-0.25, 0.25]


def test_reference_procedural_assets():
    """square / stage / ripples (src/procedural_assets.jl) and the FTri
    transforms (src/geo.jl:132-150)."""
    sq = S.square()
    assert sq.shape == (2, 10, 3) and (sq[:, 0] == [0, 0, 1]).all()
    np.testing.assert_array_equal(sq[1, 1:4], [[1, 0, 0], [0, 1, 0], [1, 1, 0]])
    st = S.stage()
    assert st.shape == (3, 10, 3)
    np.testing.assert_allclose(np.linalg.norm(st[:, 0], axis=1), 1.0, rtol=1e-6)
    r = S.ripples(0.3)
    assert r.shape == (80000, 10, 3) and np.isfinite(r).all()
    # per grid row y: 200 first triangles (x ascending), then 200 second ones
    np.testing.assert_allclose(r[1, 1, :2], [0.005, 0.0], atol=1e-9)
    np.testing.assert_allclose(r[200, 1, :2], [0.005, 0.005], atol=1e-9)
    np.testing.assert_allclose(r[400, 1, :2], [0.0, 0.005], atol=1e-9)
    # plane normals: +z for the first triangles, -z for the second (their
    # winding, as in the reference); vertex normals (df/dx, df/dy, -1)
    first = (np.arange(80000) // 200) % 2 == 0
    assert (r[first, 0, 2] > 0).all() and (r[~first, 0, 2] < 0).all() and (r[:, 4:7, 2] == -1).all()
    assert np.abs(r[:, 1:4, 2]).max() <= 4 * 0.000125 + 1e-9
    assert not np.array_equal(S.ripples(0.0)[:, 1:4, 2], r[:, 1:4, 2])  # the surface moves with t
    w = S.ripples_scene(0.1)
    assert w.n_tris == 80003 and w.first_diffuse == 80002 and w.n_rays == 1 << 20
    s2 = S.scale(sq, 2.0)
    np.testing.assert_array_equal(s2[:, 1:4], sq[:, 1:4] * 2)
    np.testing.assert_array_equal(s2[:, 0], sq[:, 0])
    Rz = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    rot = S.rotate(st, Rz)
    np.testing.assert_allclose(rot[:, 1:4], st[:, 1:4] @ Rz.T, atol=1e-6)
    np.testing.assert_array_equal(rot[:, 7:10], st[:, 7:10])
