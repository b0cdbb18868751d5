"""Mesh ingest (splat_obj_to_ftri, mesh_to_FTri src/geo.jl:289-341) on the
host: OBJ round trips, fan triangulation, index forms, errors."""
import os

import numpy as np
import pytest

from splat_gb300 import _lib as L
from splat_gb300 import scenes as S


def test_obj_round_trip_is_bit_exact(tmp_path):
    tris = S.sphere_tris(3, noise_amp=0.05)
    P, N, UV = tris[:, 1:4], tris[:, 4:7], tris[:, 7:10]
    p = str(tmp_path / "sphere.obj")
    S.write_obj(p, P, N, UV)
    got = S.load_obj(p)
    want = S.ftri_records(P, N, UV)
    assert got.shape == want.shape == (1280, 10, 3)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_fan_triangulation_and_index_forms(tmp_path):
    p = str(tmp_path / "poly.obj")
    open(p, "w").write(
        "# quad, pentagon with negative indices, v//n, bare v\n"
        "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 0.5 1.5 0\n"
        "vt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n"
        "vn 0 0 1\n"
        "f 1/1/1 2/2/1 3/3/1 4/4/1\n"
        "f -5//-1 -4//-1 -3//-1 -1//-1 -2//-1\n"
        "f 1 2 3\n")
    t = S.load_obj(p)
    assert t.shape == (2 + 3 + 1, 10, 3)
    # quad a b c d -> (a, b, c), (a, c, d)
    np.testing.assert_array_equal(t[0, 1:4], [[0, 0, 0], [1, 0, 0], [1, 1, 0]])
    np.testing.assert_array_equal(t[1, 1:4], [[0, 0, 0], [1, 1, 0], [0, 1, 0]])
    np.testing.assert_array_equal(t[1, 7:10], [[0, 0, 0], [1, 1, 0], [0, 1, 0]])
    # plane normal cross(v1 - v2, v2 - v3)
    np.testing.assert_array_equal(t[0, 0], np.cross(t[0, 1] - t[0, 2], t[0, 2] - t[0, 3]))
    # pentagon: fan from the first corner, negative indices from the end
    np.testing.assert_array_equal(t[2, 1:4], [[0, 0, 0], [1, 0, 0], [1, 1, 0]])
    np.testing.assert_array_equal(t[4, 1:4], [[0, 0, 0], [0.5, 1.5, 0], [0, 1, 0]])
    assert (t[2:5, 7:10] == 0).all()
    # no normals: the unit face normal at every corner
    np.testing.assert_allclose(t[5, 4:7], [[0, 0, 1]] * 3)


@pytest.mark.parametrize("body,what", [("v 0 0 0\nf 1 2 3\n", "bad face index"),
                                        ("v 0 0\n", "bad vertex"), ("v 0 0 0\nv 1 0 0\nf 1 2\n", "degenerate")])
def test_malformed_files_fail_cleanly(tmp_path, body, what):
    p = str(tmp_path / "bad.obj")
    open(p, "w").write(body)
    with pytest.raises(L.SplatError, match=what):
        S.load_obj(p)
    with pytest.raises(L.SplatError, match="cannot open"):
        S.load_obj(str(tmp_path / "missing.obj"))


# the reference checkout, when the environment names one (REFERENCE_ROOT)
REF_ICOS = os.path.join(os.environ.get("REFERENCE_ROOT", ""), "objs", "icos.obj")


@pytest.mark.skipif(not os.environ.get("REFERENCE_ROOT") or not os.path.exists(REF_ICOS),
                    reason="REFERENCE_ROOT unset or without objs/icos.obj")
def test_reference_icosphere_asset_loads():
    """The reference's own smoke-test asset (objs/icos.obj, subdivision-3
    icosphere): 1280 triangles, unit vertex normals, outward plane normals."""
    t = S.load_obj(REF_ICOS)
    assert t.shape == (1280, 10, 3)
    np.testing.assert_allclose(np.linalg.norm(t[:, 4:7], axis=2), 1.0, atol=1e-4)
    centroid = t[:, 1:4].mean(axis=1)
    assert (np.einsum("ij,ij->i", t[:, 0], centroid) != 0).all()
    tris, fd = S.assemble_meshes([t, S.translate(t, (0, 2, 0))], [S.translate(t, (1, 0, -4))])
    assert tris.shape[0] == 1 + 3 * 1280 and fd == 2 + 2 * 1280
