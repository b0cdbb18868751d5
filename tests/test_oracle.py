"""The CPU oracle pinned against everything the reference itself pins:

* test/geo.jl:4-29 -- reflect axis cases, the regression golden vector
  (||reflect(d0, n) - d1|| < 1e-6) and distance_to_plane's sign symmetries
  (the test file uses the stale name V3 for R3; restated with R3 semantics);
* src/atomic_argmin.jl:32-96 -- test_reversibility, test_comparison and
  test_comparison2 of the order-preserving float -> u32 map;
* the published Philox4x32-10 known-answer vectors (Random123 kat_vectors);
* structural facts of the reference's formulas (upres, glass, generator
  derivatives) and conservation laws of the trace step.
"""
import numpy as np
import pytest

from oracle import oracle as O
from splat_gb300 import scenes as S
from splat_gb300 import types as T

# --------------------------------------------------------------- test/geo.jl


@pytest.mark.parametrize("v,n,want", [
    ((-1, -1, 0), (0, 1, 0), (-1, 1, 0)),
    ((-1, -1, 0), (0, -1, 0), (-1, 1, 0)),
    ((-1, -1, 0), (1, 0, 0), (1, -1, 0)),
    ((-1, -1, 0), (-1, 0, 0), (1, -1, 0)),
    ((-4, -1, 0), (0, 1, 0), (-4, 1, 0)),
    ((-1, -4, 0), (0, 1, 0), (-1, 4, 0)),
])
def test_reflect_axis_cases(v, n, want):
    np.testing.assert_allclose(O.reflect(v, n), np.asarray(want, np.float32), rtol=0, atol=1e-6)


def test_reflect_regression_vector():
    d0 = (-0.0993602, -0.990078, 0.0993602)
    n = (0.21059, 0.310929, -0.926809)
    d1 = np.asarray((0.077896, -0.728365, -0.680746), np.float32)
    assert np.linalg.norm(O.reflect(d0, n) - d1) < 1e-6


def test_distance_to_plane_symmetries():
    a = O.distance_to_plane((1, 2, 4), (2, 3, 1), (-2, 0, -2), (8, 1, 0))
    # the normal's sign does not matter (bit-equal)
    assert a == O.distance_to_plane((1, 2, 4), (2, 3, 1), (-2, 0, -2), (-8, -1, 0))
    # a reversed direction gives the negated distance (bit-equal)
    assert O.distance_to_plane((1, 2, 4), (-2, -3, -1), (-2, 0, -2), (8, 1, 0)) == -a


# ------------------------------------------------------ src/atomic_argmin.jl


def _test_array(rng):
    parts = [rng.random(1000, dtype=np.float32) * np.float32(2.0 ** i) * np.float32(2) - np.float32(1)
             for i in range(-100, 101, 5)]
    return np.concatenate(parts + [np.array([-np.inf, 0.0, np.inf], np.float32)]).astype(np.float32)


def _enc(a):
    u = a.view(np.uint32)
    return np.where(u > np.uint32(1 << 31), ~u, u | np.uint32(1 << 31)).astype(np.uint32)


def test_argmin_encoding_matches_oracle_and_is_reversible():
    rng = np.random.default_rng(0)
    A = _test_array(rng)
    sample = A[rng.integers(0, len(A), 2000)]
    for x in sample[:400]:
        assert O.monotonic_u32(float(x)) == int(_enc(np.array([x], np.float32))[0])
        assert O.monotonic_f32(O.monotonic_u32(float(x))) == x
    # reversibility of the whole array (test_reversibility)
    enc = _enc(A)
    dec = np.array([O.monotonic_f32(int(e)) for e in enc[::37]], np.float32)
    assert np.array_equal(dec, A[::37])


def test_argmin_encoding_preserves_order():
    """test_comparison: x < y iff enc(x) < enc(y) for all pairs."""
    rng = np.random.default_rng(1)
    A = _test_array(rng)[rng.integers(0, 41003, 3000)]
    B = _test_array(rng)[rng.integers(0, 41003, 3000)]
    ea, eb = _enc(A), _enc(B)
    assert np.array_equal(A[:, None] < B[None, :], ea[:, None] < eb[None, :])


def test_argmin_decoding_preserves_order():
    """test_comparison2: decoded floats keep the order of their codes."""
    rng = np.random.default_rng(2)
    n = 2000
    A = (rng.integers(0, 1 << 32, n, dtype=np.uint64) % (1 << 24) + rng.integers(0, 1 << 32, n, dtype=np.uint64) % (1 << 31)).astype(np.uint32)
    dec = np.array([O.monotonic_f32(int(a)) for a in A], np.float32)
    ok = ~np.isnan(dec)
    a, d = A[ok], dec[ok]
    assert np.array_equal(a[:, None] < a[None, :], d[:, None] < d[None, :])


def test_pack_and_retrieve():
    k = O.pack_argmin(1.5, 77)
    assert O.retrieve_arg(k) == 77
    assert O.pack_argmin(1.0, 9) < O.pack_argmin(1.0, 10) < O.pack_argmin(2.0, 3)
    assert O.pack_argmin(float("inf"), 1) == 0xFF80000000000001


# ------------------------------------------------------------------ Philox


@pytest.mark.parametrize("ctr,key,want", [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
])
def test_philox_known_answers(ctr, key, want):
    assert list(O.philox(ctr, key)) == want


# ---------------------------------------------------------- formula facts


def test_upres_and_glass():
    assert list(O.upres(1)) == [0.0]
    assert list(O.upres(2)) == [-0.25, 0.25]
    assert np.array_equal(O.upres(4), T.upres(4))
    lin = (T.MATERIAL_LINEAR_REF, 0.0, 0.0)
    assert O.glass(lin, 400.0) == np.float32(1.3)
    assert abs(O.glass(lin, 700.0) - 1.4) < 1e-6
    assert abs(O.glass(S.CAUCHY_GLASS, 500.0) - (1.5 + 0.004 / 0.25)) < 1e-6


def test_can_refract_and_reflectance():
    assert O.can_refract((0, 0, -1), (0, 0, 1), 1.0, 1.5)
    s = np.sin(np.radians(60.0))
    v = (s, 0.0, -np.cos(np.radians(60.0)))
    assert not O.can_refract(v, (0, 0, 1), 1.5, 1.0)  # total internal reflection
    assert O.can_refract(v, (0, 0, 1), 1.0, 1.5)
    assert O.reflectance(v, (0, 0, 1), 1.2, 1.2) == 0.0  # equal media


def test_generator_derivatives_are_the_reference_constants():
    light = S.hemisphere_light(5, 32, 1.0)
    rays = O.rays_from_light(light, 2, (T.LAMBDA_FIXED, 1, 550.0, 550.0), seed=3)
    h2 = np.float32(32 // 2 // 2)
    np.testing.assert_array_equal(rays["dp_dx"], np.broadcast_to(light["dim1"] / h2, rays["dp_dx"].shape))
    np.testing.assert_array_equal(rays["dp_dy"], np.broadcast_to(light["dim2"] / h2, rays["dp_dy"].shape))
    assert (rays["lam"] == 550.0).all() and (rays["status"] == T.STATUS_ACTIVE).all()
    assert (rays["ignore_tri"] == 1).all() and (rays["dest"] == 0).all()
    assert len(rays) == 16 * 16
    # column-major over (row, col): ray k has row k % h + 1
    assert np.all(np.floor(rays["x"]) == (np.arange(256) % 16 + 1))


def test_trace_conserves_rays_and_is_deterministic():
    tris, fd = S.assemble(S.sphere_tris(2), S.floor_tris(-1.5, 4.0))
    wl = S.Workload(name="t", tris=tris, first_diffuse=fd, light=S.hemisphere_light(1, 32, 1.05), depth=3,
                    material=S.CAUCHY_GLASS, map_w=32, map_h=32, accum="i32", spectrum=S.stratified_spectrum(3),
                    lambda_mode=(T.LAMBDA_UNIFORM, 1, 400.0, 700.0))
    tex, st, rays = O.trace_forward(wl, keep_rays=True)
    tex2, st2, _ = O.trace_forward(wl, nthreads=1)
    assert np.array_equal(tex, tex2) and np.array_equal(st, st2)
    counts = np.bincount(rays["status"], minlength=3)
    assert st[0] == len(rays) == counts.sum()
    assert st[6] == counts[T.STATUS_DIFFUSE]
    # bounce b+1 sees exactly the rays still active after bounce b
    assert st[1] <= st[0] and st[2] <= st[1]
    # splitting the ray range splits the fixed-point map exactly
    a, _, _ = O.trace_forward(wl, 0, 400)
    b, _, _ = O.trace_forward(wl, 400, len(rays))
    assert np.array_equal(a + b, tex)


def test_brute_force_tie_rule_prefers_the_smaller_index():
    """Coincident triangles (equal t): the lexicographic (t, index) minimum
    (src/hitters.jl:26, :187-197) returns the smaller index."""
    tri = S.floor_tris(0.0, 1.0)[:1]
    tris = np.concatenate([np.zeros((1, 10, 3), np.float32), tri, tri], 0)
    rays = np.zeros(1, dtype=T.ADRAY)
    rays["pos"] = [0.5, 1.0, 0.3]
    rays["dir"] = [0.0, -1.0, 0.0]
    rays["ignore_tri"] = 1
    hit, t = O.next_hit(rays, tris)
    assert hit[0] == 2 and t[0] == 1.0
    rays["ignore_tri"] = 2
    hit, _ = O.next_hit(rays, tris)
    assert hit[0] == 3
