"""The camera pass's host-side pieces without a GPU: the library's retina
factors and get_camera against the oracle's restatements (bit-exact), the
oracle's camera-ray derivatives against central differences of the
double-precision direction, and the reference's retina-curve facts."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from splat_gb300 import _lib as L
from splat_gb300 import scenes as S


def lib_retina(spec) -> np.ndarray:
    spec = np.ascontiguousarray(spec, np.float32)
    out = np.zeros((3, len(spec)), np.float32)
    L.check(L.load().splat_retina_factors(spec.ctypes.data, len(spec), out.ctypes.data))
    return out


@pytest.mark.parametrize("spec", [
    np.arange(400, 701, 25, dtype=np.float32),          # the reference's 400:25:700
    S.stratified_spectrum(16),
    np.array([380, 399, 399.5, 400, 460, 462, 466, 534, 536, 612, 700, 701, 720], np.float32),  # knots, outside
    np.random.default_rng(1).uniform(390, 710, 64).astype(np.float32),
])
def test_retina_factors_match_the_literal_piecewise_tree(spec):
    """The library's segment search equals the reference's comparison tree
    (restated literally in the oracle) bit for bit, knots and extrapolation
    included."""
    got = lib_retina(spec)
    want = O.retina_factors(spec)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_retina_curves_are_normalised():
    """Each curve sums to 1 over 400..700 nm (it is divided by that sum) and
    is non-negative inside the knots."""
    x = np.arange(400, 701, dtype=np.float32)
    r = lib_retina(x).astype(np.float64)
    np.testing.assert_allclose(r.sum(axis=1), 1.0, rtol=1e-6)
    assert (r >= 0).all()
    # the red curve's peak is at 602 nm, green's at 534, blue's at 463
    assert [int(x[np.argmax(r[c])]) for c in range(3)] == [602, 534, 463]


def test_camera_look_at_matches_oracle():
    for pos, at, up, fov in [((0, 5, 5), (0, 0, 0), (0, 0, -1), 45 * np.pi / 180),
                             ((0.0, 2.5, 5.0), (0.0, -0.5, 0.0), (0.0, 1.0, 0.0), 0.9),
                             ((3.1, -2.2, 0.7), (0.3, 0.1, -0.2), (0.2, 0.9, 0.1), 1.7)]:
        f = lambda v: (C.c_float * 3)(*[float(a) for a in v])  # noqa: E731
        cam = L.Camera()
        L.check(L.load().splat_camera_look_at(f(pos), f(at), f(up), float(fov), C.byref(cam)))
        ref = O.camera_look_at(pos, at, up, fov)
        assert bytes(cam) == bytes(ref)
    bad = L.Camera()
    assert L.load().splat_camera_look_at(f((0, 0, 0)), f((0, 1, 0)), f((0, 1, 0)), 1.0, C.byref(bad)) == L.ERR_INVALID


def test_camera_ray_derivatives_match_central_differences():
    """dd/dx and dd/dy of camera_ray (ForwardDiff in the reference) against
    central differences of the same double-precision direction."""
    cam = O.camera_look_at((0, 5, 5), (0, 0, 0), (0, 0, -1), 45 * np.pi / 180)
    h, w = 36, 64
    rays = O.camera_rays(cam, h, w, 550.0, seed=3)
    R, U, D = (np.array(v, np.float64) for v in (cam.right, cam.up, cam.dir))
    scale = h * (1 / np.sqrt(2)) / np.float64(np.float32(cam.fov_half_sin))

    def direction(x, y):
        vx, vy = (x - h / 2) / scale, (y - w / 2) / scale
        return vx * R + vy * U + np.sqrt(1 - vx * vx - vy * vy) * D

    eps = 1e-4
    for g in [0, 7, h * 11 + 5, h * w - 1]:
        x, y = g % h + 1, g // h + 1
        ddx = (direction(x + eps, y) - direction(x - eps, y)) / (2 * eps)
        ddy = (direction(x, y + eps) - direction(x, y - eps)) / (2 * eps)
        np.testing.assert_allclose(rays[g]["dd_dx"], ddx, rtol=1e-5, atol=1e-7)
        np.testing.assert_allclose(rays[g]["dd_dy"], ddy, rtol=1e-5, atol=1e-7)
        assert rays[g]["dest"] == (y - 1) * h + x
    assert (rays["ignore_tri"] == 1).all() and (rays["x"] == 0).all() and (rays["lam"] == 550.0).all()
    # unit-length up to the small jitter term dv * 0.025 / max(h, w)
    n = np.linalg.norm(rays["dir"].astype(np.float64), axis=1)
    assert np.abs(n - 1).max() < 0.025 * np.sqrt(3) / max(h, w) + 1e-6


def test_checkered_map_is_the_reference_pattern():
    m = S.checkered_map(4, 3, 2, 12.0)
    assert m.shape == (24, 24, 2)
    assert m[0, 0, 0] == 0 and m[4, 0, 0] == 12 and m[4, 4, 1] == 0 and m[0, 4, 0] == 12
