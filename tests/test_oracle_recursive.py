"""Pin the oracle's RecursiveGaussianFilter (oracle/gauss_oracle.c,
orc_recursive_gaussian_f64) before trusting it.

1. Bit-exact f64 against the `rec_*` cases of tests/golden/golden.npz (the
   pure-Python transcription of recursive_gaussian.rs in
   tests/golden/make_golden.py).
2. The reference's own tests (recursive_gaussian.rs:248-303), re-run against the
   oracle.
3. The Young & van Vliet coefficients have unit DC gain: B + a1 + a2 + a3 = 1.
"""
import numpy as np
import pytest

import oracle

REC = ["impulse1d_s2", "const2d_s1p5", "rand2d_s3", "rand3d_s1p2_aniso", "rand3d_axis1_s0p3", "u8_2d_s2",
       "thin3d_s2"]


def rec_meta(golden, name):
    m = golden[f"rec_{name}__meta"]
    return float(m[0]), int(m[1]), [float(v) for v in m[2:]]


@pytest.mark.parametrize("name", REC)
def test_recursive_oracle_matches_golden(golden, name):
    sigma, axis, spacing = rec_meta(golden, name)
    got = oracle.recursive_gaussian_f64(golden[f"rec_{name}__in"], sigma, spacing, axis)
    want = golden[f"rec_{name}__f64"]
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


@pytest.mark.parametrize("sigma", [0.1, 0.5, 1.0, 2.0, 2.5, 4.0, 12.0])
def test_yvv_unit_dc_gain(sigma):
    b, a1, a2, a3 = oracle.yvv_coeffs(sigma)
    assert abs(b + a1 + a2 + a3 - 1.0) < 1e-12


def test_yvv_small_and_nan_sigma_clamp():
    """sigma.max(0.5) (recursive_gaussian.rs:34): below 0.5 and NaN use 0.5."""
    want = oracle.yvv_coeffs(0.5)
    assert np.array_equal(oracle.yvv_coeffs(0.1), want)
    assert np.array_equal(oracle.yvv_coeffs(float("nan")), want)


def _impulse(n):
    x = np.zeros(n, np.float32)
    x[n // 2] = 1.0
    return x


def test_energy_conserved_1d():
    """recursive_gaussian.rs:259-266"""
    out = oracle.recursive_gaussian_f32(_impulse(51), 2.0)
    assert abs(float(out.sum(dtype=np.float32)) - 1.0) < 0.02


def test_peak_at_centre():
    """recursive_gaussian.rs:268-277"""
    out = oracle.recursive_gaussian_f32(_impulse(51), 2.0)
    assert out[25] > out[28]


def test_constant_image_unchanged():
    """recursive_gaussian.rs:279-293"""
    out = oracle.recursive_gaussian_f32(np.full((15, 15), 4.0, np.float32), 1.5)
    assert np.all(np.abs(out[3:12, 3:12] - 4.0) < 0.05)


def test_single_axis_filter():
    """recursive_gaussian.rs:295-302"""
    out = oracle.recursive_gaussian_f32(_impulse(31), 2.0, axis=0)
    assert abs(float(out.sum(dtype=np.float32)) - 1.0) < 0.02


def test_u8_output_conversion():
    """u8::from_f64 (pixel.rs:36): round half away from zero, clamp, NaN -> 0."""
    v = np.array([0.49999999999999994, 0.5, 1.5, 2.5, -0.5, 255.5, np.nan, -3.0, 254.4])
    assert list(oracle.from_f64_u8(v)) == [0, 1, 2, 3, 0, 255, 0, 0, 254]


RECD = ["gm2d", "gm3d_sub", "lap2d", "deriv3d_o1_a2", "deriv2d_o2_a0_sub", "deriv2d_o3", "grad3d", "hess2d",
        "hess2d_sub", "gm_u8_2d", "lap3d_zc_sub"]
# zero crossings of these Laplacian cases (ZeroCrossingBasedEdgeDetectionFilter)
RECZ = {"lap2d": "lap2d", "lap3d_sub": "lap3d_zc_sub"}


def recd_meta(golden, name):
    m = golden[f"recd_{name}__meta"]
    x = golden[f"recd_{name}__in"]
    D = x.ndim
    sigma, kind, axis, order = float(m[0]), int(m[1]), int(m[2]), int(m[3])
    sp = [float(v) for v in m[4:4 + D]]
    ri = tuple(int(v) for v in m[4 + D:4 + 2 * D])
    rs = tuple(int(v) for v in m[4 + 2 * D:4 + 3 * D])
    return x, sigma, kind, axis, order, sp, (ri, rs)


@pytest.mark.parametrize("name", RECD)
def test_recursive_derivative_oracle_matches_golden(golden, name):
    """The derivative users (edges.rs:686-950) against the pure-Python transcription."""
    x, sigma, kind, axis, order, sp, req = recd_meta(golden, name)
    got = oracle.recursive_derivative(x, sigma, kind, sp, axis, order, requested=req)
    want = golden[f"recd_{name}__out"]
    assert got.shape == want.shape
    if want.dtype == np.uint8:
        assert np.array_equal(got, want)
    else:
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_recursive_derivative_of_a_ramp():
    """The first derivative is the central difference of the smoothed image, in f64."""
    x = np.tile(np.arange(16, dtype=np.float32) * 0.5, (12, 1))
    g = oracle.recursive_derivative(x, 0.5, oracle.REC_DERIVATIVE, axis=0, order=1)
    sm = oracle.recursive_gaussian_f32(x, 0.5)
    want = (sm[:, 2:].astype(np.float64) - sm[:, :-2]) / 2.0
    assert np.array_equal(g[:, 1:-1], want.astype(np.float32))


def test_difference_of_gaussians_oracle():
    """DifferenceOfGaussiansFilter (edges.rs:995-1006): the f64 difference of the two
    smoothings, each first converted to the pixel type."""
    x = np.random.default_rng(7).random((9, 11), dtype=np.float32)
    s1 = oracle.recursive_gaussian_f32(x, 1.0).astype(np.float64)
    s2 = oracle.recursive_gaussian_f32(x, 2.5).astype(np.float64)
    got = oracle.recursive_difference_of_gaussians(x, 1.0, 2.5)
    assert np.array_equal(got.view(np.uint32), (s1 - s2).astype(np.float32).view(np.uint32))


@pytest.mark.parametrize("name", sorted(RECZ))
def test_zero_crossing_edges_oracle_matches_golden(golden, name):
    """ZeroCrossingBasedEdgeDetectionFilter (edges.rs:1019-1052) against the pure-Python
    transcription of ZeroCrossingFilter over the Laplacian golden case."""
    x, sigma, kind, axis, order, sp, req = recd_meta(golden, RECZ[name])
    got = oracle.recursive_zero_crossing_edges(x, sigma, sp, requested=req)
    want = golden[f"recz_{name}__out"]
    assert got.dtype == want.dtype and np.array_equal(got, want)


def test_zero_crossings_of_a_sign_change():
    """A Laplacian that changes sign between two columns marks both columns."""
    x = np.zeros((6, 12), np.float32)
    x[:, 6:] = 10.0
    z = oracle.recursive_zero_crossing_edges(x, 0.8)
    assert z.dtype == np.float32 and set(np.unique(z)) <= {0.0, 1.0}
    assert z[:, 5].all() and z[:, 6].all() and not z[:, 0].any() and not z[:, -1].any()


def _ramp(n):
    return np.arange(n, dtype=np.float32)


def test_reference_stencil_tests_through_the_smoothing():
    """The reference's stencil tests (edges.rs:1614-1662: derivative of a ramp is 1,
    second derivative of x^2 is 2, gradient magnitude of a ramp is 1, Laplacian of a
    ramp is 0), re-run on the derivative users: the recursive smoothing keeps ramps and
    quadratics up to a constant away from the edges, so the same values hold inside."""
    r = _ramp(80)
    inner = slice(20, 60)
    d = oracle.recursive_derivative(r, 1.0, oracle.REC_DERIVATIVE, axis=0, order=1)
    assert np.all(np.abs(d[inner] - 1.0) < 1e-3)
    q = (np.arange(80, dtype=np.float64) ** 2).astype(np.float32)
    d2 = oracle.recursive_derivative(q, 1.0, oracle.REC_DERIVATIVE, axis=0, order=2)
    assert np.all(np.abs(d2[inner] - 2.0) < 1e-2)
    g = oracle.recursive_derivative(r, 1.0, oracle.REC_GRADIENT_MAGNITUDE)
    assert np.all(np.abs(g[inner] - 1.0) < 1e-3)
    lap = oracle.recursive_derivative(r, 1.0, oracle.REC_LAPLACIAN)
    assert np.all(np.abs(lap[inner]) < 1e-3)
    # a flat image has no edges (edges.rs:1665-1671 for Sobel; here every derivative user)
    flat = np.ones((6, 7), np.float32)
    for kind in (oracle.REC_GRADIENT_MAGNITUDE, oracle.REC_LAPLACIAN):
        assert np.all(np.abs(oracle.recursive_derivative(flat, 1.5, kind)) < 1e-5)
    assert not oracle.recursive_zero_crossing_edges(flat, 1.5).any()
