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
