"""Pin the oracle's convolve_axis family (MeanFilter, BoxMeanFilterN,
BinomialBlurFilter) before trusting it.

1. Bit-exact against the `sep_*` cases of tests/golden/golden.npz (the
   pure-Python transcription of mean.rs and binomial_blur.rs in
   tests/golden/make_golden.py).
2. The reference's own tests of these filters, re-run against the oracle:
   mean.rs:246-293 and binomial_blur.rs:92-129.
3. Known answers: with one round the binomial schedule is the Gaussian's; in
   the interior n rounds equal one pass of the (2n + 1)-tap binomial kernel.
"""
import math

import numpy as np
import pytest

import oracle

GOLDEN_SEP = ["mean1d_const_r2", "mean1d_ramp_r2", "boxmean2d_const", "mean2d_r3", "mean2d_sub_r2",
              "mean3d_r2", "boxmean3d_aniso", "mean2d_r6_tiny", "mean_vec2d_r1", "binomial1d_const_r4",
              "binomial1d_impulse_r4", "binomial2d_r3", "binomial2d_sub_r2", "binomial3d_r2",
              "binomial3d_r0"]
GOLDEN_SEP_U8 = ["mean_u8_2d_r2", "binomial_u8_2d_r2"]


def sep_meta(golden, name):
    """(kernels, reps, comps, requested) of a golden family case."""
    m = [int(v) for v in golden[f"sep_{name}__meta"]]
    fam, reps, comps = m[0], m[1], m[2]
    x = golden[f"sep_{name}__in"]
    D = x.ndim - (1 if comps > 1 else 0)
    radii = m[3:3 + D]
    ri, rs = tuple(m[6:6 + D]), tuple(m[6 + D:6 + 2 * D])
    kernels = [oracle.BINOMIAL_KERNEL] * D if fam == 2 else [oracle.box_kernel(r) for r in radii]
    return kernels, reps, comps, (ri, rs)


@pytest.mark.parametrize("name", GOLDEN_SEP)
def test_family_oracle_matches_golden(golden, name):
    kernels, reps, comps, req = sep_meta(golden, name)
    got = oracle.separable_f32(golden[f"sep_{name}__in"], kernels, reps, requested=req, comps=comps)
    want = golden[f"sep_{name}__out"]
    assert got.shape == want.shape
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("name", GOLDEN_SEP_U8)
def test_family_oracle_matches_golden_u8(golden, name):
    kernels, reps, comps, req = sep_meta(golden, name)
    got = oracle.separable_u8(golden[f"sep_{name}__in"], kernels, reps, requested=req, comps=comps)
    assert np.array_equal(got, golden[f"sep_{name}__out"])


def test_box_kernel():
    """mean.rs:15-18"""
    for r in (0, 1, 2, 5):
        k = oracle.box_kernel(r)
        assert len(k) == 2 * r + 1 and np.all(k == 1.0 / (2 * r + 1))


def test_mean_constant_image():
    """mean.rs:254-262"""
    out = oracle.mean_f32(np.full(10, 5.0, np.float32), 2)
    assert np.all(np.abs(out - 5.0) < 1e-5)


def test_mean_ramp_interior():
    """mean.rs:264-276"""
    out = oracle.mean_f32(np.arange(20, dtype=np.float32), 2)
    for i in range(2, 18):
        assert abs(out[i] - i) < 1e-4


def test_box_mean_2d_constant():
    """mean.rs:278-292"""
    out = oracle.box_mean_f32(np.full((8, 8), 3.0, np.float32), (1, 2))
    assert np.all(np.abs(out - 3.0) < 1e-5)


def test_binomial_constant_image_preserved():
    """binomial_blur.rs:96-106"""
    out = oracle.binomial_f32(np.full(20, 3.0, np.float32), 4)
    assert np.all(np.abs(out[4:16] - 3.0) < 1e-5)


def test_binomial_impulse_spreads():
    """binomial_blur.rs:108-121"""
    x = np.zeros(21, np.float32)
    x[10] = 1.0
    out = oracle.binomial_f32(x, 4)
    assert 0.0 < out[10] < 1.0
    assert abs(float(out.sum(dtype=np.float32)) - 1.0) < 0.05


def test_binomial_effective_sigma():
    """binomial_blur.rs:123-128: sqrt(n / 4)"""
    assert abs(math.sqrt(4 / 4.0) - 1.0) < 1e-10


def test_one_round_is_the_gaussian_schedule():
    """With reps = 1 the binomial schedule is the Gaussian's (gaussian.rs:79-85),
    so a Gaussian-like kernel through the family equals the Gaussian oracle."""
    rng = np.random.default_rng(3)
    x = rng.standard_normal((7, 9, 10)).astype(np.float32)
    w = oracle.build_kernel(1.2, oracle.kernel_radius(1.2, 1.0))
    a = oracle.separable_f32(x, [w] * 3, 1, requested=((1, 2, 1), (7, 5, 4)))
    b = oracle.gaussian_f32(x, 1.2, requested=((1, 2, 1), (7, 5, 4)))
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_binomial_interior_is_the_composite_kernel():
    """n rounds of [1,2,1]/4 = one pass of C(2n, k) / 4^n away from the clamp (FP64)."""
    rng = np.random.default_rng(4)
    x = rng.standard_normal((12, 13, 14))
    n = 3
    comp = np.array([math.comb(2 * n, k) for k in range(2 * n + 1)]) / 4.0 ** n
    a = oracle.separable_f64(x, [oracle.BINOMIAL_KERNEL] * 3, n)
    b = oracle.separable_f64(x, [comp] * 3, 1)
    assert np.abs(a - b)[n:-n, n:-n, n:-n].max() < 1e-13
    assert np.abs(a - b).max() > 1e-3  # repeated clamping differs at the edges


def test_family_mt_port_matches_serial():
    rng = np.random.default_rng(5)
    x = rng.standard_normal((6, 11, 12)).astype(np.float32)
    a = oracle.separable_f32(x, [oracle.BINOMIAL_KERNEL] * 3, 2)
    b = oracle.separable_f32_mt(x, [oracle.BINOMIAL_KERNEL] * 3, 2, nthreads=3)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
