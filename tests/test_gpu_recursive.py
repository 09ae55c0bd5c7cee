"""GPU parity of RecursiveGaussianFilter / RecursiveGaussianAxisFilter through
itkg_recursive_gaussian_generate_region, against the oracle on the same
seeded inputs: reference rounding (f64, the reference's operation order)
bit-exact; FMA rounding (f64 with fused multiply-adds) within 1e-5 normwise
(max|gpu - ref| / max|ref|)."""
import numpy as np
import pytest

import oracle
from test_gpu_parity import bits_equal, normwise
from test_oracle_recursive import REC, rec_meta

pytestmark = pytest.mark.gpu

TOL_FMA = 1e-5


def run(itkg, arr, sigma, spacing=None, axis=None, rounding=0, requested=None, index=None, host=False,
        out_dtype=None):
    img = itkg.Image(arr, index=index, spacing=spacing)
    src = img if host else itkg.DeviceImage.from_host(img)
    f = itkg.RecursiveGaussianFilter(src, sigma, axis=axis, rounding=rounding)
    req = itkg.Region(*requested) if requested else img.region
    out = f.generate_region(req, out_dtype=out_dtype)
    return out.data if host else out.download()


@pytest.mark.parametrize("name", REC)
def test_golden_bit_exact(gpu, golden, name):
    sigma, axis, spacing = rec_meta(golden, name)
    x = golden[f"rec_{name}__in"]
    f64 = golden[f"rec_{name}__f64"]
    got = run(gpu, x, sigma, spacing, None if axis < 0 else axis)
    if x.dtype == np.uint8:
        assert np.array_equal(got, oracle.from_f64_u8(f64))
    else:
        assert bits_equal(got, f64.astype(np.float32))


@pytest.mark.parametrize("shape,sigma,spacing", [((30, 36, 40), 2.0, None), ((17, 33, 29), 5.5, (0.7, 0.9, 2.5)),
                                                 ((64, 96), 1.2, None), ((300,), 8.0, None),
                                                 ((96, 128, 160), 2.0, None)])
@pytest.mark.parametrize("rounding", [0, 1])
def test_random(gpu, shape, sigma, spacing, rounding):
    x = np.random.default_rng(len(shape) * 7 + int(sigma * 10)).standard_normal(shape).astype(np.float32)
    want = oracle.recursive_gaussian_f32(x, sigma, spacing)
    got = run(gpu, x, sigma, spacing, rounding=rounding)
    if rounding == 0:
        assert bits_equal(got, want)
    else:
        assert normwise(got, want) <= TOL_FMA


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_axis_filter(gpu, axis):
    x = np.random.default_rng(80 + axis).random((12, 14, 16), dtype=np.float32)
    want = oracle.recursive_gaussian_f32(x, 1.7, axis=axis)
    got = run(gpu, x, 1.7, axis=axis)
    assert bits_equal(got, want)
    assert gpu.last_kernel() == "recursive_lines_f64"


def test_subregion_with_offset_index(gpu):
    x = np.random.default_rng(90).standard_normal((20, 22, 24)).astype(np.float32)
    index = (3, -5, 10)
    req = ((7, 0, 12), (11, 9, 6))
    want = oracle.recursive_gaussian_f32(x, 2.3, requested=req, index=index)
    got = run(gpu, x, 2.3, requested=req, index=index)
    assert bits_equal(got, want)


def test_i16_input_and_u8_output(gpu):
    rng = np.random.default_rng(91)
    x16 = rng.integers(-1000, 1500, (10, 12, 14)).astype(np.int16)
    want = oracle.recursive_gaussian_f32(x16.astype(np.float64), 1.5)
    assert bits_equal(run(gpu, x16, 1.5), want)
    x8 = rng.integers(0, 256, (18, 20), dtype=np.uint8)
    f64 = oracle.recursive_gaussian_f64(x8.astype(np.float64), 2.0)
    assert np.array_equal(run(gpu, x8, 2.0, out_dtype=gpu.U8), oracle.from_f64_u8(f64))


def test_host_buffers(gpu):
    x = np.random.default_rng(92).standard_normal((24, 28, 32)).astype(np.float32)
    want = oracle.recursive_gaussian_f32(x, 3.0)
    assert bits_equal(run(gpu, x, 3.0, host=True), want)


def test_reference_tests(gpu):
    """recursive_gaussian.rs:259-302 through the GPU path."""
    imp = np.zeros(51, np.float32)
    imp[25] = 1.0
    out = run(gpu, imp, 2.0)
    assert abs(float(out.sum(dtype=np.float32)) - 1.0) < 0.02 and out[25] > out[28]
    out = run(gpu, np.full((15, 15), 4.0, np.float32), 1.5)
    assert np.all(np.abs(out[3:12, 3:12] - 4.0) < 0.05)
    imp = np.zeros(31, np.float32)
    imp[15] = 1.0
    out = run(gpu, imp, 2.0, axis=0)
    assert abs(float(out.sum(dtype=np.float32)) - 1.0) < 0.02



@pytest.mark.parametrize("sigma", [0.1, 0.5, 1.3, 2.0, 2.5, 7.0, float("nan")])
def test_coefficients_match_oracle_on_this_host(gpu, sigma):
    """The library's host-side coefficients are the oracle's bit for bit on the
    machine that runs the GPU tests too (no host-compiler FMA contraction)."""
    assert np.array_equal(gpu.yvv_coeffs(sigma), oracle.yvv_coeffs(sigma))


# ---- the derivative users (edges.rs:686-950) --------------------------------
from test_oracle_recursive import RECD, RECZ, recd_meta  # noqa: E402


def run_deriv(itkg, arr, sigma, kind, spacing=None, axis=0, order=1, requested=None, index=None, host=False,
              rounding=0):
    img = itkg.Image(arr, index=index, spacing=spacing)
    src = img if host else itkg.DeviceImage.from_host(img)
    f = itkg.RecursiveGaussianDerivativeFilter(src, sigma, kind, axis=axis, order=order, rounding=rounding)
    req = itkg.Region(*requested) if requested else img.region
    out = f.generate_region(req)
    return out.data if host else out.download()


def _same(got, want):
    if want.dtype == np.uint8:
        return np.array_equal(got, want)
    return got.shape == want.shape and bits_equal(got, want)


@pytest.mark.parametrize("name", RECD)
def test_derivative_golden_bit_exact(gpu, golden, name):
    x, sigma, kind, axis, order, sp, req = recd_meta(golden, name)
    got = run_deriv(gpu, x, sigma, kind, sp, axis, order, requested=req)
    assert _same(got, golden[f"recd_{name}__out"]), gpu.last_kernel()


@pytest.mark.parametrize("kind,axis,order", [(0, 0, 1), (1, 0, 1), (2, 1, 1), (2, 2, 2), (3, 0, 1)])
def test_derivative_random_3d(gpu, kind, axis, order):
    x = np.random.default_rng(100 + kind).standard_normal((20, 26, 31)).astype(np.float32)
    sp = (0.8, 1.1, 1.7)
    req = ((3, 2, 4), (25, 21, 12))
    want = oracle.recursive_derivative(x, 2.2, kind, sp, axis, order, requested=req)
    got = run_deriv(gpu, x, 2.2, kind, sp, axis, order, requested=req)
    assert _same(got, want)
    assert gpu.last_kernel() == "recursive_derivative"


def test_hessian_2d_and_host_buffers(gpu):
    x = np.random.default_rng(110).random((40, 52), dtype=np.float32)
    want = oracle.recursive_derivative(x, 1.6, oracle.REC_HESSIAN, (0.9, 1.3))
    assert _same(run_deriv(gpu, x, 1.6, 4, (0.9, 1.3),
                           host=True), want)
    want = oracle.recursive_derivative(x, 1.6, oracle.REC_GRADIENT, (0.9, 1.3))
    assert _same(run_deriv(gpu, x, 1.6, 3, (0.9, 1.3)), want)  # 2 components


def test_derivative_u8(gpu):
    x = np.random.default_rng(111).integers(0, 256, (18, 22), dtype=np.uint8)
    for kind in (0, 1):
        want = oracle.recursive_derivative(x, 1.3, kind)
        assert _same(run_deriv(gpu, x, 1.3, kind), want)


def test_derivative_convenience_classes(gpu):
    x = np.random.default_rng(112).standard_normal((10, 12, 14)).astype(np.float32)
    d = gpu.DeviceImage.from_host(gpu.Image(x))
    g = gpu.GradientMagnitudeRecursiveGaussianFilter(d, 1.5).generate_region(d.region).download()
    assert _same(g, oracle.recursive_derivative(x, 1.5, 0))
    g = gpu.DiscreteGaussianDerivativeFilter(d, 1.5, axis=2, order=2).generate_region(d.region).download()
    assert _same(g, oracle.recursive_derivative(x, 1.5, 2, axis=2, order=2))
    g = gpu.GradientRecursiveGaussianFilter(d, 1.5).generate_region(d.region).download()
    assert _same(g, oracle.recursive_derivative(x, 1.5, 3))


@pytest.mark.parametrize("dtype", [np.float32, np.uint8])
def test_difference_of_gaussians(gpu, dtype):
    rng = np.random.default_rng(113)
    x = (rng.random((16, 20, 24)) * 200).astype(dtype)
    req = ((2, 3, 1), (19, 15, 12))
    want = oracle.recursive_difference_of_gaussians(x, 1.2, 3.0, (0.9, 1.0, 1.4), requested=req)
    d = gpu.DeviceImage.from_host(gpu.Image(x, spacing=(0.9, 1.0, 1.4)))
    got = gpu.DifferenceOfGaussiansFilter(d, 1.2, 3.0).generate_region(gpu.Region(*req)).download()
    assert _same(got, want)
    assert gpu.last_kernel() == "recursive_difference"


@pytest.mark.parametrize("name", sorted(RECZ))
def test_zero_crossing_golden(gpu, golden, name):
    x, sigma, kind, axis, order, sp, req = recd_meta(golden, RECZ[name])
    got = run_deriv(gpu, x, sigma, gpu.REC_ZERO_CROSSING, sp, requested=req)
    assert _same(got, golden[f"recz_{name}__out"])
    assert gpu.last_kernel() == "recursive_zero_crossing"


@pytest.mark.parametrize("dtype", [np.float32, np.uint8])
def test_zero_crossing_edges(gpu, dtype):
    rng = np.random.default_rng(114)
    x = (rng.standard_normal((18, 21, 25)) * 40 + 100).astype(dtype)
    req = ((2, 1, 3), (20, 18, 13))
    sp = (1.0, 0.7, 1.6)
    want = oracle.recursive_zero_crossing_edges(x, 1.4, sp, requested=req)
    d = gpu.DeviceImage.from_host(gpu.Image(x, spacing=sp))
    got = gpu.ZeroCrossingBasedEdgeDetectionFilter(d, 1.4).generate_region(gpu.Region(*req)).download()
    assert _same(got, want)
    if dtype == np.float32:
        assert 0 < int(want.sum()) < want.size
