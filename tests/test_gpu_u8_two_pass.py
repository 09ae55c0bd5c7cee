"""GaussianFilter<Image<u8>> in the reference's u8 pixel arithmetic
(NumericPixel for u8, src/pixel.rs:430-435: each tap is
round(x as f64 * w).clamp(0, 255) as u8, added with a wrapping u8 add) through
the two-pass 3-D kernels, bit-exact against the oracle's restatement and
against the per-axis passes."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def run_u8(itkg, arr, sigma, spacing=None, requested=None, index=None, algo=None):
    img = itkg.Image(arr, index=index, spacing=spacing)
    dev = itkg.DeviceImage.from_host(img)
    f = itkg.GaussianFilter(dev, sigma, arithmetic=itkg.ARITH_PIXEL_U8,
                            algorithm=algo if algo is not None else itkg.ALGO_AUTO)
    req = itkg.Region(*requested) if requested else img.region
    return f.generate_region(req, out_dtype=itkg.U8).download()


CASES = [
    # (shape z, y, x), sigma, spacing, requested (index, size) or None
    ((20, 40, 64), 1.5, None, None),                     # whole quads: 4-byte stores
    ((17, 33, 50), 2.2, None, None),                     # ragged width: element stores
    ((24, 70, 72), 1.0, (1.0, 1.0, 2.0), None),          # z radius 2, x-y radius 3
    ((30, 45, 96), 4.0, None, None),                     # radius 12, the largest the kernels take
    ((26, 50, 80), 2.0, None, ((16, 5, 3), (48, 30, 14))),  # sub-region, clamped only at some edges
    ((9, 140, 36), 0.8, None, None),                     # several tiles along y, short z
]


@pytest.mark.parametrize("shape,sigma,spacing,req", CASES)
def test_u8_pixel_two_pass_bit_exact(gpu, shape, sigma, spacing, req):
    arr = np.random.default_rng(sum(shape)).integers(0, 256, shape, dtype=np.uint8)
    got = run_u8(gpu, arr, sigma, spacing=spacing, requested=req)
    assert gpu.last_kernel() == "z_pass_u8_pixel"
    want = oracle.gaussian_u8(arr, sigma, spacing=spacing, requested=req)
    assert np.array_equal(got, want)


def test_u8_pixel_two_pass_wrapping_sums(gpu):
    """Bright images, where the tap values of one output add up to more than
    255 and the u8 add wraps (the reference's wrapping add, not saturation)."""
    arr = np.full((12, 36, 40), 255, np.uint8)
    arr[:, :, ::3] = 250
    wrapped = False
    for sigma in (0.7, 1.3, 2.9):
        got = run_u8(gpu, arr, sigma)
        want = oracle.gaussian_u8(arr, sigma)
        assert np.array_equal(got, want), sigma
        wrapped |= bool((want < 200).any())
    assert wrapped  # sigma 2.9: the sums pass 255 and wrap


def test_u8_pixel_two_pass_offset_index(gpu):
    """The x-y kernel's tile loads start on 16-byte columns of the input: a
    request starting 16 columns into the buffer takes the two-pass kernels,
    one starting elsewhere the per-axis passes -- bit-identical either way."""
    arr = np.random.default_rng(5).integers(0, 256, (15, 29, 44), dtype=np.uint8)
    index = (7, -4, 30)
    for req, two_pass in ((((23, 0, 33), (16, 20, 9)), True), (((11, 0, 33), (28, 20, 9)), False)):
        got = run_u8(gpu, arr, 1.7, index=index, requested=req)
        assert (gpu.last_kernel() == "z_pass_u8_pixel") == two_pass
        assert np.array_equal(got, oracle.gaussian_u8(arr, 1.7, index=index, requested=req))


def test_u8_pixel_two_pass_equals_per_axis(gpu):
    arr = np.random.default_rng(6).integers(0, 256, (22, 41, 52), dtype=np.uint8)
    for sigma in (0.6, 1.1, 3.3):
        a = run_u8(gpu, arr, sigma, algo=gpu.ALGO_TWO_PASS)
        assert gpu.last_kernel() == "z_pass_u8_pixel"
        b = run_u8(gpu, arr, sigma, algo=gpu.ALGO_PER_AXIS)
        assert gpu.last_kernel() != "z_pass_u8_pixel"
        assert np.array_equal(a, b), sigma


def test_u8_pixel_two_pass_sigma_sweep(gpu):
    """Every radius 1 .. 12 (sigma 0.3 .. 4.0): each kernel's f32 tap constants
    reproduce its u8 tap tables, so the two-pass kernels take every one."""
    arr = np.random.default_rng(7).integers(0, 256, (14, 30, 40), dtype=np.uint8)
    for sigma in np.arange(0.3, 4.01, 0.17):
        got = run_u8(gpu, arr, float(sigma))
        assert gpu.last_kernel() == "z_pass_u8_pixel", sigma
        assert np.array_equal(got, oracle.gaussian_u8(arr, float(sigma))), sigma
