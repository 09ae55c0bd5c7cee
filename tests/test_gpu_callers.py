"""GPU parity of the in-crate callers of GaussianFilter: SliceBySliceFilter
(spatial.rs:1284-1340) through itkg_slice_by_slice_generate_region and
BSplineDownsampleFilter (spatial.rs:1128-1166) through
itkg_bspline_downsample_generate_region, against the oracle: bit-exact in
reference rounding, within 1e-5 normwise in FMA rounding."""
import numpy as np
import pytest

import oracle
from test_gpu_parity import bits_equal, normwise
from test_oracle_callers import dfb_meta, slice_meta

pytestmark = pytest.mark.gpu


def run_slices(itkg, arr, sigma, spacing=None, requested=None, index=None, host=False, rounding=0):
    img = itkg.Image(arr, index=index, spacing=spacing)
    src = img if host else itkg.DeviceImage.from_host(img)
    f = itkg.SliceBySliceFilter(src, sigma, rounding=rounding)
    req = itkg.Region(*requested) if requested else img.region
    out = f.generate_region(req)
    return out.data if host else out.download()


def run_bspline(itkg, arr, spacing=None, host=False, rounding=0):
    img = itkg.Image(arr, spacing=spacing)
    src = img if host else itkg.DeviceImage.from_host(img)
    out = itkg.BSplineDownsampleFilter(src, rounding=rounding).generate_region()
    return out.data if host else out.download()


@pytest.mark.parametrize("name", ["slices_s1p2", "slices_u8_s1"])
def test_slice_golden(gpu, golden, name):
    sigma, sp, req = slice_meta(golden, name)
    want = golden[f"cal_{name}__out"]
    got = run_slices(gpu, golden[f"cal_{name}__in"], sigma, sp, requested=req)
    assert got.dtype == want.dtype and np.array_equal(np.asarray(got).view(np.uint8), want.view(np.uint8))


@pytest.mark.parametrize("name", ["bspline3d_odd", "bspline2d_aniso"])
def test_bspline_golden(gpu, golden, name):
    sp = [float(v) for v in golden[f"cal_{name}__meta"][2:]]
    assert bits_equal(run_bspline(gpu, golden[f"cal_{name}__in"], sp), golden[f"cal_{name}__out"])


@pytest.mark.parametrize("host", [False, True])
def test_slices_random(gpu, host):
    x = np.random.default_rng(61).standard_normal((20, 40, 52)).astype(np.float32)
    req = ((3, 5, 2), (44, 30, 15))
    index = (0, 0, 0)
    want = oracle.slice_by_slice(x, 2.0, (0.9, 1.2, 3.0), requested=req)
    got = run_slices(gpu, x, 2.0, (0.9, 1.2, 3.0), requested=req, host=host)
    assert bits_equal(got, want)
    got = run_slices(gpu, x, 2.0, (0.9, 1.2, 3.0), requested=req, rounding=1)
    assert normwise(got, want) <= 1e-5


def test_slices_u8(gpu):
    x = np.random.default_rng(62).integers(0, 256, (6, 30, 34), dtype=np.uint8)
    assert np.array_equal(run_slices(gpu, x, 1.4), oracle.slice_by_slice(x, 1.4))


@pytest.mark.parametrize("shape", [(33, 40, 47), (64, 64, 64), (21, 30)])
def test_bspline_random(gpu, shape):
    x = np.random.default_rng(63).standard_normal(shape).astype(np.float32)
    want = oracle.bspline_downsample(x)
    for host in (False, True):
        assert bits_equal(run_bspline(gpu, x, host=host), want)
    assert normwise(run_bspline(gpu, x, rounding=1), want) <= 1e-5


def test_bspline_u8(gpu):
    x = np.random.default_rng(64).integers(0, 256, (15, 17, 19), dtype=np.uint8)
    assert np.array_equal(run_bspline(gpu, x), oracle.bspline_downsample(x))


@pytest.mark.parametrize("which,kernel", [(1, "tile2d"), (2, "fused2d")])
def test_slices_take_the_fused_2d_kernels(gpu, which, kernel):
    from itkg import _abi
    x = np.random.default_rng(65).standard_normal((9, 33, 70)).astype(np.float32)
    _abi.lib().itkg_debug_set_2d_kernel(which)
    try:
        for rounding, suffix in ((0, "_f32_ref"), (1, "_f32_fma")):
            got = run_slices(gpu, x, 1.7, rounding=rounding)
            assert gpu.last_kernel() == kernel + suffix
            want = oracle.slice_by_slice(x, 1.7)
            assert bits_equal(got, want) if rounding == 0 else normwise(got, want) <= 1e-5
    finally:
        _abi.lib().itkg_debug_set_2d_kernel(0)



def run_dfb(itkg, field, sigma, requested=None, index=None, host=False, rounding=0):
    img = itkg.Image(field, index=index, components=2)
    src = img if host else itkg.DeviceImage.from_host(img)
    f = itkg.DisplacementFieldToBSplineFilter(src, sigma, rounding=rounding)
    req = itkg.Region(*requested) if requested else img.region
    out = f.generate_region(req)
    return out.data if host else out.download()


@pytest.mark.parametrize("name", ["dfbspline_s2", "dfbspline_sub_s1p5"])
def test_displacement_field_to_bspline_golden(gpu, golden, name):
    sigma, req = dfb_meta(golden, name)
    for host in (False, True):
        assert bits_equal(run_dfb(gpu, golden[f"cal_{name}__in"], sigma, requested=req, host=host),
                          golden[f"cal_{name}__out"])


@pytest.mark.parametrize("shape", [(64, 80), (300, 257), (1700, 2000)])
def test_displacement_field_to_bspline_random(gpu, shape):
    """VecPixel<f32, 2> through the 2-D tile kernel (small fields) or the
    per-axis passes (large ones), sub-regions clamped at the request."""
    f = np.random.default_rng(sum(shape)).standard_normal(shape + (2,)).astype(np.float32)
    index = (3, -2)
    req = ((3 + shape[1] // 5, -2 + shape[0] // 4), (shape[1] // 2, shape[0] // 2))
    for r in (None, req):
        want = oracle.displacement_field_to_bspline(f, 2.0, index=index, requested=r)
        got = run_dfb(gpu, f, 2.0, requested=r, index=index)
        assert bits_equal(got, want), (shape, r, gpu.last_kernel())
        got = run_dfb(gpu, f, 2.0, requested=r, index=index, rounding=1)
        assert normwise(got, want) <= 1e-5
