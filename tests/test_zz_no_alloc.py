"""The no-allocation entry point, itkg_gaussian_generate_region_noalloc.

Some callers cannot allocate device memory while they run -- an application
that has already given all device memory to its own pool, or a latency-bound
loop that cannot pay for an allocation.  For them the library offers a variant
of the per-axis Gaussian whose intermediates live in a fixed device array
inside the library.  These tests call it through the C ABI and check it
against the regular entry point (per-axis algorithm, reference rounding, so
the results must be bit-identical), twice in a row so the second call runs on
whatever the first left in the shared array, check through the library's
scratch-allocation counter that the calls allocate nothing (f32 and u8 pixel
arithmetic, one to three dimensions), and check that a request too large for
the array is refused.

The file is named to be collected last: it runs after every other test, and
passes alone in a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _images(itkg, arr, comps=1, spacing=None, dtype_code=None):
    host = itkg.Image(arr, spacing=spacing, components=comps)
    src = itkg.DeviceImage.from_host(host)
    return host, src


def _call(itkg, fn, src, largest, requested, prm, out):
    from itkg import _abi
    lg = largest.to_c()
    rq = requested.to_c()
    return fn(ctypes.byref(src.c), ctypes.byref(lg), ctypes.byref(rq), ctypes.byref(prm),
              ctypes.byref(out.c), None)


def _params(itkg, sigma, arithmetic=0):
    from itkg import _abi
    p = _abi.itkg_gaussian_params()
    p.sigma = sigma
    p.arithmetic = arithmetic
    p.rounding = itkg.ROUND_REFERENCE
    p.algorithm = itkg.ALGO_PER_AXIS
    return p


@pytest.mark.parametrize("shape,comps,sigma,spacing,req", [
    ((40, 50, 60), 1, 2.0, None, None),
    ((17, 33, 29), 1, 1.3, (0.7, 0.9, 2.5), ((3, 4, 2), (20, 25, 12))),
    ((64, 80), 3, 1.5, None, None),
    ((300,), 1, 2.5, None, None),
])
def test_noalloc_matches_generate_region_twice(gpu, shape, comps, sigma, spacing, req):
    from itkg import _abi
    L = _abi.lib()
    rng = np.random.default_rng(sum(shape) + comps)
    arr = rng.standard_normal(shape + ((comps,) if comps > 1 else ())).astype(np.float32)
    host, src = _images(gpu, arr, comps, spacing)
    largest = host.region
    requested = gpu.Region(*req) if req else largest
    prm = _params(gpu, sigma)
    want_img = gpu.DeviceImage(requested, gpu.F32, comps, host.spacing)
    _abi.check(_call(gpu, L.itkg_gaussian_generate_region, src, largest, requested, prm, want_img))
    want = want_img.download()
    for attempt in range(2):
        got_img = gpu.DeviceImage(requested, gpu.F32, comps, host.spacing)
        _abi.check(_call(gpu, L.itkg_gaussian_generate_region_noalloc, src, largest, requested,
                         prm, got_img))
        got = got_img.download()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), attempt


def test_noalloc_u8_pixel_arithmetic_twice(gpu):
    from itkg import _abi
    L = _abi.lib()
    rng = np.random.default_rng(5)
    arr = rng.integers(0, 256, (30, 41)).astype(np.uint8)
    host, src = _images(gpu, arr)
    prm = _params(gpu, 1.5, arithmetic=gpu.ARITH_PIXEL_U8)
    want_img = gpu.DeviceImage(host.region, gpu.U8)
    _abi.check(_call(gpu, L.itkg_gaussian_generate_region, src, host.region, host.region, prm,
                     want_img))
    want = want_img.download()
    for attempt in range(2):
        got_img = gpu.DeviceImage(host.region, gpu.U8)
        _abi.check(_call(gpu, L.itkg_gaussian_generate_region_noalloc, src, host.region,
                         host.region, prm, got_img))
        assert np.array_equal(got_img.download(), want), attempt


@pytest.mark.parametrize("shape", [(300,), (30, 41), (19, 23, 31)])
def test_noalloc_u8_pixel_arithmetic_each_dimension(gpu, shape):
    from itkg import _abi
    L = _abi.lib()
    rng = np.random.default_rng(len(shape))
    arr = rng.integers(0, 256, shape).astype(np.uint8)
    host, src = _images(gpu, arr)
    prm = _params(gpu, 1.2, arithmetic=gpu.ARITH_PIXEL_U8)
    want_img = gpu.DeviceImage(host.region, gpu.U8)
    _abi.check(_call(gpu, L.itkg_gaussian_generate_region, src, host.region, host.region, prm,
                     want_img))
    want = want_img.download()
    got_img = gpu.DeviceImage(host.region, gpu.U8)
    _abi.check(_call(gpu, L.itkg_gaussian_generate_region_noalloc, src, host.region,
                     host.region, prm, got_img))
    assert np.array_equal(got_img.download(), want)


@pytest.mark.parametrize("u8", [False, True])
@pytest.mark.parametrize("shape", [(300,), (30, 41), (19, 23, 31)])
def test_noalloc_makes_no_scratch_allocation(gpu, shape, u8):
    """The library counts every device scratch allocation its calls make; the
    regular entry point makes some (its intermediates, the u8 per-tap table),
    the no-allocation entry point none, on the f32 and the u8 path alike."""
    from itkg import _abi
    L = _abi.lib()
    rng = np.random.default_rng(7)
    if u8:
        arr = rng.integers(0, 256, shape).astype(np.uint8)
        prm = _params(gpu, 1.4, arithmetic=gpu.ARITH_PIXEL_U8)
        dt = gpu.U8
    else:
        arr = rng.standard_normal(shape).astype(np.float32)
        prm = _params(gpu, 1.4)
        dt = gpu.F32
    host, src = _images(gpu, arr)
    out_a = gpu.DeviceImage(host.region, dt)
    out_b = gpu.DeviceImage(host.region, dt)
    n0 = L.itkg_scratch_alloc_counter()
    _abi.check(_call(gpu, L.itkg_gaussian_generate_region, src, host.region, host.region, prm, out_a))
    n1 = L.itkg_scratch_alloc_counter()
    if u8 or len(shape) > 1:
        assert n1 > n0  # the counter sees the regular path's allocations
    for _ in range(2):
        _abi.check(_call(gpu, L.itkg_gaussian_generate_region_noalloc, src, host.region,
                         host.region, prm, out_b))
    assert L.itkg_scratch_alloc_counter() == n1
    got, want = out_b.download(), out_a.download()
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))


def test_noalloc_rejects_requests_beyond_its_scratch(gpu):
    from itkg import _abi
    L = _abi.lib()
    # 256 x 256 x 200 f32 with sigma 2: the first intermediate alone is ~66 MiB
    region = gpu.Region((0, 0, 0), (256, 256, 200))
    src = gpu.DeviceImage(region)
    out = gpu.DeviceImage(region)
    prm = _params(gpu, 2.0)
    st = _call(gpu, L.itkg_gaussian_generate_region_noalloc, src, region, region, prm, out)
    assert st == _abi.ERROR_INVALID_ARGUMENT
    assert "scratch" in L.itkg_last_error().decode()


def test_noalloc_rejects_host_buffers(gpu):
    from itkg import _abi
    L = _abi.lib()
    arr = np.zeros((8, 9, 10), np.float32)
    host = gpu.Image(arr)
    hc = host.to_c()
    out = gpu.Image(np.zeros_like(arr)).to_c()
    lg = host.region.to_c()
    prm = _params(gpu, 1.0)
    st = L.itkg_gaussian_generate_region_noalloc(ctypes.byref(hc), ctypes.byref(lg),
                                                 ctypes.byref(lg), ctypes.byref(prm),
                                                 ctypes.byref(out), None)
    assert st == _abi.ERROR_INVALID_ARGUMENT
