"""C-ABI checks that need no GPU: the library loads, exports every symbol
include/itkg.h declares, its host-side geometry matches the reference
restatement, and invalid calls fail with a status (never a crash)."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "itkg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(itkg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(itkg_lib):
    syms = header_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(itkg_lib, s)]
    assert not missing, missing


def test_python_binding_declares_every_symbol(itkg_lib):
    from itkg import _abi
    assert set(header_symbols()) == set(_abi.SIGNATURES)


def test_abi_version(itkg_lib):
    assert itkg_lib.itkg_abi_version() == 1


@pytest.mark.parametrize("sigma,spacing", [(1.5, 1.0), (2.0, 1.0), (1.5, 0.7), (1.5, 2.5),
                                           (0.5, 1.0), (4.0, 1.0), (8.0, 1.0), (1.0, 3.0),
                                           (-1.0, 1.0), (0.0, 1.0), (float("nan"), 1.0),
                                           (1.0, -1.0), (2.0 / 3.0, 1.0), (1e-9, 1.0)])
def test_kernel_radius_and_weights_match_oracle(itkg_lib, sigma, spacing):
    import itkg
    r = itkg.kernel_radius(sigma, spacing)
    assert r == oracle.kernel_radius(sigma, spacing)
    if r < 100:
        a = itkg.build_kernel(sigma / spacing, r)
        b = oracle.build_kernel(sigma / spacing, r)
        assert np.array_equal(np.isnan(a), np.isnan(b))
        assert np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])


def test_kernel_radius_saturates(itkg_lib):
    import itkg
    assert itkg.kernel_radius(float("inf"), 1.0) == 2**64 - 1
    assert itkg.kernel_radius(1.0, 0.0) == 2**64 - 1


def test_region_ops_reference_tests(itkg_lib):
    # image.rs:180-195
    import itkg
    r = itkg.Region((10, 20), (5, 8))
    c = r.to_c()
    radii = (ctypes.c_uint64 * 3)(2, 2, 0)
    out = itkg._abi.itkg_region()
    itkg.check = itkg._abi.check
    itkg._abi.check(itkg_lib.itkg_region_padded_per_axis(ctypes.byref(c), 2, radii, ctypes.byref(out)))
    assert itkg.Region.from_c(out, 2) == itkg.Region((8, 18), (9, 12))
    b = itkg.Region((0, 0), (10, 10)).to_c()
    q = itkg.Region((-2, 3), (8, 10)).to_c()
    itkg._abi.check(itkg_lib.itkg_region_clipped_to(ctypes.byref(q), 2, ctypes.byref(b), ctypes.byref(out)))
    assert itkg.Region.from_c(out, 2) == itkg.Region((0, 3), (6, 7))


@pytest.mark.parametrize("index,size,n", [((0, 0), (4, 6), 3), ((0, 0), (4, 7), 3),
                                          ((0, 0), (4, 2), 10), ((5,), (10,), 4),
                                          ((0, 0, 0), (256, 256, 256), 8),
                                          ((3, -2, 7), (9, 5, 13), 4), ((0, 0), (4, 0), 3),
                                          ((0, 0, 0), (5, 5, 5), 0)])
def test_split_region_matches_oracle(itkg_lib, index, size, n):
    import itkg
    got = [(p.index, p.size) for p in itkg.split_region(itkg.Region(index, size), n)]
    want = oracle.split_region(index, size, n)
    assert got == want


def test_input_region_for_output(itkg_lib):
    import itkg
    img = itkg.Image(np.zeros((30, 40, 50), np.float32), spacing=(0.7, 0.7, 2.5))
    f = itkg.GaussianFilter(img, 1.5)
    req = itkg.Region((10, 0, 20), (5, 40, 10))
    got = f.input_region_for_output(req)
    # radii (7, 7, 2); z is clipped at the largest region's end (30)
    assert got == itkg.Region((3, 0, 18), (19, 40, 12))
    c = req.to_c()
    lg = img.region.to_c()
    sp = (ctypes.c_double * 3)(0.7, 0.7, 2.5)
    out = itkg._abi.itkg_region()
    itkg._abi.check(itkg_lib.itkg_gaussian_input_region_for_output(
        ctypes.byref(c), ctypes.byref(lg), 3, sp, 1.5, ctypes.byref(out)))
    assert itkg.Region.from_c(out, 3) == got


def _call(itkg_lib, inp, largest, req, prm, out):
    return itkg_lib.itkg_gaussian_generate_region(
        ctypes.byref(inp) if inp is not None else None,
        ctypes.byref(largest) if largest is not None else None,
        ctypes.byref(req) if req is not None else None,
        ctypes.byref(prm) if prm is not None else None,
        ctypes.byref(out) if out is not None else None, None)


def _host_pair():
    import itkg
    a = itkg.Image(np.zeros((6, 7, 8), np.float32))
    b = itkg.Image(np.zeros((6, 7, 8), np.float32))
    p = itkg._abi.itkg_gaussian_params()
    p.sigma = 1.0
    return a, b, p


def test_invalid_arguments_return_status(itkg_lib):
    import itkg
    E = itkg._abi.ERROR_INVALID_ARGUMENT
    a, b, p = _host_pair()
    ac, bc = a.to_c(), b.to_c()
    lg, rq = a.region.to_c(), a.region.to_c()
    assert _call(itkg_lib, None, lg, rq, p, bc) == E
    assert _call(itkg_lib, ac, lg, rq, None, bc) == E
    assert _call(itkg_lib, ac, None, rq, p, bc) == E
    bad = a.to_c()
    bad.dim = 4
    assert _call(itkg_lib, bad, lg, rq, p, bc) == E
    bad = a.to_c()
    bad.pitch[0] = 8
    assert _call(itkg_lib, bad, lg, rq, p, bc) == E
    bad = a.to_c()
    bad.dtype = 17
    assert _call(itkg_lib, bad, lg, rq, p, bc) == E
    p2 = itkg._abi.itkg_gaussian_params()
    p2.sigma = 1.0
    p2.rounding = 9
    assert _call(itkg_lib, ac, lg, rq, p2, bc) == E
    p2.rounding = 0
    p2.reserved = 1
    assert _call(itkg_lib, ac, lg, rq, p2, bc) == E
    # requested outside the largest region
    out_req = itkg.Region((5, 0, 0), (8, 7, 6)).to_c()
    assert _call(itkg_lib, ac, lg, out_req, p, bc) == E
    # input buffer does not cover input_region_for_output(requested)
    small = itkg.Image(np.zeros((6, 7, 4), np.float32)).to_c()
    assert _call(itkg_lib, small, lg, rq, p, bc) == E
    assert "input_region_for_output" in itkg_lib.itkg_last_error().decode()
    # absurd radius (the reference would fail to allocate)
    p3 = itkg._abi.itkg_gaussian_params()
    p3.sigma = 1e12
    assert _call(itkg_lib, ac, lg, rq, p3, bc) == E
    # u8 pixel arithmetic with an f32 input
    p4 = itkg._abi.itkg_gaussian_params()
    p4.sigma = 1.0
    p4.arithmetic = itkg.ARITH_PIXEL_U8
    assert _call(itkg_lib, ac, lg, rq, p4, bc) == E


def test_unsupported_combinations_return_status(itkg_lib):
    import itkg
    a, b, p = _host_pair()
    bc = b.to_c()
    bc.dtype = itkg.I16
    bc.pitch[0], bc.pitch[1], bc.pitch[2] = 2, 16, 112
    assert _call(itkg_lib, a.to_c(), a.region.to_c(), a.region.to_c(), p, bc) == itkg._abi.ERROR_UNSUPPORTED


def test_empty_request_is_a_noop(itkg_lib):
    import itkg
    a, b, p = _host_pair()
    empty = itkg.Region((0, 0, 0), (8, 0, 6)).to_c()
    assert _call(itkg_lib, a.to_c(), a.region.to_c(), empty, p, b.to_c()) == 0


def test_valid_call_without_gpu_reports_no_device(itkg_lib):
    import itkg
    if itkg.device_count() > 0:
        pytest.skip("a GPU is present")
    a, b, p = _host_pair()
    st = _call(itkg_lib, a.to_c(), a.region.to_c(), a.region.to_c(), p, b.to_c())
    assert st in (itkg._abi.ERROR_NO_DEVICE, itkg._abi.ERROR_CUDA)
    assert itkg_lib.itkg_last_error().decode() != ""


@pytest.mark.parametrize("sigma", [0.1, 0.5, 1.3, 2.5, 7.0, float("nan")])
def test_yvv_coefficients_match_oracle(itkg_lib, sigma):
    """The library's Young & van Vliet coefficients (recursive_gaussian.rs:33-49) are the oracle's, bit for bit."""
    import itkg
    assert np.array_equal(itkg.yvv_coeffs(sigma), oracle.yvv_coeffs(sigma))


def _sep_params(radius=(1, 1, 1), reps=1, kernels=None):
    import itkg
    ks = kernels if kernels is not None else [itkg.box_kernel(r) for r in radius]
    p = itkg._abi.itkg_separable_params()
    for d, k in enumerate(ks):
        p.radius[d] = (len(k) - 1) // 2
        p.weights[d] = k.ctypes.data
    p.repetitions = reps
    return p, ks


def test_separable_invalid_arguments_return_status(itkg_lib):
    import itkg
    E = itkg._abi.ERROR_INVALID_ARGUMENT
    a, b, _ = _host_pair()
    ac, bc = a.to_c(), b.to_c()
    lg, rq = a.region.to_c(), a.region.to_c()

    def call(p):
        return itkg_lib.itkg_separable_generate_region(ctypes.byref(ac), ctypes.byref(lg), ctypes.byref(rq),
                                                       ctypes.byref(p) if p is not None else None,
                                                       ctypes.byref(bc), None)
    assert call(None) == E
    p, ks = _sep_params()
    p.weights[1] = None
    assert call(p) == E
    p, ks = _sep_params()
    p.radius[0] = 1 << 21
    assert call(p) == E
    p, ks = _sep_params(reps=1 << 21)
    assert call(p) == E
    p, ks = _sep_params()
    p.rounding = 7
    assert call(p) == E
    # input buffer smaller than requested padded by radius x repetitions
    p, ks = _sep_params(reps=3)
    small = itkg.Image(np.zeros((6, 7, 4), np.float32)).to_c()
    rq2 = itkg.Region((0, 0, 0), (4, 7, 6)).to_c()
    st = itkg_lib.itkg_separable_generate_region(ctypes.byref(small), ctypes.byref(lg), ctypes.byref(rq2),
                                                 ctypes.byref(p), ctypes.byref(bc), None)
    assert st == E and "input_region_for_output" in itkg_lib.itkg_last_error().decode()


def test_separable_input_region_and_box_kernel(itkg_lib):
    import itkg
    r = itkg.Region((10, 4, 2), (5, 6, 7)).to_c()
    lg = itkg.Region((0, 0, 0), (40, 30, 20)).to_c()
    out = itkg._abi.itkg_region()
    radius = (ctypes.c_uint64 * 3)(1, 2, 3)
    itkg._abi.check(itkg_lib.itkg_separable_input_region_for_output(ctypes.byref(r), ctypes.byref(lg), 3, radius, 2,
                                                                    ctypes.byref(out)))
    assert itkg.Region.from_c(out, 3) == itkg.Region((8, 0, 0), (9, 14, 15))  # z: [2 - 6, 8 + 6] clipped
    assert np.array_equal(itkg.box_kernel(3), oracle.box_kernel(3))


def test_recursive_invalid_arguments_return_status(itkg_lib):
    import itkg
    E = itkg._abi.ERROR_INVALID_ARGUMENT
    a, b, _ = _host_pair()
    ac, bc = a.to_c(), b.to_c()
    lg, rq = a.region.to_c(), a.region.to_c()

    def call(p, inp=ac, out=bc, req=rq):
        return itkg_lib.itkg_recursive_gaussian_generate_region(
            ctypes.byref(inp), ctypes.byref(lg), ctypes.byref(req), ctypes.byref(p) if p is not None else None,
            ctypes.byref(out), None)
    assert call(None) == E
    p = itkg._abi.itkg_recursive_params()
    p.sigma = 2.0
    p.axis = 3
    assert call(p) == E
    p.axis = -2
    assert call(p) == E
    p.axis, p.rounding = -1, 5
    assert call(p) == E
    p.rounding = 0
    p.reserved[1] = 1
    assert call(p) == E
    p.reserved[1] = 0
    # the input must cover the whole largest region
    small = itkg.Image(np.zeros((6, 7, 4), np.float32)).to_c()
    assert call(p, inp=small) == E and "largest" in itkg_lib.itkg_last_error().decode()
    # i16 output is not a NumericPixel of the recursive filter
    bad = b.to_c()
    bad.dtype = itkg.I16
    bad.pitch[0], bad.pitch[1], bad.pitch[2] = 2, 16, 112
    assert call(p, out=bad) == itkg._abi.ERROR_UNSUPPORTED
    empty = itkg.Region((0, 0, 0), (8, 0, 6)).to_c()
    assert call(p, req=empty) == 0


@pytest.mark.parametrize("sigma", [0.2, 1.0, 1.3, 3.7, 6.0])
def test_unsharp_kernel_matches_oracle(itkg_lib, sigma):
    import itkg
    assert np.array_equal(itkg.unsharp_kernel(sigma), oracle.unsharp_kernel(sigma))


def test_unsharp_invalid_arguments_return_status(itkg_lib):
    import itkg
    E = itkg._abi.ERROR_INVALID_ARGUMENT
    a, b, _ = _host_pair()
    ac, bc = a.to_c(), b.to_c()
    lg, rq = a.region.to_c(), a.region.to_c()

    def call(p, inp=ac, out=bc, req=rq):
        return itkg_lib.itkg_unsharp_mask_generate_region(
            ctypes.byref(inp), ctypes.byref(lg), ctypes.byref(req), ctypes.byref(p) if p is not None else None,
            ctypes.byref(out), None)
    assert call(None) == E
    p = itkg._abi.itkg_unsharp_params()
    p.sigma, p.amount = 0.0, 0.5
    assert call(p) == E and "sigma" in itkg_lib.itkg_last_error().decode()
    p.sigma = float("nan")
    assert call(p) == E
    p.sigma, p.rounding = 1.0, 4
    assert call(p) == E
    p.rounding, p.reserved = 0, 1
    assert call(p) == E
    p.reserved = 0
    # output dtype must be the input's
    bad = itkg.Image(np.zeros((6, 7, 8), np.uint8)).to_c()
    assert call(p, out=bad) == E
    # the input must cover the padded request
    small = itkg.Image(np.zeros((6, 7, 4), np.float32)).to_c()
    assert call(p, inp=small) == E and "input_region_for_output" in itkg_lib.itkg_last_error().decode()
    empty = itkg.Region((0, 0, 0), (8, 0, 6)).to_c()
    assert call(p, req=empty) == 0
    r = ctypes.c_uint64()
    w = np.zeros(3)
    assert itkg_lib.itkg_unsharp_kernel(1.0, ctypes.byref(r), w.ctypes.data, 3) == E  # 7 weights needed
    assert r.value == 3


def test_callers_invalid_arguments_return_status(itkg_lib):
    import itkg
    E = itkg._abi.ERROR_INVALID_ARGUMENT
    a, b, p = _host_pair()
    ac, bc = a.to_c(), b.to_c()
    rq = a.region.to_c()
    # SliceBySliceFilter: 3-D only, the input must contain the request
    assert itkg_lib.itkg_slice_by_slice_generate_region(ctypes.byref(ac), ctypes.byref(rq), None,
                                                        ctypes.byref(bc), None) == E
    img2 = itkg.Image(np.zeros((5, 6), np.float32)).to_c()
    rq2 = itkg.Region((0, 0), (6, 5)).to_c()
    assert itkg_lib.itkg_slice_by_slice_generate_region(ctypes.byref(img2), ctypes.byref(rq2), ctypes.byref(p),
                                                        ctypes.byref(img2), None) == itkg._abi.ERROR_UNSUPPORTED
    big = itkg.Region((0, 0, 0), (8, 7, 9)).to_c()
    assert itkg_lib.itkg_slice_by_slice_generate_region(ctypes.byref(ac), ctypes.byref(big), ctypes.byref(p),
                                                        ctypes.byref(bc), None) == E
    # BSplineDownsampleFilter: the output must hold the downsampled largest region
    lg = a.region.to_c()
    small = itkg.Image(np.zeros((2, 2, 2), np.float32)).to_c()
    assert itkg_lib.itkg_bspline_downsample_generate_region(ctypes.byref(ac), ctypes.byref(lg), ctypes.byref(p),
                                                            ctypes.byref(small), None) == E
    assert "downsampled" in itkg_lib.itkg_last_error().decode()
    half = itkg.Image(np.zeros((3, 4, 4), np.float32)).to_c()
    assert itkg_lib.itkg_bspline_downsample_generate_region(ctypes.byref(small), ctypes.byref(lg), ctypes.byref(p),
                                                            ctypes.byref(half), None) == E
