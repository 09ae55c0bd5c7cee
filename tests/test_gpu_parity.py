"""GPU parity through the C ABI: every result is compared with the oracle on the
same seeded inputs.  Reference rounding must be bit-exact; FMA rounding must be
within 1e-5 normwise relative (max|gpu-ref| / max|ref|), the tolerance the
path is specified to; bf16/f16 storage is checked against the FP64 oracle
within the storage type's half-ulp bound."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

CASES = ["impulse2d_s1p5", "impulse3d_s1", "vecpixel2d_s1", "rand2d_s1p5", "rand2d_sub_s1p5",
         "rand3d_s1p2", "rand3d_aniso", "rand3d_sub_s2", "tiny2d_s3", "line1d_s2"]
ALGOS = ["auto", "per_axis"]


def _algo(itkg, name):
    return {"auto": itkg.ALGO_AUTO, "per_axis": itkg.ALGO_PER_AXIS, "fused": itkg.ALGO_FUSED,
            "two_pass": itkg.ALGO_TWO_PASS}[name]


def bits_equal(a, b):
    """Bit-exact equality; NaNs compare equal to NaNs whatever their payload
    (x86 and the GPU produce different NaN bit patterns for the same invalid
    operation, and the reference attaches no meaning to them)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    return np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32))


def normwise(a, ref):
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.abs(np.asarray(a, np.float64) - ref).max() / max(np.abs(ref).max(), 1e-300))


def run_device(itkg, arr, sigma, spacing=None, comps=1, requested=None, rounding=0, algo="auto",
               out_dtype=None, index=None, cast=False, arithmetic=None):
    """Upload, run generate_region on device buffers, download."""
    img = itkg.Image(arr, index=index, spacing=spacing, components=comps)
    dev = itkg.DeviceImage.from_host(img)
    src = itkg.CastFilter(dev, itkg.F32) if cast else dev
    f = itkg.GaussianFilter(src, sigma, rounding=rounding, algorithm=_algo(itkg, algo),
                            arithmetic=arithmetic)
    req = itkg.Region(*requested) if requested else img.region
    out = f.generate_region(req, out_dtype=out_dtype)
    return out.download()


def meta(golden, name):
    m = golden[f"{name}__meta"]
    D = (len(m) - 2) // 3
    return (float(m[0]), [float(v) for v in m[1:1 + D]], int(m[1 + D]),
            tuple(int(v) for v in m[2 + D:2 + 2 * D]), tuple(int(v) for v in m[2 + 2 * D:]))


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("name", CASES)
def test_golden_bit_exact(gpu, golden, name, algo):
    sigma, spacing, comps, ri, rs = meta(golden, name)
    got = run_device(gpu, golden[f"{name}__in"], sigma, spacing, comps, (ri, rs), algo=algo)
    assert bits_equal(got, golden[f"{name}__out"]), gpu.last_kernel()


@pytest.mark.parametrize("name", ["u8pixel2d_s1p5", "u8pixel2d_wrap_s1"])
def test_golden_u8_pixel_arithmetic(gpu, golden, name):
    sigma, spacing, comps, ri, rs = meta(golden, name)
    got = run_device(gpu, golden[f"{name}__in"], sigma, spacing, comps, (ri, rs),
                     arithmetic=gpu.ARITH_PIXEL_U8, out_dtype=gpu.U8)
    assert np.array_equal(got, golden[f"{name}__out"])


def test_golden_i16_cast(gpu, golden):
    name = "i16cast3d_s1p5"
    sigma, spacing, comps, ri, rs = meta(golden, name)
    got = run_device(gpu, golden[f"{name}__in"], sigma, spacing, comps, (ri, rs), cast=True)
    assert bits_equal(got, golden[f"{name}__out"])


def test_golden_stream_full(gpu, golden):
    x = np.zeros((20, 20), np.float32)
    x[10, 10] = 1.0
    dev = gpu.DeviceImage.from_host(gpu.Image(x))
    out = gpu.stream_full(gpu.GaussianFilter(dev, 1.5), 4).download()
    assert bits_equal(out, golden["stream4_impulse2d__out"])


SHAPES = [
    ((7,), 1, 0.8), ((300,), 1, 2.5), ((33, 45), 1, 1.5), ((64, 64), 3, 1.2), ((5, 3), 1, 4.0),
    ((9, 17, 31), 1, 1.0), ((16, 16, 16), 1, 2.0), ((21, 13, 40), 3, 1.1), ((1, 1, 1), 1, 1.0),
    ((2, 50, 3), 1, 2.2), ((40, 1, 40), 1, 1.5), ((12, 30, 70), 1, 3.3),
]


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("shape,comps,sigma", SHAPES)
def test_random_shapes_reference_rounding(gpu, shape, comps, sigma, algo):
    rng = np.random.default_rng(hash((shape, comps)) % 2**32)
    arr = rng.standard_normal(shape + ((comps,) if comps > 1 else ())).astype(np.float32)
    want = oracle.gaussian_f32(arr, sigma, comps=comps)
    got = run_device(gpu, arr, sigma, comps=comps, algo=algo)
    assert bits_equal(got, want), gpu.last_kernel()


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("shape,comps,sigma", SHAPES)
def test_random_shapes_fma_within_1e5(gpu, shape, comps, sigma, algo):
    rng = np.random.default_rng(1 + hash((shape, comps)) % 2**32)
    arr = rng.random(shape + ((comps,) if comps > 1 else ()), dtype=np.float32)
    want = oracle.gaussian_f32(arr, sigma, comps=comps)
    got = run_device(gpu, arr, sigma, comps=comps, algo=algo, rounding=gpu.ROUND_FMA)
    assert normwise(got, want) <= 1e-5


@pytest.mark.parametrize("algo", ALGOS)
def test_subregions_with_offset_index(gpu, algo):
    rng = np.random.default_rng(7)
    arr = rng.random((23, 29, 31), dtype=np.float32)
    index = (5, -3, 100)
    spacing = (0.9, 1.1, 1.7)
    for ri, rs in [((5, -3, 100), (31, 29, 23)), ((9, 0, 104), (20, 11, 9)),
                   ((30, 20, 121), (6, 6, 2)), ((5, -3, 100), (1, 1, 1))]:
        want = oracle.gaussian_f32(arr, 2.1, spacing=spacing, index=index, requested=(ri, rs))
        got = run_device(gpu, arr, 2.1, spacing=spacing, index=index, requested=(ri, rs), algo=algo)
        assert bits_equal(got, want), (ri, rs, gpu.last_kernel())


@pytest.mark.parametrize("algo", ALGOS)
def test_stream_full_equals_full_3d(gpu, algo):
    rng = np.random.default_rng(8)
    arr = rng.random((37, 20, 24), dtype=np.float32)
    dev = gpu.DeviceImage.from_host(gpu.Image(arr))
    f = gpu.GaussianFilter(dev, 2.0, algorithm=_algo(gpu, algo))
    full = f.generate_region(dev.region).download()
    for n in (1, 3, 8, 100):
        piece = gpu.stream_full(f, n).download()
        assert bits_equal(piece, full)
    assert bits_equal(full, oracle.gaussian_f32(arr, 2.0))


def test_sigma_edge_cases(gpu):
    arr = (np.arange(30, dtype=np.float32).reshape(5, 6) - 10.0)
    assert bits_equal(run_device(gpu, arr, -2.0), oracle.gaussian_f32(arr, -2.0))
    assert np.isnan(run_device(gpu, arr, 0.0)).all()
    assert np.isnan(run_device(gpu, arr, float("nan"))).all() == np.isnan(oracle.gaussian_f32(arr, float("nan"))).all()


def test_nonfinite_inputs_propagate_like_reference(gpu):
    rng = np.random.default_rng(9)
    arr = rng.random((12, 15, 11), dtype=np.float32)
    arr[3, 4, 5] = np.inf
    arr[8, 1, 2] = np.nan
    arr[0, 0, 0] = -0.0
    want = oracle.gaussian_f32(arr, 1.3)
    got = run_device(gpu, arr, 1.3)
    assert bits_equal(got, want)


@pytest.mark.parametrize("in_dtype", [np.int16, np.uint8])
def test_cast_inputs_bit_exact(gpu, in_dtype):
    rng = np.random.default_rng(10)
    if in_dtype == np.int16:
        arr = rng.integers(-1000, 1500, (10, 24, 20)).astype(np.int16)
    else:
        arr = rng.integers(0, 256, (10, 24, 20)).astype(np.uint8)
    want = oracle.gaussian_f32(arr.astype(np.float32), 1.5, spacing=(0.7, 0.7, 2.5))
    got = run_device(gpu, arr, 1.5, spacing=(0.7, 0.7, 2.5), cast=True)
    assert bits_equal(got, want)


def test_u8_output_round_clamp(gpu):
    rng = np.random.default_rng(12)
    arr = rng.integers(0, 256, (30, 40)).astype(np.uint8)
    f32 = oracle.gaussian_f32(arr.astype(np.float32), 2.0)
    want = oracle.cast_f32_to_u8(f32)
    got = run_device(gpu, arr, 2.0, cast=True, out_dtype=gpu.U8)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("out", ["bf16", "f16"])
def test_half_storage_outputs(gpu, out):
    rng = np.random.default_rng(13)
    arr = rng.integers(-1000, 1500, (12, 40, 36)).astype(np.int16)
    ref64 = oracle.gaussian_f64(arr.astype(np.float64), 1.5, spacing=(0.7, 0.7, 2.5))
    code = gpu.BF16 if out == "bf16" else gpu.F16
    raw = run_device(gpu, arr, 1.5, spacing=(0.7, 0.7, 2.5), cast=True, out_dtype=code,
                     rounding=gpu.ROUND_FMA)
    if out == "bf16":
        got = (raw.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
        half_ulp_rel = 2.0 ** -8   # 8 significand bits: half an ulp <= 2^-8 |v|
    else:
        got = raw.astype(np.float64)
        half_ulp_rel = 2.0 ** -11  # 11 significand bits
    # storage rounding: |err| <= half an ulp of the value (plus f32 arithmetic noise)
    err = np.abs(got - ref64)
    assert (err <= np.abs(ref64) * half_ulp_rel * 1.0001 + 1e-4).all()
    ulp_rel = 2.0 * half_ulp_rel
    # bf16 output equals rounding the f32 result to nearest-even
    f32 = oracle.gaussian_f32(arr.astype(np.float32), 1.5, spacing=(0.7, 0.7, 2.5))
    assert normwise(got, f32) <= ulp_rel


def _f32_to_bf16_bits(v):
    """Round f32 to bf16 to nearest, ties to even (finite values), as bits."""
    b = np.ascontiguousarray(v, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((b + 0x7FFF + ((b >> 16) & 1)) >> 16).astype(np.uint16)


@pytest.mark.parametrize("out", ["bf16", "f16"])
@pytest.mark.parametrize("shape,req", [((14, 40, 64), None),                          # whole quads: 8-byte stores
                                        ((14, 40, 66), None),                          # ragged width: element stores
                                        ((20, 45, 72), ((4, 3, 2), (36, 30, 15)))])    # sub-region, whole quads
@pytest.mark.parametrize("algo", ["two_pass", "auto"])
def test_half_storage_bit_exact_in_reference_rounding(gpu, out, shape, req, algo):
    """In reference rounding the bf16 / f16 output is the reference's f32
    result rounded to nearest-even, bit for bit, whichever store the z pass
    takes (one 8-byte store per quad, or element by element)."""
    arr = np.random.default_rng(15).standard_normal(shape).astype(np.float32) * 40
    code = gpu.BF16 if out == "bf16" else gpu.F16
    raw = run_device(gpu, arr, 1.6, requested=req, out_dtype=code, algo=algo)
    assert gpu.last_kernel().startswith("z_pass"), gpu.last_kernel()
    want32 = oracle.gaussian_f32(arr, 1.6, requested=req)
    want = _f32_to_bf16_bits(want32) if out == "bf16" else want32.astype(np.float16).view(np.uint16)
    assert np.array_equal(np.asarray(raw).view(np.uint16), want)


def test_host_buffers_through_abi(gpu):
    rng = np.random.default_rng(14)
    arr = rng.random((18, 22, 26), dtype=np.float32)
    img = gpu.Image(arr)
    f = gpu.GaussianFilter(img, 1.7)
    got = f.generate_region(gpu.Region((2, 3, 4), (20, 15, 10))).data
    want = oracle.gaussian_f32(arr, 1.7, requested=((2, 3, 4), (20, 15, 10)))
    assert bits_equal(got, want)
    got = gpu.stream_full(f, 5).data
    assert bits_equal(got, oracle.gaussian_f32(arr, 1.7))


def test_large_radius_per_axis(gpu):
    rng = np.random.default_rng(15)
    arr = rng.random((30, 40, 50), dtype=np.float32)
    want = oracle.gaussian_f32(arr, 8.0)
    got = run_device(gpu, arr, 8.0)
    assert bits_equal(got, want)


FUSED_CASES = [((9, 17, 31), 1.0, None), ((16, 16, 16), 2.0, None), ((40, 50, 70), 2.0, None),
               ((5, 70, 40), 2.2, None), ((12, 30, 70), 2.6, None), ((1, 1, 1), 1.0, None),
               ((33, 65, 97), 1.5, None), ((20, 20, 20), 0.3, None), ((3, 40, 33), 1.2, None),
               ((24, 48, 40), 1.5, (0.7, 0.7, 2.5))]


@pytest.mark.parametrize("shape,sigma,spacing", FUSED_CASES)
def test_fused3d_reference_rounding_bit_exact(gpu, shape, sigma, spacing):
    rng = np.random.default_rng(sum(shape))
    arr = rng.standard_normal(shape).astype(np.float32)
    want = oracle.gaussian_f32(arr, sigma, spacing=spacing)
    got = run_device(gpu, arr, sigma, spacing=spacing, algo="fused")
    assert gpu.last_kernel().startswith("fused3d"), gpu.last_kernel()
    assert bits_equal(got, want)


@pytest.mark.parametrize("shape,sigma,spacing", FUSED_CASES)
def test_fused3d_fma_within_1e5(gpu, shape, sigma, spacing):
    rng = np.random.default_rng(1 + sum(shape))
    arr = rng.random(shape, dtype=np.float32)
    want = oracle.gaussian_f32(arr, sigma, spacing=spacing)
    got = run_device(gpu, arr, sigma, spacing=spacing, algo="fused", rounding=gpu.ROUND_FMA)
    assert gpu.last_kernel().startswith("fused3d"), gpu.last_kernel()
    assert normwise(got, want) <= 1e-5


def test_fused3d_subregions_and_tight_buffers(gpu):
    # requested sub-regions; the input buffer is exactly input_region_for_output
    rng = np.random.default_rng(21)
    full = rng.random((30, 41, 53), dtype=np.float32)
    for ri, rs in [((7, 5, 4), (33, 20, 11)), ((0, 0, 0), (53, 41, 30)), ((50, 40, 29), (3, 1, 1)),
                   ((10, 0, 12), (1, 41, 6))]:
        want = oracle.gaussian_f32(full, 1.9, requested=(ri, rs))
        img = gpu.Image(full)
        f = gpu.GaussianFilter(img, 1.9)
        need = f.input_region_for_output(gpu.Region(ri, rs))
        (x0, y0, z0), (sx, sy, sz) = need.index, need.size
        sub = np.ascontiguousarray(full[z0:z0 + sz, y0:y0 + sy, x0:x0 + sx])
        dev = gpu.DeviceImage(need)
        dev.upload(sub)
        fd = gpu.GaussianFilter(dev, 1.9, algorithm=gpu.ALGO_FUSED)
        # the tight buffer's largest region is still the full image
        from itkg import _abi
        import ctypes
        out = gpu.DeviceImage(gpu.Region(ri, rs))
        lg = img.region.to_c()
        rq = gpu.Region(ri, rs).to_c()
        prm = fd.params()
        _abi.check(_abi.lib().itkg_gaussian_generate_region(
            ctypes.byref(dev.c), ctypes.byref(lg), ctypes.byref(rq), ctypes.byref(prm),
            ctypes.byref(out.c), None))
        assert gpu.last_kernel().startswith("fused3d")
        assert bits_equal(out.download(), want), (ri, rs)


def _dense_device(gpu, arr):
    """Device image with the dense (unpadded) layout of `arr` -- rows of
    arbitrary byte length, so the fused kernel must use its cp.async gather."""
    import ctypes
    from itkg import _abi
    L = _abi.lib()
    p = ctypes.c_void_p()
    _abi.check(L.itkg_device_alloc(arr.nbytes, ctypes.byref(p)))
    _abi.check(L.itkg_memcpy(p, arr.ctypes.data, arr.nbytes, 0, None))
    _abi.check(L.itkg_stream_synchronize(None))
    im = gpu.Image(arr).to_c()
    im.location = gpu._abi.DEVICE
    im.data = p.value
    return im, p


@pytest.mark.parametrize("rounding", ["reference", "fma"])
def test_fused3d_tma_and_gather_paths_agree(gpu, rounding):
    import ctypes
    from itkg import _abi
    L = _abi.lib()
    rng = np.random.default_rng(31)
    arr = rng.random((21, 27, 31), dtype=np.float32)  # 31 floats per row: not 16-byte pitched
    want = oracle.gaussian_f32(arr, 2.0)
    rnd = gpu.ROUND_REFERENCE if rounding == "reference" else gpu.ROUND_FMA
    got_tma = run_device(gpu, arr, 2.0, algo="fused", rounding=rnd)
    assert "tma" in gpu.last_kernel(), gpu.last_kernel()
    src, p = _dense_device(gpu, arr)
    out = gpu.DeviceImage(gpu.Image(arr).region)
    prm = _abi.itkg_gaussian_params()
    prm.sigma = 2.0
    prm.rounding = rnd
    prm.algorithm = gpu.ALGO_FUSED
    lg = gpu.Image(arr).region.to_c()
    _abi.check(L.itkg_gaussian_generate_region(ctypes.byref(src), ctypes.byref(lg), ctypes.byref(lg),
                                               ctypes.byref(prm), ctypes.byref(out.c), None))
    kern = gpu.last_kernel()
    got_gather = out.download()
    L.itkg_device_free(p)
    assert kern.startswith("fused3d") and "tma" not in kern, kern
    if rounding == "reference":
        assert bits_equal(got_tma, want) and bits_equal(got_gather, want)
    else:
        assert normwise(got_tma, want) <= 1e-5 and normwise(got_gather, want) <= 1e-5
    flag = ctypes.c_uint32(1)
    _abi.check(L.itkg_device_fault(1, ctypes.byref(flag)))
    assert flag.value == 0


def _typed_input(kind, shape, rng):
    """Input of the given storage type and its exact f32 value."""
    if kind == "i16":
        a = rng.integers(-1000, 1500, shape).astype(np.int16)
        return a, a.astype(np.float32)
    if kind == "u8":
        a = rng.integers(0, 256, shape).astype(np.uint8)
        return a, a.astype(np.float32)
    if kind == "f16":
        a = (rng.standard_normal(shape) * 100).astype(np.float16)
        return a, a.astype(np.float32)
    # bf16: build from f32 with the low 16 bits cleared (exactly representable)
    f = (rng.standard_normal(shape) * 100).astype(np.float32)
    bits = (f.view(np.uint32) & 0xFFFF0000).astype(np.uint32)
    return (bits >> 16).astype(np.uint16), bits.view(np.float32)


@pytest.mark.parametrize("kind", ["i16", "u8", "bf16", "f16"])
@pytest.mark.parametrize("sigma,spacing", [(1.5, (0.7, 0.7, 2.5)), (1.0, None), (2.0, None)])
def test_fused3d_native_inputs(gpu, kind, sigma, spacing):
    """Fused kernel reading i16 / u8 / bf16 / f16 directly (the cast fused into
    the load): bit-exact in reference rounding, 1e-5 in FMA rounding."""
    import ctypes
    from itkg import _abi
    rng = np.random.default_rng(41)
    raw, f32 = _typed_input(kind, (22, 40, 56), rng)
    want = oracle.gaussian_f32(f32, sigma, spacing=spacing)
    code = {"i16": gpu.I16, "u8": gpu.U8, "bf16": gpu.BF16, "f16": gpu.F16}[kind]
    img = gpu.Image(raw, spacing=spacing, bf16=(kind == "bf16"))
    dev = gpu.DeviceImage.from_host(img)
    for rounding in (gpu.ROUND_REFERENCE, gpu.ROUND_FMA):
        f = gpu.GaussianFilter(gpu.CastFilter(dev, gpu.F32), sigma, rounding=rounding,
                               algorithm=gpu.ALGO_FUSED, arithmetic=gpu.ARITH_F32)
        got = f.generate_region(dev.region).download()
        assert gpu.last_kernel().startswith(f"fused3d_{kind}"), gpu.last_kernel()
        if rounding == gpu.ROUND_REFERENCE:
            assert bits_equal(got, want)
        else:
            assert normwise(got, want) <= 1e-5


FUSED2D_CASES = [((1, 1), 1, 1.0), ((7, 600), 1, 1.0), ((64, 64), 1, 0.3), ((130, 1030), 1, 2.6),
                 ((33, 517), 1, 1.5), ((5, 3), 1, 2.0), ((40, 70), 3, 1.5), ((9, 515), 3, 2.4),
                 ((1, 40), 3, 0.9), ((200, 100), 3, 0.6), ((90, 300), 1, 3.2), ((41, 77), 3, 4.0),
                 ((130, 20), 3, 3.5), ((9, 600), 1, 4.0)]


@pytest.fixture(params=[(1, "tile2d"), (2, "fused2d")], ids=["tile", "rows"])
def kernel2d(request, gpu):
    """Both fused 2-D kernels: the tile kernel and the row-marching kernel
    (itkg_debug_set_2d_kernel); yields the kernel's launch-name prefix."""
    from itkg import _abi
    which, name = request.param
    _abi.lib().itkg_debug_set_2d_kernel(which)
    yield name
    _abi.lib().itkg_debug_set_2d_kernel(0)


@pytest.mark.parametrize("shape,comps,sigma", FUSED2D_CASES)
def test_fused2d_reference_rounding_bit_exact(gpu, kernel2d, shape, comps, sigma):
    """The fused 2-D kernels (scalar and VecPixel<f32, 3>): bit-exact with the
    reference pass-by-pass arithmetic."""
    rng = np.random.default_rng(sum(shape) + comps)
    arr = rng.standard_normal(shape + ((comps,) if comps > 1 else ())).astype(np.float32)
    want = oracle.gaussian_f32(arr, sigma, comps=comps)
    got = run_device(gpu, arr, sigma, comps=comps, algo="fused")
    assert gpu.last_kernel() == f"{kernel2d}_f32_ref", gpu.last_kernel()
    assert bits_equal(got, want)


@pytest.mark.parametrize("shape,comps,sigma", FUSED2D_CASES)
def test_fused2d_fma_within_1e5(gpu, kernel2d, shape, comps, sigma):
    rng = np.random.default_rng(3 + sum(shape) + comps)
    arr = rng.random(shape + ((comps,) if comps > 1 else ()), dtype=np.float32)
    want = oracle.gaussian_f32(arr, sigma, comps=comps)
    got = run_device(gpu, arr, sigma, comps=comps, algo="fused", rounding=gpu.ROUND_FMA)
    assert gpu.last_kernel() == f"{kernel2d}_f32_fma", gpu.last_kernel()
    assert normwise(got, want) <= 1e-5


@pytest.mark.parametrize("comps", [1, 3])
def test_fused2d_subregions_offset_index_and_outputs(gpu, kernel2d, comps):
    """Requested sub-regions of an image with a non-zero index, and the
    converted output types, through the fused 2-D kernel."""
    rng = np.random.default_rng(17 + comps)
    arr = rng.random((45, 700) + ((comps,) if comps > 1 else ()), dtype=np.float32)
    index = (-20, 11)
    for ri, rs in [((-20, 11), (700, 45)), ((480, 20), (200, 9)), ((-20, 55), (1, 1)),
                   ((0, 11), (513, 45)), ((679, 40), (1, 16))]:
        want = oracle.gaussian_f32(arr, 1.7, comps=comps, index=index, requested=(ri, rs))
        got = run_device(gpu, arr, 1.7, comps=comps, index=index, requested=(ri, rs), algo="fused")
        assert gpu.last_kernel() == f"{kernel2d}_f32_ref", gpu.last_kernel()
        assert bits_equal(got, want), (ri, rs)
    want = oracle.gaussian_f32(arr * 255, 1.7, comps=comps)
    got = run_device(gpu, arr * 255, 1.7, comps=comps, algo="fused", out_dtype=gpu.U8)
    assert gpu.last_kernel() == f"{kernel2d}_f32_ref", gpu.last_kernel()
    assert np.array_equal(got, oracle.cast_f32_to_u8(want))


def test_fused2d_falls_back_for_unequal_radii(gpu):
    """Anisotropic radii have no fused 2-D kernel: auto takes the per-axis
    path (still bit-exact) and an explicit fused request is refused."""
    from itkg import _abi
    rng = np.random.default_rng(5)
    arr = rng.random((30, 40), dtype=np.float32)
    want = oracle.gaussian_f32(arr, 1.5, spacing=(0.5, 1.0))
    got = run_device(gpu, arr, 1.5, spacing=(0.5, 1.0))
    assert gpu.last_kernel().startswith("per_axis"), gpu.last_kernel()
    assert bits_equal(got, want)
    with pytest.raises(_abi.ItkgError):
        run_device(gpu, arr, 1.5, spacing=(0.5, 1.0), algo="fused")


TWO_PASS_CASES = [((9, 17, 31), 1.0, None), ((16, 16, 16), 2.0, None), ((40, 50, 70), 2.0, None),
                  ((5, 70, 40), 2.2, None), ((12, 130, 70), 2.6, None), ((1, 1, 1), 1.0, None),
                  ((33, 65, 97), 1.5, None), ((20, 20, 20), 0.3, None), ((3, 40, 33), 1.2, None),
                  ((24, 48, 40), 1.5, (0.7, 0.7, 2.5)), ((30, 20, 10), 1.0, (1.0, 1.0, 0.5)),
                  # radii 9..12: 32 x 64 tiles, z pass up to rz = 12
                  ((40, 70, 90), 3.0, None), ((33, 130, 45), 3.4, None), ((26, 30, 70), 4.0, None),
                  ((50, 20, 36), 4.0, (1.0, 1.0, 2.0)), ((12, 64, 64), 1.2, (0.3, 0.3, 1.0))]


@pytest.mark.parametrize("shape,sigma,spacing", TWO_PASS_CASES)
def test_two_pass_reference_rounding_bit_exact(gpu, shape, sigma, spacing):
    """x-y slice kernel + z kernel: bit-exact with the reference pass by pass."""
    rng = np.random.default_rng(5 + sum(shape))
    arr = rng.standard_normal(shape).astype(np.float32)
    want = oracle.gaussian_f32(arr, sigma, spacing=spacing)
    img = gpu.Image(arr, spacing=spacing)
    dev = gpu.DeviceImage.from_host(img)
    got = gpu.GaussianFilter(dev, sigma, algorithm=gpu.ALGO_TWO_PASS).generate_region(img.region).download()
    assert gpu.last_kernel() == "z_pass_f32_ref", gpu.last_kernel()
    assert bits_equal(got, want)


@pytest.mark.parametrize("shape,sigma,spacing", TWO_PASS_CASES)
def test_two_pass_fma_within_1e5(gpu, shape, sigma, spacing):
    rng = np.random.default_rng(6 + sum(shape))
    arr = rng.random(shape, dtype=np.float32)
    want = oracle.gaussian_f32(arr, sigma, spacing=spacing)
    img = gpu.Image(arr, spacing=spacing)
    dev = gpu.DeviceImage.from_host(img)
    f = gpu.GaussianFilter(dev, sigma, rounding=gpu.ROUND_FMA, algorithm=gpu.ALGO_TWO_PASS)
    got = f.generate_region(img.region).download()
    assert gpu.last_kernel() == "z_pass_f32_fma", gpu.last_kernel()
    assert normwise(got, want) <= 1e-5


def test_two_pass_chunked_z_bit_exact(gpu):
    """1024 x 1024 slices: the intermediate is split into several z chunks
    (each with its own halo slices); the result must not depend on it."""
    rng = np.random.default_rng(77)
    arr = rng.random((23, 1024, 1024), dtype=np.float32)
    for sigma, spacing in [(1.0, (1.0, 1.0, 1.5)), (0.5, None)]:
        want = oracle.gaussian_f32(arr, sigma, spacing=spacing)
        img = gpu.Image(arr, spacing=spacing)
        dev = gpu.DeviceImage.from_host(img)
        got = gpu.GaussianFilter(dev, sigma, algorithm=gpu.ALGO_TWO_PASS).generate_region(img.region).download()
        assert gpu.last_kernel() == "z_pass_f32_ref"
        assert bits_equal(got, want)


def test_two_pass_subregions_offset_index_and_outputs(gpu):
    rng = np.random.default_rng(31)
    arr = rng.random((30, 41, 53), dtype=np.float32)
    index = (8, -3, 100)
    for ri, rs in [((8, -3, 100), (53, 41, 30)), ((12, 0, 104), (33, 20, 11)), ((60, 37, 129), (1, 1, 1)),
                   ((16, -3, 110), (4, 41, 6)), ((8, 30, 100), (45, 8, 30))]:
        want = oracle.gaussian_f32(arr, 1.9, index=index, requested=(ri, rs))
        img = gpu.Image(arr, index=index)
        dev = gpu.DeviceImage.from_host(img)
        f = gpu.GaussianFilter(dev, 1.9, algorithm=gpu.ALGO_TWO_PASS)
        got = f.generate_region(gpu.Region(ri, rs)).download()
        assert gpu.last_kernel() == "z_pass_f32_ref", gpu.last_kernel()
        assert bits_equal(got, want), (ri, rs)
    # converted outputs
    img = gpu.Image(arr * 255, index=index)
    dev = gpu.DeviceImage.from_host(img)
    want = oracle.gaussian_f32(arr * 255, 1.9, index=index)
    got = gpu.GaussianFilter(dev, 1.9, algorithm=gpu.ALGO_TWO_PASS).generate_region(img.region, out_dtype=gpu.U8)
    assert np.array_equal(got.download(), oracle.cast_f32_to_u8(want))


def test_two_pass_refuses_unaligned_start_and_auto_falls_back(gpu):
    """A requested x start that is not 16-byte aligned within the buffer has
    no TMA tile: an explicit two-pass request is refused, auto still gives the
    bit-exact result through another kernel."""
    from itkg import _abi
    rng = np.random.default_rng(32)
    arr = rng.random((12, 20, 30), dtype=np.float32)
    img = gpu.Image(arr)
    dev = gpu.DeviceImage.from_host(img)
    req = gpu.Region((3, 0, 0), (20, 20, 12))
    with pytest.raises(_abi.ItkgError):
        gpu.GaussianFilter(dev, 1.2, algorithm=gpu.ALGO_TWO_PASS).generate_region(req)
    got = gpu.GaussianFilter(dev, 1.2).generate_region(req).download()
    assert not gpu.last_kernel().startswith("z_pass"), gpu.last_kernel()
    assert bits_equal(got, oracle.gaussian_f32(arr, 1.2, requested=((3, 0, 0), (20, 20, 12))))


@pytest.mark.parametrize("kind", ["i16", "u8", "bf16", "f16"])
def test_two_pass_native_inputs(gpu, kind):
    rng = np.random.default_rng(43)
    raw, f32 = _typed_input(kind, (22, 40, 56), rng)
    spacing = (0.7, 0.7, 2.5)
    want = oracle.gaussian_f32(f32, 1.5, spacing=spacing)
    img = gpu.Image(raw, spacing=spacing, bf16=(kind == "bf16"))
    dev = gpu.DeviceImage.from_host(img)
    for rounding in (gpu.ROUND_REFERENCE, gpu.ROUND_FMA):
        f = gpu.GaussianFilter(gpu.CastFilter(dev, gpu.F32), 1.5, rounding=rounding,
                               algorithm=gpu.ALGO_TWO_PASS, arithmetic=gpu.ARITH_F32)
        got = f.generate_region(dev.region).download()
        assert gpu.last_kernel().startswith("z_pass_f32"), gpu.last_kernel()
        if rounding == gpu.ROUND_REFERENCE:
            assert bits_equal(got, want)
        else:
            assert normwise(got, want) <= 1e-5


def test_two_pass_fma_subregions_and_tight_buffers(gpu):
    """FMA rounding filters a zero-filled halo and adds the clamped taps back at
    the image's edges; check it on requested sub-regions, with the input buffer
    both the whole image and exactly input_region_for_output."""
    import ctypes
    from itkg import _abi
    rng = np.random.default_rng(23)
    full = rng.random((30, 41, 53), dtype=np.float32)
    img = gpu.Image(full)
    dev_full = gpu.DeviceImage.from_host(img)
    for sigma in (0.4, 1.9, 2.5):
        # x starts on 16-byte boundaries of the whole-image buffer (a TMA tile rule)
        for ri, rs in [((0, 0, 0), (53, 41, 30)), ((8, 5, 4), (33, 20, 11)), ((48, 40, 29), (5, 1, 1)),
                       ((12, 0, 12), (1, 41, 6)), ((0, 35, 0), (53, 6, 30))]:
            want = oracle.gaussian_f32(full, sigma, requested=(ri, rs))
            f = gpu.GaussianFilter(dev_full, sigma, rounding=gpu.ROUND_FMA, algorithm=gpu.ALGO_TWO_PASS)
            got = f.generate_region(gpu.Region(ri, rs)).download()
            assert gpu.last_kernel() == "z_pass_f32_fma"
            assert normwise(got, want) <= 1e-5, (sigma, ri, rs)
            need = gpu.GaussianFilter(img, sigma).input_region_for_output(gpu.Region(ri, rs))
            (x0, y0, z0), (sx, sy, sz) = need.index, need.size
            if (x0 - ri[0]) % 4:
                continue  # no 16-byte aligned tile start in this tight buffer
            dev = gpu.DeviceImage(need)
            dev.upload(np.ascontiguousarray(full[z0:z0 + sz, y0:y0 + sy, x0:x0 + sx]))
            out = gpu.DeviceImage(gpu.Region(ri, rs))
            lg, rq = img.region.to_c(), gpu.Region(ri, rs).to_c()
            prm = f.params()
            _abi.check(_abi.lib().itkg_gaussian_generate_region(
                ctypes.byref(dev.c), ctypes.byref(lg), ctypes.byref(rq), ctypes.byref(prm),
                ctypes.byref(out.c), None))
            assert gpu.last_kernel() == "z_pass_f32_fma"
            assert normwise(out.download(), want) <= 1e-5, ("tight", sigma, ri, rs)


@pytest.mark.parametrize("rounding", ["reference", "fma"])
def test_host_buffers_pipelined_staging(gpu, rounding):
    """Host buffers large enough to be staged in overlapping slabs along the
    last axis: the result is the device-path result (bit-exact in reference
    rounding), for whole and sub-region requests, 3-D and 2-D."""
    rnd = gpu.ROUND_REFERENCE if rounding == "reference" else gpu.ROUND_FMA
    rng = np.random.default_rng(51)
    for arr, sigma, req in [(rng.random((96, 200, 256), dtype=np.float32), 2.0, None),
                            (rng.random((96, 200, 256), dtype=np.float32), 1.3, ((8, 5, 3), (240, 190, 90))),
                            (rng.random((2100, 2304), dtype=np.float32), 1.5, None),
                            (rng.random((2100, 2304), dtype=np.float32), 0.8, ((0, 17), (2300, 2050)))]:
        img = gpu.Image(arr)
        region = gpu.Region(*req) if req else img.region
        host = gpu.GaussianFilter(img, sigma, rounding=rnd).generate_region(region).data
        dev = gpu.DeviceImage.from_host(img)
        on_dev = gpu.GaussianFilter(dev, sigma, rounding=rnd).generate_region(region).download()
        assert bits_equal(host, on_dev), (arr.shape, sigma, req)
        if rounding == "reference":
            want = oracle.gaussian_f32(arr, sigma, requested=req) if req else oracle.gaussian_f32(arr, sigma)
            assert bits_equal(host, want)


@pytest.mark.parametrize("shape", [(9, 14, 20), (30, 40)])
def test_two_component_pixels(gpu, shape):
    """VecPixel<f32, 2> images (displacement fields): every component
    filtered on its own, bit-exact in reference rounding (3-D through the
    per-axis passes, 2-D through the tile kernel)."""
    arr = np.random.default_rng(sum(shape)).standard_normal(shape + (2,)).astype(np.float32)
    want = oracle.gaussian_f32(arr, 1.4, comps=2)
    got = run_device(gpu, arr, 1.4, comps=2)
    assert bits_equal(got, want), gpu.last_kernel()
    got = run_device(gpu, arr, 1.4, comps=2, rounding=gpu.ROUND_FMA)
    assert normwise(got, want) <= 1e-5
