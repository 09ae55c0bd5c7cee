"""The one-trip 3-D forward (ITKG_ALGO_ONE_TRIP): x, y and z passes in one
kernel.  Reference rounding must be bit-identical to the oracle (the C
restatement of gaussian.rs / conv.rs) for every radius pair it takes, ragged
tiles, sub-regions, offset indices, anisotropic spacing and the z segments of
the work split; FMA rounding within 1e-5 normwise; narrow outputs convert as
the other kernels do; stream_full pieces equal the full request."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32))


def normwise(a, ref):
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.abs(np.asarray(a, np.float64) - ref).max() / max(np.abs(ref).max(), 1e-300))


def run(gpu, arr, sigma, rounding, spacing=None, requested=None, index=None, out_dtype=None):
    img = gpu.Image(arr, index=index, spacing=spacing)
    dev = gpu.DeviceImage.from_host(img)
    f = gpu.GaussianFilter(dev, sigma, rounding=rounding, algorithm=gpu.ALGO_ONE_TRIP)
    req = gpu.Region(*requested) if requested else img.region
    return f.generate_region(req, out_dtype=out_dtype).download()


CASES = [
    ((40, 64, 64), 2.0, None),             # r = 6 on every axis, whole tiles
    ((33, 70, 37), 2.0, None),             # ragged tiles on x and y
    ((9, 17, 31), 1.0, None),              # r = 3, thin z
    ((1, 1, 1), 1.0, None),                # a single voxel
    ((5, 3, 4), 2.5, None),                # radius 8, above the image size
    ((50, 130, 90), 2.6, None),            # r = 8, several tiles and segments
    ((24, 80, 96), 1.5, (0.7, 0.7, 2.5)),  # radii (7, 7, 2), the CT spacing
    ((30, 66, 48), 1.5, (0.6, 0.6, 0.6)),  # radii (8, 8, 8)
    ((44, 72, 40), 0.35, None),            # r = 2
    ((20, 40, 24), 0.3, None),             # r = 1
    ((70, 65, 33), 1.2, (0.5, 0.5, 1.0)),  # radii (8, 8, 4)
]


@pytest.mark.parametrize("shape,sigma,spacing", CASES)
def test_reference_rounding_bit_exact(gpu, shape, sigma, spacing):
    rng = np.random.default_rng(sum(shape))
    arr = rng.standard_normal(shape).astype(np.float32)
    want = oracle.gaussian_f32(arr, sigma, spacing=spacing)
    got = run(gpu, arr, sigma, gpu.ROUND_REFERENCE, spacing=spacing)
    assert gpu.last_kernel() == "one_trip_f32_ref", gpu.last_kernel()
    assert bits_equal(got, want)


@pytest.mark.parametrize("shape,sigma,spacing", CASES)
def test_fma_rounding_within_1e5(gpu, shape, sigma, spacing):
    rng = np.random.default_rng(1 + sum(shape))
    arr = rng.random(shape, dtype=np.float32)
    want = oracle.gaussian_f32(arr, sigma, spacing=spacing)
    got = run(gpu, arr, sigma, gpu.ROUND_FMA, spacing=spacing)
    assert gpu.last_kernel() == "one_trip_f32_fma", gpu.last_kernel()
    assert normwise(got, want) <= 1e-5


@pytest.mark.parametrize("rounding", ["reference", "fma"])
def test_subregions_and_offset_index(gpu, rounding):
    rng = np.random.default_rng(7)
    arr = rng.random((40, 90, 100), dtype=np.float32)
    index = (8, -3, 100)
    spacing = (0.9, 0.9, 1.7)  # radii (7, 7, 4)
    rnd = gpu.ROUND_REFERENCE if rounding == "reference" else gpu.ROUND_FMA
    for ri, rs in [((8, -3, 100), (100, 90, 40)), ((12, 0, 104), (52, 71, 9)), ((60, 20, 121), (20, 6, 2)),
                   ((8, -3, 100), (4, 1, 1)), ((40, 50, 110), (68, 37, 30))]:
        want = oracle.gaussian_f32(arr, 2.1, spacing=spacing, index=index, requested=(ri, rs))
        got = run(gpu, arr, 2.1, rnd, spacing=spacing, index=index, requested=(ri, rs))
        assert gpu.last_kernel().startswith("one_trip"), gpu.last_kernel()
        if rounding == "reference":
            assert bits_equal(got, want), (ri, rs)
        else:
            assert normwise(got, want) <= 1e-5, (ri, rs)


def test_nonfinite_inputs_like_reference(gpu):
    rng = np.random.default_rng(9)
    arr = rng.random((20, 70, 40), dtype=np.float32)
    arr[3, 4, 5] = np.inf
    arr[8, 60, 2] = np.nan
    arr[0, 0, 0] = -0.0
    want = oracle.gaussian_f32(arr, 1.3)
    assert bits_equal(run(gpu, arr, 1.3, gpu.ROUND_REFERENCE), want)


@pytest.mark.parametrize("out", ["bf16", "f16", "u8"])
def test_narrow_outputs(gpu, out):
    rng = np.random.default_rng(11)
    arr = (rng.random((24, 70, 48), dtype=np.float32) * 300.0).astype(np.float32)
    f32 = oracle.gaussian_f32(arr, 1.5)
    code = {"bf16": gpu.BF16, "f16": gpu.F16, "u8": gpu.U8}[out]
    raw = run(gpu, arr, 1.5, gpu.ROUND_REFERENCE, out_dtype=code)
    if out == "u8":
        assert np.array_equal(raw, oracle.cast_f32_to_u8(f32))
    elif out == "bf16":
        got = (raw.astype(np.uint32) << 16).view(np.float32)
        assert normwise(got, f32) <= 2.0 ** -8
    else:
        assert normwise(raw.astype(np.float32), f32) <= 2.0 ** -11


@pytest.mark.parametrize("rounding", ["reference", "fma"])
def test_stream_full_pieces_equal_full(gpu, rounding):
    rng = np.random.default_rng(12)
    arr = rng.random((37, 80, 64), dtype=np.float32)
    dev = gpu.DeviceImage.from_host(gpu.Image(arr))
    rnd = gpu.ROUND_REFERENCE if rounding == "reference" else gpu.ROUND_FMA
    f = gpu.GaussianFilter(dev, 2.0, rounding=rnd, algorithm=gpu.ALGO_ONE_TRIP)
    full = f.generate_region(dev.region).download()
    for n in (1, 3, 8, 100):
        assert bits_equal(gpu.stream_full(f, n).download(), full), n
    if rounding == "reference":
        assert bits_equal(full, oracle.gaussian_f32(arr, 2.0))


def test_unsupported_geometry_is_refused(gpu):
    from itkg import _abi
    rng = np.random.default_rng(13)
    arr = rng.random((10, 20, 30), dtype=np.float32)
    dev = gpu.DeviceImage.from_host(gpu.Image(arr))
    with pytest.raises(_abi.ItkgError) as ei:  # radius 12 on x and y
        gpu.GaussianFilter(dev, 4.0, algorithm=gpu.ALGO_ONE_TRIP).generate_region(dev.region)
    assert ei.value.status == _abi.ERROR_UNSUPPORTED
