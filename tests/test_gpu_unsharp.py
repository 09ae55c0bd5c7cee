"""GPU parity of UnsharpMaskFilter (edges.rs:374-452) through
itkg_unsharp_mask_generate_region, against the oracle on the same seeded
inputs: reference rounding bit-exact (f32 and u8, scalar and 3-component
pixels); FMA rounding of the blur within 2e-5 normwise
(max|gpu - ref| / max|ref|: the blur's 1e-5 bound times 1 + amount)."""
import numpy as np
import pytest

import oracle
from test_gpu_parity import bits_equal, normwise
from test_oracle_unsharp import USH, ush_meta

pytestmark = pytest.mark.gpu

TOL_FMA = 2e-5


def run(itkg, arr, sigma, amount=0.5, threshold=0.0, requested=None, index=None, comps=1, host=False,
        rounding=0):
    img = itkg.Image(arr, index=index, components=comps)
    src = img if host else itkg.DeviceImage.from_host(img)
    f = itkg.UnsharpMaskFilter(src, sigma, amount, threshold, rounding=rounding)
    req = itkg.Region(*requested) if requested else img.region
    out = f.generate_region(req)
    return out.data if host else out.download()


@pytest.mark.parametrize("host", [False, True])
@pytest.mark.parametrize("name", USH)
def test_golden_bit_exact(gpu, golden, name, host):
    sigma, amount, threshold, comps, req = ush_meta(golden, name)
    got = run(gpu, golden[f"ush_{name}__in"], sigma, amount, threshold, requested=req, comps=comps, host=host)
    want = golden[f"ush_{name}__out"]
    assert got.dtype == want.dtype
    assert np.array_equal(np.asarray(got).view(np.uint8), want.view(np.uint8))


@pytest.mark.parametrize("shape,sigma,amount,threshold", [((40, 48, 56), 1.5, 0.5, 0.0),
                                                          ((33, 29, 70), 3.7, 1.2, 0.3),
                                                          ((20, 24, 31), 5.0, 0.5, 0.0),
                                                          ((96, 128), 2.2, 0.8, 0.05),
                                                          ((500,), 4.0, 2.0, 0.0)])
def test_random_bit_exact(gpu, shape, sigma, amount, threshold):
    x = np.random.default_rng(len(shape) * 11 + int(sigma * 10)).standard_normal(shape).astype(np.float32)
    want = oracle.unsharp_mask(x, sigma, amount, threshold)
    assert bits_equal(run(gpu, x, sigma, amount, threshold), want)


def test_subregion_with_offset_index(gpu):
    x = np.random.default_rng(3).random((30, 34, 38), dtype=np.float32)
    index = (5, -3, 2)
    req = ((9, 4, 6), (20, 17, 19))
    want = oracle.unsharp_mask(x, 1.8, 0.6, 0.02, index=index, requested=req)
    for host in (False, True):
        assert bits_equal(run(gpu, x, 1.8, 0.6, 0.02, requested=req, index=index, host=host), want)


@pytest.mark.parametrize("shape,sigma", [((24, 30, 36), 1.5), ((64, 80), 2.5)])
def test_u8(gpu, shape, sigma):
    x = np.random.default_rng(17).integers(0, 256, shape, dtype=np.uint8)
    want = oracle.unsharp_mask(x, sigma, 0.9, 2.0)
    got = run(gpu, x, sigma, 0.9, 2.0)
    assert got.dtype == np.uint8 and np.array_equal(got, want)


def test_vector_pixels(gpu):
    x = np.random.default_rng(23).random((14, 16, 18, 3), dtype=np.float32)
    want = oracle.unsharp_mask(x, 1.2, 0.5, 0.0, comps=3)
    got = run(gpu, x, 1.2, 0.5, 0.0, comps=3)
    assert bits_equal(got, want)
    assert np.array_equal(got[..., 1], got[..., 0]) and np.array_equal(got[..., 2], got[..., 0])


def test_fma_rounding(gpu):
    x = np.random.default_rng(29).standard_normal((48, 56, 64)).astype(np.float32)
    want = oracle.unsharp_mask(x, 2.0, 1.0, 0.0)
    assert normwise(run(gpu, x, 2.0, 1.0, 0.0, rounding=1), want) <= TOL_FMA


def test_threshold_and_amount_edges(gpu):
    x = np.random.default_rng(31).random((10, 12, 14), dtype=np.float32)
    assert bits_equal(run(gpu, x, 1.0, 0.8, np.inf), x)
    assert bits_equal(run(gpu, x, 1.0, 0.0, 0.0), x)
    assert bits_equal(run(gpu, x, 1.0, -0.5, 0.1), oracle.unsharp_mask(x, 1.0, -0.5, 0.1))


def test_epilogue_edge_values(gpu):
    # The f32 point-wise step decides most voxels in f32 and the rest in f64:
    # thresholds equal to some |orig - blur| exactly, amounts that create
    # exact f32 ties (0.5, 1.5) or are not f32 (0.1), values over a wide
    # exponent range, zeros of both signs, infinities and NaN.
    rng = np.random.default_rng(41)
    x = (rng.standard_normal((12, 20, 24)) * np.exp(rng.uniform(-30, 30, (12, 20, 24)))).astype(np.float32)
    x[0, :4, :4] = 0.0
    x[1, :4, :4] = -0.0
    x[2, 0, :3] = [np.inf, -np.inf, np.nan]
    x[3] = np.float32(1.0) + np.arange(20 * 24, dtype=np.float32).reshape(20, 24) * np.float32(2.0 ** -23)
    blur = oracle.separable_f32(x, [oracle.unsharp_kernel(1.1)] * 3)
    e = np.abs(x[4:].astype(np.float64) - blur[4:].astype(np.float64))
    e = e[np.isfinite(e) & (e > 0)]
    for amount in (0.5, 1.5, 0.1, -2.0):
        for thr in (0.0, float(e[7]), float(e[123]), -1.0, np.inf):
            want = oracle.unsharp_mask(x, 1.1, amount, thr)
            got = run(gpu, x, 1.1, amount, thr)
            assert bits_equal(got, want), (amount, thr)


def test_exact_ties_from_small_integers(gpu):
    # integer-valued f32 images with amount 0.5: orig + amount * edge often
    # lands exactly halfway between two f32 values at large magnitudes
    x = np.random.default_rng(43).integers(-2 ** 24, 2 ** 24, (16, 18, 20)).astype(np.float32)
    for amount in (0.5, 0.25, 3.0):
        assert bits_equal(run(gpu, x, 0.9, amount, 0.0), oracle.unsharp_mask(x, 0.9, amount, 0.0))


def test_every_voxel_undecided(gpu):
    # values past the f32 test's magnitude guard: every voxel takes the f64
    # sequence, more per block than the deferred list holds (the rest in place)
    x = (np.float32(2.0 ** 95) * (1 + np.random.default_rng(47).random((160, 256, 256), dtype=np.float32)))
    x = x.astype(np.float32)
    want = oracle.unsharp_mask(x, 1.0, 0.5, 0.0)
    assert bits_equal(run(gpu, x, 1.0, 0.5, 0.0), want)


@pytest.mark.parametrize("rounding", [0, 1])
def test_fused_z_store_and_fallback_paths(gpu, rounding):
    # 3-D f32 with whole aligned quads: the two-pass z kernel stores the
    # point-wise step; odd widths take the blur image + point-wise kernels
    rng = np.random.default_rng(53)
    for shape, fused in (((24, 28, 64), True), ((24, 28, 30), False)):
        x = rng.standard_normal(shape).astype(np.float32)
        want = oracle.unsharp_mask(x, 1.3, 0.7, 0.01)
        got = run(gpu, x, 1.3, 0.7, 0.01, rounding=rounding)
        if rounding == 0:
            assert bits_equal(got, want)
        else:
            assert normwise(got, want) <= TOL_FMA
        assert gpu.last_kernel().startswith("z_pass_unsharp") == fused, gpu.last_kernel()


@pytest.mark.parametrize("amount,threshold", [(0.5, 0.0), (1.5, 3.0), (0.1, 2.5), (3.0, -1.0), (0.7, float("nan"))])
def test_u8_amounts_and_thresholds(gpu, amount, threshold):
    # u8 pixels: integer edges, exact ties at amount 0.5 / 1.5, integer thresholds met exactly
    x = np.random.default_rng(71).integers(0, 256, (20, 26, 36), dtype=np.uint8)
    want = oracle.unsharp_mask(x, 1.2, amount, threshold)
    assert np.array_equal(run(gpu, x, 1.2, amount, threshold), want)
