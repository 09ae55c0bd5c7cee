"""GPU parity of the convolve_axis family (MeanFilter, BoxMeanFilterN,
BinomialBlurFilter and explicit kernels) through itkg_separable_generate_region,
against the oracle on the same seeded inputs: reference rounding bit-exact,
FMA rounding within 1e-5 normwise (max|gpu - ref| / max|ref|)."""
import math

import numpy as np
import pytest

import oracle
from test_gpu_parity import bits_equal, normwise

pytestmark = pytest.mark.gpu

TOL_FMA = 1e-5


def _algo(itkg, name):
    return {"auto": itkg.ALGO_AUTO, "per_axis": itkg.ALGO_PER_AXIS, "fused": itkg.ALGO_FUSED,
            "two_pass": itkg.ALGO_TWO_PASS}[name]


def run(itkg, make, arr, comps=1, requested=None, rounding=0, algo="auto", index=None, host=False,
        arithmetic=None, out_dtype=None):
    img = itkg.Image(arr, index=index, components=comps)
    src = img if host else itkg.DeviceImage.from_host(img)
    f = make(src, rounding=rounding, algorithm=_algo(itkg, algo), arithmetic=arithmetic)
    req = itkg.Region(*requested) if requested else img.region
    out = f.generate_region(req, out_dtype=out_dtype)
    return (out.data if host else out.download()), itkg.last_kernel()


def vol(shape, seed):
    return np.random.default_rng(seed).standard_normal(shape).astype(np.float32)


@pytest.mark.parametrize("family", ["mean", "boxmean", "binomial"])
def test_golden_family_bit_exact(gpu, golden, family):
    from test_oracle_family import GOLDEN_SEP, sep_meta
    for name in GOLDEN_SEP:
        if not name.startswith(family):
            continue
        kernels, reps, comps, req = sep_meta(golden, name)
        got, k = run(gpu, lambda s, **kw: gpu.SeparableFilter(s, kernels, reps, **kw),
                     golden[f"sep_{name}__in"], comps=comps, requested=req)
        assert bits_equal(got, golden[f"sep_{name}__out"]), (name, k)


@pytest.mark.parametrize("name", ["mean_u8_2d_r2", "binomial_u8_2d_r2"])
def test_golden_family_u8_pixel(gpu, golden, name):
    from test_oracle_family import sep_meta
    kernels, reps, comps, req = sep_meta(golden, name)
    got, _ = run(gpu, lambda s, **kw: gpu.SeparableFilter(s, kernels, reps, **kw), golden[f"sep_{name}__in"],
                 requested=req, arithmetic=gpu.ARITH_PIXEL_U8, out_dtype=gpu.U8)
    assert np.array_equal(got, golden[f"sep_{name}__out"])


MEAN3D = [(1, "auto", "z_pass"), (2, "auto", "z_pass"), (6, "auto", "z_pass"), (12, "auto", "z_pass"),
          (13, "auto", "per_axis"), (3, "fused", "fused3d"), (4, "per_axis", "per_axis")]


@pytest.mark.parametrize("r,algo,kernel", MEAN3D)
@pytest.mark.parametrize("rounding", [0, 1])
def test_mean_3d(gpu, r, algo, kernel, rounding):
    x = vol((30, 36, 40), 10 + r)
    want = oracle.mean_f32(x, r)
    got, k = run(gpu, lambda s, **kw: gpu.MeanFilter(s, r, **kw), x, rounding=rounding, algo=algo)
    assert kernel in k, k
    if rounding == 0:
        assert bits_equal(got, want), k
    else:
        assert normwise(got, want) <= TOL_FMA, k


@pytest.mark.parametrize("radii,kernel", [((2, 2, 5), "z_pass"), ((1, 3, 2), "per_axis"), ((7, 7, 2), "z_pass")])
def test_box_mean_3d_anisotropic(gpu, radii, kernel):
    x = vol((24, 33, 40), 20)
    want = oracle.box_mean_f32(x, radii)
    got, k = run(gpu, lambda s, **kw: gpu.BoxMeanFilterN(s, radii, **kw), x)
    assert kernel in k and bits_equal(got, want), k


@pytest.mark.parametrize("comps", [1, 3])
@pytest.mark.parametrize("rounding", [0, 1])
def test_mean_2d(gpu, comps, rounding):
    shape = (70, 90, 3) if comps == 3 else (70, 90)
    x = np.random.default_rng(30 + comps).random(shape, dtype=np.float32)
    want = oracle.mean_f32(x, 3, comps=comps)
    got, k = run(gpu, lambda s, **kw: gpu.MeanFilter(s, 3, **kw), x, comps=comps, rounding=rounding)
    if rounding == 0:
        assert bits_equal(got, want), k
    else:
        assert normwise(got, want) <= TOL_FMA, k


@pytest.mark.parametrize("shape", [(50,), (40, 45), (20, 26, 31)])
@pytest.mark.parametrize("reps", [0, 1, 2, 5])
@pytest.mark.parametrize("rounding", [0, 1])
def test_binomial(gpu, shape, reps, rounding):
    x = vol(shape, 40 + reps)
    want = oracle.binomial_f32(x, reps)
    got, k = run(gpu, lambda s, **kw: gpu.BinomialBlurFilter(s, reps, **kw), x, rounding=rounding)
    if rounding == 0 or reps == 0:
        assert bits_equal(got, want), k
    else:
        assert normwise(got, want) <= TOL_FMA, k


def test_binomial_reference_tests(gpu):
    """binomial_blur.rs:96-121 through the GPU path."""
    c = np.full(20, 3.0, np.float32)
    out, _ = run(gpu, lambda s, **kw: gpu.BinomialBlurFilter(s, 4, **kw), c)
    assert np.all(np.abs(out[4:16] - 3.0) < 1e-5)
    imp = np.zeros(21, np.float32)
    imp[10] = 1.0
    out, _ = run(gpu, lambda s, **kw: gpu.BinomialBlurFilter(s, 4, **kw), imp)
    assert 0.0 < out[10] < 1.0 and abs(float(out.sum()) - 1.0) < 0.05
    assert abs(gpu.BinomialBlurFilter.effective_sigma_pixels(4) - 1.0) < 1e-10


def test_mean_reference_tests(gpu):
    """mean.rs:254-292 through the GPU path."""
    out, _ = run(gpu, lambda s, **kw: gpu.MeanFilter(s, 2, **kw), np.full(10, 5.0, np.float32))
    assert np.all(np.abs(out - 5.0) < 1e-5)
    out, _ = run(gpu, lambda s, **kw: gpu.MeanFilter(s, 2, **kw), np.arange(20, dtype=np.float32))
    assert all(abs(out[i] - i) < 1e-4 for i in range(2, 18))
    out, _ = run(gpu, lambda s, **kw: gpu.BoxMeanFilterN(s, (1, 2), **kw), np.full((8, 8), 3.0, np.float32))
    assert np.all(np.abs(out - 3.0) < 1e-5)


@pytest.mark.parametrize("family", ["mean", "binomial"])
def test_subregion_with_offset_index(gpu, family):
    x = vol((22, 30, 36), 50)
    index = (5, -3, 7)
    req = ((13, 2, 10), (16, 20, 9))  # absolute; x start 8 pixels into the buffer
    if family == "mean":
        want = oracle.mean_f32(x, 2, index=index, requested=req)
        make = lambda s, **kw: gpu.MeanFilter(s, 2, **kw)
    else:
        want = oracle.binomial_f32(x, 3, index=index, requested=req)
        make = lambda s, **kw: gpu.BinomialBlurFilter(s, 3, **kw)
    got, k = run(gpu, make, x, index=index, requested=req)
    assert bits_equal(got, want), k


def test_asymmetric_kernel_runs_per_axis(gpu):
    x = vol((18, 21, 25), 60)
    ks = [np.array([0.1, 0.2, 0.7]), np.array([0.5, 0.25, 0.125, 0.0625, 0.0625]), np.array([1.0])]
    want = oracle.separable_f32(x, ks, 1)
    got, k = run(gpu, lambda s, **kw: gpu.SeparableFilter(s, ks, 1, **kw), x)
    assert "per_axis" in k and bits_equal(got, want), k


@pytest.mark.parametrize("algo,kernel", [("two_pass", "z_pass"), ("fused", "fused3d"), ("per_axis", "per_axis")])
@pytest.mark.parametrize("rounding", [0, 1])
def test_binomial_rounds_through_single_round_kernels(gpu, algo, kernel, rounding):
    """Each round is one single-round call (x, y, z) in the chosen kernels."""
    x = vol((24, 28, 32), 61)
    want = oracle.binomial_f32(x, 3)
    got, k = run(gpu, lambda s, **kw: gpu.BinomialBlurFilter(s, 3, **kw), x, algo=algo, rounding=rounding)
    assert kernel in k, k
    if rounding == 0:
        assert bits_equal(got, want), k
    else:
        assert normwise(got, want) <= TOL_FMA, k


def test_explicit_single_launch_kernels_refuse_asymmetric(gpu):
    x = vol((10, 12, 16), 61)
    ks = [np.array([0.1, 0.2, 0.7])] * 3
    with pytest.raises(gpu.ItkgError) as e:
        run(gpu, lambda s, **kw: gpu.SeparableFilter(s, ks, 1, **kw), x, algo="fused")
    assert e.value.status == 2  # ITKG_ERROR_UNSUPPORTED


def test_unsharp_style_gaussian_kernel(gpu):
    """edges.rs:414-430 builds exp(-d^2 / (2 sigma^2)) normalised and runs one
    pass per axis over the padded input; on the requested region that is one
    round of the family with that kernel."""
    sigma = 1.7
    r = math.ceil(3 * sigma)
    d = np.arange(2 * r + 1) - r
    w = np.exp(-(d * d) / (2 * sigma * sigma))
    w = w / w.sum()
    x = vol((26, 28, 32), 62)
    want = oracle.separable_f32(x, [w] * 3, 1)
    got, k = run(gpu, lambda s, **kw: gpu.SeparableFilter(s, [w] * 3, 1, **kw), x)
    assert bits_equal(got, want), k


@pytest.mark.parametrize("reps", [1, 3])
def test_host_buffers_staged(gpu, reps):
    """Host buffers above 8 MiB of output are staged in slabs; each slab's
    input covers its rounds' halo."""
    x = vol((160, 120, 128), 70 + reps)  # 9.4 MiB f32
    want = oracle.binomial_f32(x, reps)
    got, k = run(gpu, lambda s, **kw: gpu.BinomialBlurFilter(s, reps, **kw), x, host=True)
    assert bits_equal(got, want), k


@pytest.mark.parametrize("r", [1, 2, 5])
def test_mean_u8_pixel_arithmetic_takes_the_two_pass_kernels(gpu, r):
    """MeanFilter over Image<u8, 3> in u8 pixel arithmetic (one round of a
    symmetric kernel): the two-pass u8 kernels, bit-identical to the oracle
    and to the per-axis passes."""
    x = np.random.default_rng(40 + r).integers(0, 256, (18, 30, 48), dtype=np.uint8)
    k = oracle.box_kernel(r)
    want = oracle.separable_u8(x, [k, k, k])
    make = lambda s, **kw: gpu.MeanFilter(s, r, **kw)
    got, kern = run(gpu, make, x, arithmetic=gpu.ARITH_PIXEL_U8, out_dtype=gpu.U8)
    assert kern == "z_pass_u8_pixel", kern
    assert np.array_equal(got, want)
    got, kern = run(gpu, make, x, algo="per_axis", arithmetic=gpu.ARITH_PIXEL_U8, out_dtype=gpu.U8)
    assert kern != "z_pass_u8_pixel", kern
    assert np.array_equal(got, want)
