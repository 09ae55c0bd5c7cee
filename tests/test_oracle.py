"""Pin the CPU oracle (oracle/gauss_oracle.c) before trusting it.

1. Bit-exact against tests/golden/golden.npz (a literal pure-Python
   transcription of the reference, tests/golden/make_golden.py).
2. The reference's own tests for this path, re-run against the oracle:
   gaussian.rs:107-127, tests/pipeline.rs:19-153, tests/blur_png.rs:17-73,
   image.rs:180-210, region_splitter.rs:354-396.
3. Closed-form known answers (impulse response = outer product of the f32
   weights; FP64 oracle agrees with the f32 restatement).
"""
import math

import numpy as np
import pytest

import oracle

CASES = ["impulse2d_s1p5", "impulse3d_s1", "vecpixel2d_s1", "rand2d_s1p5", "rand2d_sub_s1p5",
         "rand3d_s1p2", "rand3d_aniso", "rand3d_sub_s2", "tiny2d_s3", "line1d_s2",
         "i16cast3d_s1p5"]
U8_CASES = ["u8pixel2d_s1p5", "u8pixel2d_wrap_s1"]


def meta(golden, name, D):
    m = golden[f"{name}__meta"]
    sigma = float(m[0])
    spacing = [float(v) for v in m[1:1 + D]]
    comps = int(m[1 + D])
    ri = tuple(int(v) for v in m[2 + D:2 + 2 * D])
    rs = tuple(int(v) for v in m[2 + 2 * D:2 + 3 * D])
    return sigma, spacing, comps, ri, rs


def spatial_dim(golden, name):
    m = golden[f"{name}__meta"]
    return (len(m) - 2) // 3


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_golden_f32(golden, name):
    D = spatial_dim(golden, name)
    sigma, spacing, comps, ri, rs = meta(golden, name, D)
    x = golden[f"{name}__in"].astype(np.float32)
    got = oracle.gaussian_f32(x, sigma, spacing=spacing, requested=(ri, rs), comps=comps)
    want = golden[f"{name}__out"]
    assert got.shape == want.shape
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("name", U8_CASES)
def test_oracle_matches_golden_u8(golden, name):
    D = spatial_dim(golden, name)
    sigma, spacing, comps, ri, rs = meta(golden, name, D)
    got = oracle.gaussian_u8(golden[f"{name}__in"], sigma, spacing=spacing, requested=(ri, rs))
    assert np.array_equal(got, golden[f"{name}__out"])


def test_u8_wrap_case_actually_wraps(golden):
    # All-255 input: the per-tap rounded products sum past 255 and wrap in the
    # reference's release build (u8 `+`), so the output is not 255.
    out = golden["u8pixel2d_wrap_s1__out"]
    assert (out != 255).all()


def test_oracle_stream_full_golden(golden):
    x = np.zeros((20, 20), np.float32)
    x[10, 10] = 1.0
    got = oracle.stream_full_f32(x, 1.5, 4)
    assert np.array_equal(got, golden["stream4_impulse2d__out"])


@pytest.mark.parametrize("sigma,spacing", [(1.5, 1.0), (2.0, 1.0), (1.5, 0.7), (1.5, 2.5),
                                           (0.5, 1.0), (8.0, 1.0)])
def test_oracle_kernel_golden(golden, sigma, spacing):
    r = oracle.kernel_radius(sigma, spacing)
    k = oracle.build_kernel(sigma / spacing, r)
    assert np.array_equal(k, golden[f"kernel_{sigma}_{spacing}"])


def test_kernel_radius_rust_semantics():
    # ceil(3*sigma/spacing) as usize: saturating, NaN -> 0, negative -> 0
    assert oracle.kernel_radius(1.5, 1.0) == 5
    assert oracle.kernel_radius(2.0, 1.0) == 6
    assert oracle.kernel_radius(1.5, 0.7) == 7
    assert oracle.kernel_radius(1.5, 2.5) == 2
    assert oracle.kernel_radius(8.0, 1.0) == 24
    assert oracle.kernel_radius(-1.0, 1.0) == 0
    assert oracle.kernel_radius(float("nan"), 1.0) == 0
    assert oracle.kernel_radius(0.0, 1.0) == 0


# ---- reference tests re-run against the oracle ----------------------------------

def test_gaussian_impulse_energy_and_peak_2d():
    # gaussian.rs:107-127, tests/pipeline.rs:37-54
    img = np.zeros((21, 21), np.float32)
    img[10, 10] = 1.0
    out = oracle.gaussian_f32(img, 1.5)
    assert abs(float(out.sum(dtype=np.float32)) - 1.0) < 0.01
    assert (out <= out[10, 10] + 1e-6).all()


def test_gaussian_3d_energy():
    # tests/pipeline.rs:60-72
    img = np.zeros((11, 11, 11), np.float32)
    img[5, 5, 5] = 1.0
    out = oracle.gaussian_f32(img, 1.0)
    assert abs(float(out.sum(dtype=np.float32)) - 1.0) < 0.05


def test_vector_pixel_channel_sums():
    # tests/pipeline.rs:78-100
    img = np.zeros((11, 11, 3), np.float32)
    img[5, 5] = [1.0, 2.0, 3.0]
    out = oracle.gaussian_f32(img, 1.0, comps=3)
    for c, want in enumerate([1.0, 2.0, 3.0]):
        assert abs(float(out[..., c].sum(dtype=np.float32)) - want) < 0.05


def test_streaming_matches_full_bitwise():
    # tests/pipeline.rs:106-129 (tolerance 1e-6 there; the restatement is bitwise)
    img = np.zeros((20, 20), np.float32)
    img[10, 10] = 1.0
    full = oracle.gaussian_f32(img, 1.5)
    streamed = oracle.stream_full_f32(img, 1.5, 4)
    assert np.array_equal(full, streamed)
    rng = np.random.default_rng(3)
    vol = rng.random((19, 9, 7), dtype=np.float32)
    assert np.array_equal(oracle.gaussian_f32(vol, 1.3), oracle.stream_full_f32(vol, 1.3, 5))


def test_threshold_chain():
    # tests/pipeline.rs:135-153
    img = np.zeros((21, 21), np.float32)
    img[10, 10] = 1.0
    out = oracle.gaussian_f32(img, 1.5)
    lit = int((np.where(out > 0.01, 1.0, 0.0) > 0.5).sum())
    assert 0 < lit < 21 * 21


def test_blur_u8_roundtrip():
    # tests/blur_png.rs:17-73 minus the PNG file round trip
    img = np.zeros((32, 32), np.uint8)
    img[16, 16] = 255
    out = oracle.cast_f32_to_u8(oracle.gaussian_f32(img.astype(np.float32), 2.0))
    assert out.max() < 255
    assert out[16, 16] == out.max()
    assert int(out.astype(np.uint32).sum()) >= 255 * 85 // 100


def test_region_and_splitter_reference_tests():
    # region_splitter.rs:354-396
    p = oracle.split_region((0, 0), (4, 6), 3)
    assert [s[1] for _, s in p] == [2, 2, 2]
    p = oracle.split_region((0, 0), (4, 7), 3)
    assert sum(s[1] for _, s in p) == 7 and all(s[1] > 0 for _, s in p)
    p = oracle.split_region((0, 0), (4, 2), 10)
    assert len(p) == 2 and sum(s[1] for _, s in p) == 2
    p = oracle.split_region((5,), (10,), 4)
    assert sum(s[0] for _, s in p) == 10 and p[0][0][0] == 5


# ---- closed-form known answers ------------------------------------------------

def test_impulse_response_is_outer_product_of_f32_weights():
    img = np.zeros((21, 21), np.float32)
    img[10, 10] = 1.0
    r = oracle.kernel_radius(1.5, 1.0)
    w32 = oracle.build_kernel(1.5, r).astype(np.float32)
    out = oracle.gaussian_f32(img, 1.5)
    want = np.zeros((21, 21), np.float32)
    for y in range(10 - r, 10 + r + 1):
        for x in range(10 - r, 10 + r + 1):
            want[y, x] = np.float32(w32[10 - x + r]) * np.float32(w32[10 - y + r])
    assert np.array_equal(out, want)


def test_fp64_oracle_close_to_f32():
    rng = np.random.default_rng(11)
    vol = rng.random((10, 14, 12))
    o64 = oracle.gaussian_f64(vol, 1.7, spacing=[1.0, 0.8, 1.3])
    o32 = oracle.gaussian_f32(vol.astype(np.float32), 1.7, spacing=[1.0, 0.8, 1.3])
    assert np.abs(o64 - o32).max() / np.abs(o64).max() < 1e-6
    # numpy FP64 whole-image path agrees with the C FP64 path
    onp = oracle.gaussian_whole_f64(vol, 1.7, spacing=[1.0, 0.8, 1.3])
    assert np.abs(onp - o64).max() < 1e-12


def test_mt_timing_port_matches_serial():
    rng = np.random.default_rng(5)
    vol = rng.random((12, 17, 9), dtype=np.float32)
    a = oracle.gaussian_f32(vol, 1.4)
    b = oracle.gaussian_f32_mt(vol, 1.4, nthreads=4)
    assert np.array_equal(a, b)


def test_sigma_edge_cases():
    img = np.arange(30, dtype=np.float32).reshape(5, 6) - 10.0
    # negative sigma: radius 0, kernel [1] -> identity (but -0.0 -> +0.0 through 0 + x*1)
    out = oracle.gaussian_f32(img, -2.0)
    assert np.array_equal(out, img)
    # sigma 0: 0/0 in build_kernel -> NaN everywhere
    assert np.isnan(oracle.gaussian_f32(img, 0.0)).all()


def test_adjoint_helpers_dot_identity():
    rng = np.random.default_rng(2)
    x = rng.standard_normal((7, 9, 8))
    y = rng.standard_normal((7, 9, 8))
    Gx = oracle.gaussian_whole_f64(x, 1.3)
    GTy = oracle.gaussian_adjoint_f64(y, 1.3)
    assert math.isclose(float((Gx * y).sum()), float((x * GTy).sum()), rel_tol=1e-12)


def test_dsigma_helper_matches_finite_difference():
    rng = np.random.default_rng(4)
    x = rng.standard_normal((6, 8, 7))
    s0, h = 1.3, 1e-5
    radii = [oracle.kernel_radius(s0, 1.0)] * 3
    d = oracle.gaussian_dsigma_f64(x, s0, radii=radii)
    fd = (oracle.gaussian_whole_f64(x, s0 + h, radii=radii)
          - oracle.gaussian_whole_f64(x, s0 - h, radii=radii)) / (2 * h)
    assert np.abs(d - fd).max() < 1e-7 * max(1.0, np.abs(d).max())
