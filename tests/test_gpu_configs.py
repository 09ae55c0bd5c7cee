"""GPU parity at the sizes the path is measured on, not only on small shapes.

  2-D   Image<f32,2> 512x512, U[0,1), sigma 1.5 (r = 5)
  3-D   Image<f32,3> 256^3 blobs + noise, sigma 2 (r = 6): reference rounding
        bit-exact for each kernel family (x-y + z, fused, per-axis) and the
        host-staged call; stream_full with 8 pieces bit-identical to the full
        request; FMA rounding within 1e-5 normwise
  CT    Image<i16,3> 512x512x384, spacing (0.7, 0.7, 2.5), sigma 1.5 mm
        (radii 7, 7, 2): f32 output bit-exact in reference rounding, within
        1e-5 in FMA rounding; bf16 / f16 storage within half an ulp of FP64
  VJP   one 192^3 blobs volume, the scale stack sigma {1, 2, 4, 8} (radii 3,
        6, 12, 24): loss, dL/dx and dL/dsigma_l against FP64 and against
        central differences (h = 1e-3, radius frozen); and the adjoint and
        dL/dsigma at radii 13..24 on their own

The oracle is the C restatement of gaussian.rs / conv.rs / pixel.rs
(reference rounding) and the FP64 numpy oracle (adjoint and sigma
derivative); inputs are the seeded synthetic volumes of itkg.workloads.
"""
import numpy as np
import pytest

import oracle
from itkg.workloads import blobs_volume, ct_volume, uniform_image

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


def _algo(itkg, name):
    return {"auto": itkg.ALGO_AUTO, "per_axis": itkg.ALGO_PER_AXIS, "fused": itkg.ALGO_FUSED,
            "two_pass": itkg.ALGO_TWO_PASS}[name]


# kernel names a call of each algorithm must report (the last launch of the call)
FAMILY = {"two_pass": "z_pass_f32", "fused": "fused3d", "per_axis": "per_axis_f32"}


# ---- 2-D: 512^2 f32, sigma 1.5 ----------------------------------------------

@pytest.mark.parametrize("algo", ["auto", "fused", "per_axis"])
def test_2d_512_reference_bit_exact_and_fma(gpu, algo):
    x = uniform_image((512, 512), seed=0)
    want = oracle.gaussian_f32(x, 1.5)
    dev = gpu.DeviceImage.from_host(gpu.Image(x))
    for rounding in (gpu.ROUND_REFERENCE, gpu.ROUND_FMA):
        got = gpu.GaussianFilter(dev, 1.5, rounding=rounding, algorithm=_algo(gpu, algo)) \
            .generate_region(dev.region).download()
        if rounding == gpu.ROUND_REFERENCE:
            assert bits_equal(got, want), gpu.last_kernel()
        else:
            assert normwise(got, want) <= 1e-5, gpu.last_kernel()


# ---- 3-D: 256^3 blobs + noise, sigma 2 ----------------------------------------

@pytest.fixture(scope="module")
def blobs256():
    x = blobs_volume((256, 256, 256), 0)
    return x, oracle.gaussian_f32_mt(x, 2.0)


@pytest.mark.parametrize("algo", ["two_pass", "fused", "per_axis"])
def test_3d_256_reference_bit_exact(gpu, blobs256, algo):
    x, want = blobs256
    dev = gpu.DeviceImage.from_host(gpu.Image(x))
    got = gpu.GaussianFilter(dev, 2.0, rounding=gpu.ROUND_REFERENCE, algorithm=_algo(gpu, algo)) \
        .generate_region(dev.region).download()
    assert gpu.last_kernel().startswith(FAMILY[algo]), gpu.last_kernel()
    assert bits_equal(got, want), gpu.last_kernel()


@pytest.mark.parametrize("algo", ["auto", "two_pass", "fused", "per_axis"])
def test_3d_256_fma_within_1e5(gpu, blobs256, algo):
    x, want = blobs256
    dev = gpu.DeviceImage.from_host(gpu.Image(x))
    got = gpu.GaussianFilter(dev, 2.0, rounding=gpu.ROUND_FMA, algorithm=_algo(gpu, algo)) \
        .generate_region(dev.region).download()
    assert normwise(got, want) <= 1e-5, gpu.last_kernel()


def test_3d_256_host_buffers_bit_exact(gpu, blobs256):
    """The host-staged call (slabs copied in and out on three streams)."""
    x, want = blobs256
    got = gpu.GaussianFilter(gpu.Image(x), 2.0).generate_region(gpu.Image(x).region).data
    assert bits_equal(got, want)


@pytest.mark.parametrize("rounding", ["reference", "fma"])
@pytest.mark.parametrize("algo", ["auto", "fused", "per_axis"])
def test_3d_256_stream_full_8_pieces_equals_full(gpu, blobs256, algo, rounding):
    x, want = blobs256
    dev = gpu.DeviceImage.from_host(gpu.Image(x))
    rnd = gpu.ROUND_REFERENCE if rounding == "reference" else gpu.ROUND_FMA
    f = gpu.GaussianFilter(dev, 2.0, rounding=rnd, algorithm=_algo(gpu, algo))
    full = f.generate_region(dev.region).download()
    pieces = gpu.stream_full(f, 8).download()
    assert bits_equal(pieces, full), gpu.last_kernel()
    if rounding == "reference":
        assert bits_equal(pieces, want)
    # the host-buffer form streams one slab at a time through the device
    host = gpu.stream_full(gpu.GaussianFilter(gpu.Image(x), 2.0, rounding=rnd,
                                              algorithm=_algo(gpu, algo)), 8).data
    assert bits_equal(host, full)


# ---- CT: i16 512 x 512 x 384, spacing (0.7, 0.7, 2.5), sigma 1.5 mm -----------

CT_SPACING = (0.7, 0.7, 2.5)


@pytest.fixture(scope="module")
def ct():
    v = ct_volume((384, 512, 512), seed=0)
    return v, oracle.gaussian_f32_mt(v.astype(np.float32), 1.5, spacing=CT_SPACING)


def _ct_run(gpu, v, out_dtype, rounding):
    dev = gpu.DeviceImage.from_host(gpu.Image(v, spacing=CT_SPACING))
    f = gpu.GaussianFilter(gpu.CastFilter(dev, gpu.F32), 1.5, rounding=rounding)
    return f.generate_region(dev.region, out_dtype=out_dtype).download()


def test_ct_f32_reference_bit_exact_and_fma(gpu, ct):
    v, want = ct
    got = _ct_run(gpu, v, gpu.F32, gpu.ROUND_REFERENCE)
    assert bits_equal(got, want), gpu.last_kernel()
    got = _ct_run(gpu, v, gpu.F32, gpu.ROUND_FMA)
    assert normwise(got, want) <= 1e-5, gpu.last_kernel()


@pytest.mark.parametrize("out", ["bf16", "f16"])
def test_ct_half_storage_within_half_ulp_of_fp64(gpu, ct, out):
    v, want32 = ct
    code = gpu.BF16 if out == "bf16" else gpu.F16
    raw = _ct_run(gpu, v, code, gpu.ROUND_FMA)
    if out == "bf16":
        got = (raw.astype(np.uint32) << 16).view(np.float32)
        half_ulp_rel = 2.0 ** -8
    else:
        got = raw.astype(np.float32)
        half_ulp_rel = 2.0 ** -11
    # FP64 oracle slab by slab (bounded memory); the z radius is 2 slices
    for z0 in range(0, 384, 64):
        lo, hi = max(0, z0 - 2), min(384, z0 + 64 + 2)
        # the slab carries the z halo (radius 2), so its slices z0 .. z0 + 63
        # are the whole volume's (a slab end that clamps is the volume's end)
        ref64 = oracle.gaussian_f64(v[lo:hi].astype(np.float64), 1.5, spacing=CT_SPACING)[z0 - lo:z0 - lo + 64]
        g = got[z0:z0 + 64].astype(np.float64)
        err = np.abs(g - ref64)
        assert (err <= np.abs(ref64) * half_ulp_rel * 1.0001 + 1e-4).all(), (out, z0, float(err.max()))
    assert normwise(got, want32) <= 2 * half_ulp_rel


# ---- VJP: 192^3 multi-scale stack, radii up to 24 -----------------------------

def _radii(sigma, spacing=None):
    sp = spacing or [1.0, 1.0, 1.0]
    return [oracle.kernel_radius(sigma, sp[d]) for d in range(3)]


def test_vjp_scale_stack_192_sigma_1_2_4_8(gpu):
    x = blobs_volume((192, 192, 192), 100)
    t = blobs_volume((192, 192, 192), 200)
    sigmas = [1.0, 2.0, 4.0, 8.0]
    dx = gpu.DeviceImage.from_host(gpu.Image(x))
    dt = gpu.DeviceImage.from_host(gpu.Image(t))
    loss, xbar, sb = gpu.scale_stack_loss_vjp(dx, dt, sigmas)
    got_x = xbar.download().astype(np.float64)
    x64, t64 = x.astype(np.float64), t.astype(np.float64)
    want_loss, want_x = 0.0, np.zeros(x.shape)
    for level, s in enumerate(sigmas):
        radii = _radii(s)
        y = oracle.gaussian_whole_f64(x64, s, radii=radii)
        d = y - t64
        want_loss += float((d * d).sum())
        want_x += oracle.gaussian_adjoint_f64(2 * d, s, radii=radii)
        want_s = float((2 * d * oracle.gaussian_dsigma_f64(x64, s, radii=radii)).sum())
        scale = float(np.abs(2 * d).sum() * np.abs(x64).max()) + 1e-30
        assert abs(sb[level] - want_s) <= 1e-5 * scale, (s, sb[level], want_s)
        h = 1e-3
        lp = float(((oracle.gaussian_whole_f64(x64, s + h, radii=radii) - t64) ** 2).sum())
        lm = float(((oracle.gaussian_whole_f64(x64, s - h, radii=radii) - t64) ** 2).sum())
        fd = (lp - lm) / (2 * h)
        assert abs(sb[level] - fd) <= 1e-4 * scale + 1e-6 * abs(fd), (s, sb[level], fd)
    assert abs(loss - want_loss) <= 1e-5 * want_loss
    assert np.abs(got_x - want_x).max() <= 1e-5 * np.abs(want_x).max()


LARGE_R = [((40, 48, 56), 4.5, None), ((36, 44, 52), 6.0, None), ((50, 54, 58), 8.0, None),
           ((30, 70, 64), 4.0, (1.0, 0.5, 0.9)), ((60, 28, 66), 5.2, (0.8, 1.3, 1.0)),
           ((12, 70, 9), 8.0, None),      # lines shorter than the radius, a ragged tile of lines
           ((130, 33, 140), 7.0, None)]   # several tiles along every pass axis


@pytest.mark.parametrize("shape,sigma,spacing", LARGE_R)
def test_vjp_radii_13_to_24(gpu, shape, sigma, spacing):
    """The tiled per-axis adjoint and dual passes for radii 13..24."""
    sp = list(spacing) if spacing else None
    radii = _radii(sigma, sp)
    assert max(radii) > 12 and max(radii) <= 24, radii
    rng = np.random.default_rng(shape[0] + shape[2])
    x = rng.standard_normal(shape).astype(np.float32)
    y = rng.standard_normal(shape).astype(np.float32)
    dx = gpu.DeviceImage.from_host(gpu.Image(x, spacing=spacing))
    dy = gpu.DeviceImage.from_host(gpu.Image(y, spacing=spacing))
    xb, sb = gpu.vjp(dx, dy, sigma)
    want_x = oracle.gaussian_adjoint_f64(y.astype(np.float64), sigma, spacing=sp, radii=radii)
    got_x = xb.download().astype(np.float64)
    assert np.abs(got_x - want_x).max() <= 1e-5 * np.abs(want_x).max(), gpu.last_kernel()
    d64 = oracle.gaussian_dsigma_f64(x.astype(np.float64), sigma, spacing=sp, radii=radii)
    want_s = float((d64 * y.astype(np.float64)).sum())
    scale = float(np.abs(d64 * y).sum()) + 1e-30
    assert abs(sb - want_s) <= 1e-5 * scale, (sb, want_s)
    h = 1e-3
    fp = oracle.gaussian_whole_f64(x.astype(np.float64), sigma + h, spacing=sp, radii=radii)
    fm = oracle.gaussian_whole_f64(x.astype(np.float64), sigma - h, spacing=sp, radii=radii)
    fd = float(((fp - fm) / (2 * h) * y.astype(np.float64)).sum())
    assert abs(sb - fd) <= 1e-4 * scale + 1e-6 * abs(fd), (sb, fd)
