"""GPU VJP checks (the reference has no VJP; these follow the specification):
FP64 dot-product test <Gx, y> = <x, G^T y>, the adjoint against an FP64
numpy adjoint, dL/dsigma against the FP64 analytic derivative and against
central finite differences (h = 1e-3, radius frozen at r(sigma))."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

SHAPES = [((40,), 2.0, None), ((33, 45), 1.5, None), ((17, 23, 29), 1.2, None),
          ((24, 20, 16), 2.0, (0.7, 0.9, 2.5)), ((6, 5, 4), 3.0, None), ((1, 9, 1), 1.0, None),
          ((48, 40, 36), 4.0, None)]


def _dev(itkg, arr, spacing=None):
    return itkg.DeviceImage.from_host(itkg.Image(np.ascontiguousarray(arr, np.float32), spacing=spacing))


def _radii(sigma, spacing, D):
    sp = spacing or [1.0] * D
    return [oracle.kernel_radius(sigma, sp[d]) for d in range(D)]


@pytest.mark.parametrize("shape,sigma,spacing", SHAPES)
def test_dot_product_identity(gpu, shape, sigma, spacing):
    rng = np.random.default_rng(len(shape) * 100 + shape[0])
    x = rng.standard_normal(shape).astype(np.float32)
    y = rng.standard_normal(shape).astype(np.float32)
    dx, dy = _dev(gpu, x, spacing), _dev(gpu, y, spacing)
    Gx = gpu.GaussianFilter(dx, sigma, rounding=gpu.ROUND_FMA).generate_region(dx.region).download()
    GTy, _ = gpu.vjp(dx, dy, sigma, want_sigma=False)
    GTy = GTy.download()
    lhs = float(np.dot(Gx.astype(np.float64).ravel(), y.astype(np.float64).ravel()))
    rhs = float(np.dot(x.astype(np.float64).ravel(), GTy.astype(np.float64).ravel()))
    scale = float(np.abs(Gx).sum() * np.abs(y).max()) + 1e-30
    assert abs(lhs - rhs) <= 1e-6 * scale, (lhs, rhs)


@pytest.mark.parametrize("shape,sigma,spacing", SHAPES)
def test_adjoint_matches_fp64(gpu, shape, sigma, spacing):
    rng = np.random.default_rng(7 + shape[0])
    x = rng.standard_normal(shape).astype(np.float32)
    y = rng.standard_normal(shape).astype(np.float32)
    got, _ = gpu.vjp(_dev(gpu, x, spacing), _dev(gpu, y, spacing), sigma, want_sigma=False)
    want = oracle.gaussian_adjoint_f64(y.astype(np.float64), sigma, spacing=list(spacing) if spacing else None)
    got = got.download().astype(np.float64)
    assert np.abs(got - want).max() / np.abs(want).max() <= 1e-5


@pytest.mark.parametrize("shape,sigma,spacing", SHAPES)
def test_sigma_bar_matches_fp64_and_finite_differences(gpu, shape, sigma, spacing):
    rng = np.random.default_rng(11 + shape[-1])
    x = rng.random(shape).astype(np.float32)
    ybar = rng.standard_normal(shape).astype(np.float32)
    sp = list(spacing) if spacing else None
    _, sb = gpu.vjp(_dev(gpu, x, spacing), _dev(gpu, ybar, spacing), sigma)
    radii = _radii(sigma, sp, len(shape))
    d64 = oracle.gaussian_dsigma_f64(x.astype(np.float64), sigma, spacing=sp, radii=radii)
    want = float((d64 * ybar.astype(np.float64)).sum())
    scale = float(np.abs(d64 * ybar).sum()) + 1e-30
    assert abs(sb - want) <= 1e-5 * scale, (sb, want)
    h = 1e-3
    fp = oracle.gaussian_whole_f64(x.astype(np.float64), sigma + h, spacing=sp, radii=radii)
    fm = oracle.gaussian_whole_f64(x.astype(np.float64), sigma - h, spacing=sp, radii=radii)
    fd = float(((fp - fm) / (2 * h) * ybar.astype(np.float64)).sum())
    assert abs(sb - fd) <= 1e-4 * scale + 1e-6 * abs(fd), (sb, fd)


@pytest.mark.parametrize("shape,sigma", [((40, 50, 60), 2.0), ((17, 23, 29), 1.2), ((5, 70, 40), 0.9),
                                         ((33, 8, 41), 1.7)])
def test_fused_vjp_matches_fp64_and_is_used(gpu, shape, sigma):
    """3-D radii <= 6 run the fused adjoint and dot kernels; check them against
    FP64 and against the dot-product identity."""
    rng = np.random.default_rng(shape[0] * 7 + shape[2])
    x = rng.standard_normal(shape).astype(np.float32)
    y = rng.standard_normal(shape).astype(np.float32)
    dx, dy = _dev(gpu, x), _dev(gpu, y)
    xb, sb = gpu.vjp(dx, dy, sigma, algorithm=gpu.ALGO_FUSED)
    assert gpu.last_kernel() == "vjp_fused_f32", gpu.last_kernel()
    want_x = oracle.gaussian_adjoint_f64(y.astype(np.float64), sigma)
    got_x = xb.download().astype(np.float64)
    assert np.abs(got_x - want_x).max() / np.abs(want_x).max() <= 1e-5
    radii = _radii(sigma, None, 3)
    d64 = oracle.gaussian_dsigma_f64(x.astype(np.float64), sigma, radii=radii)
    want_s = float((d64 * y.astype(np.float64)).sum())
    assert abs(sb - want_s) <= 1e-5 * float(np.abs(d64 * y).sum())
    Gx = gpu.GaussianFilter(dx, sigma, rounding=gpu.ROUND_FMA).generate_region(dx.region).download()
    lhs = float(np.dot(Gx.astype(np.float64).ravel(), y.astype(np.float64).ravel()))
    rhs = float(np.dot(x.astype(np.float64).ravel(), got_x.ravel()))
    assert abs(lhs - rhs) <= 1e-6 * float(np.abs(Gx).sum() * np.abs(y).max())


def test_accumulate_flags(gpu):
    rng = np.random.default_rng(3)
    x = rng.random((12, 14, 16)).astype(np.float32)
    y = rng.standard_normal((12, 14, 16)).astype(np.float32)
    dx, dy = _dev(gpu, x), _dev(gpu, y)
    base, sb = gpu.vjp(dx, dy, 1.3)
    start = rng.standard_normal((12, 14, 16)).astype(np.float32)
    acc = _dev(gpu, start)
    out, sb2 = gpu.vjp(dx, dy, 1.3, xbar=acc, sigma_bar_init=2.5,
                       flags=gpu.VJP_ACCUMULATE_XBAR | gpu.VJP_ACCUMULATE_SIGMA)
    assert np.allclose(out.download(), start + base.download(), rtol=0, atol=1e-6)
    assert abs(sb2 - (sb + 2.5)) < 1e-9 * max(1.0, abs(sb))


@pytest.mark.parametrize("shape", [(20, 18, 22), (9, 30, 7), (20, 18, 24), (12, 40, 32)])
def test_scale_stack_loss_vjp_matches_fp64(gpu, shape):
    """L = sum_l |G_l x - t|^2 over sigmas {1, 2, 4}: loss, dL/dx, dL/dsigma_l
    against FP64 numpy, and dL/dsigma_l against central differences."""
    rng = np.random.default_rng(sum(shape))
    x = rng.random(shape).astype(np.float32)
    t = rng.random(shape).astype(np.float32)
    sigmas = [1.0, 2.0, 4.0]
    loss, xbar, sb = gpu.scale_stack_loss_vjp(_dev(gpu, x), _dev(gpu, t), sigmas)
    # rows of a multiple of 4 floats take the two-pass kernels at every level
    assert gpu.last_kernel() == ("scale_stack_loss_vjp_two_pass_f32" if shape[2] % 4 == 0
                                 else "scale_stack_loss_vjp_per_axis_f32"), gpu.last_kernel()
    x64, t64 = x.astype(np.float64), t.astype(np.float64)
    want_loss, want_x, want_s = 0.0, np.zeros(shape), []
    for s in sigmas:
        radii = _radii(s, None, 3)
        y = oracle.gaussian_whole_f64(x64, s, radii=radii)
        d = y - t64
        want_loss += float((d * d).sum())
        want_x += oracle.gaussian_adjoint_f64(2 * d, s, radii=radii)
        want_s.append(float((2 * d * oracle.gaussian_dsigma_f64(x64, s, radii=radii)).sum()))
        h = 1e-3
        lp = ((oracle.gaussian_whole_f64(x64, s + h, radii=radii) - t64) ** 2).sum()
        lm = ((oracle.gaussian_whole_f64(x64, s - h, radii=radii) - t64) ** 2).sum()
        fd = (lp - lm) / (2 * h)
        assert abs(want_s[-1] - fd) <= 1e-5 * max(1.0, abs(fd))
    assert abs(loss - want_loss) <= 1e-5 * want_loss
    got_x = xbar.download().astype(np.float64)
    assert np.abs(got_x - want_x).max() <= 1e-5 * np.abs(want_x).max()
    for g, w in zip(sb, want_s):
        assert abs(g - w) <= 1e-4 * max(1.0, abs(w)), (sb, want_s)


def test_vjp_rejects_bad_sigma(gpu):
    from itkg import _abi
    x = _dev(gpu, np.zeros((4, 5, 6), np.float32))
    with pytest.raises(_abi.ItkgError):
        gpu.vjp(x, x, 0.0)
    with pytest.raises(_abi.ItkgError):
        gpu.vjp(x, x, float("nan"))


def test_per_axis_algorithm_forces_per_axis_vjp(gpu):
    """params.algorithm = per-axis keeps the VJP to the per-axis passes; both
    forms agree within the FMA tolerance."""
    from itkg import _abi
    import ctypes
    rng = np.random.default_rng(61)
    x = rng.standard_normal((30, 34, 38)).astype(np.float32)
    y = rng.standard_normal((30, 34, 38)).astype(np.float32)
    dx, dy = _dev(gpu, x), _dev(gpu, y)
    xb_f, sb_f = gpu.vjp(dx, dy, 1.4, algorithm=gpu.ALGO_FUSED)
    assert gpu.last_kernel() == "vjp_fused_f32", gpu.last_kernel()
    xb = gpu.DeviceImage(dx.region)
    p = _abi.itkg_gaussian_params()
    p.sigma, p.rounding, p.algorithm = 1.4, gpu.ROUND_FMA, gpu.ALGO_PER_AXIS
    sb = ctypes.c_double(0.0)
    _abi.check(_abi.lib().itkg_gaussian_vjp(ctypes.byref(dx.c), ctypes.byref(dy.c), ctypes.byref(p),
                                           ctypes.byref(xb.c), ctypes.byref(sb), 0, None))
    assert gpu.last_kernel() == "vjp_per_axis_f32", gpu.last_kernel()
    a, b = xb.download().astype(np.float64), xb_f.download().astype(np.float64)
    assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max()
    assert abs(sb.value - sb_f) <= 1e-5 * max(1.0, abs(sb_f))


TWO_PASS_VJP = [((40, 50, 60), 2.0, None), ((17, 23, 29), 1.2, None), ((5, 70, 40), 0.9, None),
                ((33, 8, 41), 1.7, None), ((6, 5, 4), 3.0, None), ((1, 9, 1), 1.0, None),
                ((48, 40, 36), 4.0, None), ((30, 70, 90), 3.4, None), ((20, 30, 40), 2.0, (1.0, 1.0, 2.0)),
                ((64, 130, 33), 1.5, (0.8, 0.8, 1.0))]


@pytest.mark.parametrize("shape,sigma,spacing", TWO_PASS_VJP)
def test_two_pass_vjp_matches_fp64(gpu, shape, sigma, spacing):
    """z-adjoint + x-y kernels (radii up to 12, thin images, anisotropic z):
    dL/dx against the FP64 adjoint, dL/dsigma against the FP64 analytic
    derivative, and the dot-product identity against the GPU forward."""
    rng = np.random.default_rng(shape[1] * 3 + shape[2])
    x = rng.standard_normal(shape).astype(np.float32)
    y = rng.standard_normal(shape).astype(np.float32)
    sp = list(spacing) if spacing else None
    dx, dy = _dev(gpu, x, spacing), _dev(gpu, y, spacing)
    xb, sb = gpu.vjp(dx, dy, sigma)
    assert gpu.last_kernel() == "vjp_two_pass_f32", gpu.last_kernel()
    radii = _radii(sigma, sp, 3)
    want_x = oracle.gaussian_adjoint_f64(y.astype(np.float64), sigma, spacing=sp)
    got_x = xb.download().astype(np.float64)
    assert np.abs(got_x - want_x).max() <= 1e-5 * np.abs(want_x).max()
    d64 = oracle.gaussian_dsigma_f64(x.astype(np.float64), sigma, spacing=sp, radii=radii)
    want_s = float((d64 * y.astype(np.float64)).sum())
    assert abs(sb - want_s) <= 1e-5 * float(np.abs(d64 * y).sum()), (sb, want_s)
    Gx = gpu.GaussianFilter(dx, sigma, rounding=gpu.ROUND_FMA).generate_region(dx.region).download()
    lhs = float(np.dot(Gx.astype(np.float64).ravel(), y.astype(np.float64).ravel()))
    rhs = float(np.dot(x.astype(np.float64).ravel(), got_x.ravel()))
    assert abs(lhs - rhs) <= 1e-6 * float(np.abs(Gx).sum() * np.abs(y).max())


def test_two_pass_vjp_accumulate_and_partial_requests(gpu):
    rng = np.random.default_rng(9)
    shape = (21, 35, 44)
    x = rng.random(shape).astype(np.float32)
    y = rng.standard_normal(shape).astype(np.float32)
    dx, dy = _dev(gpu, x), _dev(gpu, y)
    base, sb = gpu.vjp(dx, dy, 2.2)
    assert gpu.last_kernel() == "vjp_two_pass_f32"
    start = rng.standard_normal(shape).astype(np.float32)
    acc = _dev(gpu, start)
    out, sb2 = gpu.vjp(dx, dy, 2.2, xbar=acc, sigma_bar_init=-1.5,
                       flags=gpu.VJP_ACCUMULATE_XBAR | gpu.VJP_ACCUMULATE_SIGMA)
    assert np.allclose(out.download(), start + base.download(), rtol=0, atol=1e-6)
    assert abs(sb2 - (sb - 1.5)) < 1e-9 * max(1.0, abs(sb))
    # the same request again into a fresh buffer: the same dL/dsigma (a fixed reduction order)
    _, sb3 = gpu.vjp(dx, dy, 2.2, xbar=gpu.DeviceImage(dx.region))
    assert abs(sb3 - sb) <= 1e-12 * max(1.0, abs(sb))
