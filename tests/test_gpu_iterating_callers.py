"""GPU parity of the Gaussian callers that iterate: DemonsRegistrationFilter /
DiffeomorphicDemonsRegistrationFilter / SyNRegistrationMethod
(registration_methods.rs:39-148, 211-218) through itkg_demons_registration,
and N4BiasFieldCorrectionFilter / MRIBiasFieldCorrectionFilter
(bias_correction.rs:45-121) through itkg_n4_bias_field_correction, against the
oracle and the golden vectors.  Demons runs every f64 operation with IEEE
rounding and is bit-exact; N4's ln and exp are the device's f64 functions, so
its f32 output is checked within 1e-6 normwise (and the iteration count must
match)."""
import numpy as np
import pytest

import oracle
from test_gpu_parity import bits_equal, normwise
from test_oracle_iterating_callers import DEMONS, N4, demons_meta, n4_meta

pytestmark = pytest.mark.gpu


def run_demons(itkg, fixed, moving, iters, step=2.0, diffeo=False, sigma=1.0, host=False, fixed_index=None,
               moving_index=None):
    fi = itkg.Image(fixed, index=fixed_index)
    mi = itkg.Image(moving, index=moving_index)
    f = fi if host else itkg.DeviceImage.from_host(fi)
    m = mi if host else itkg.DeviceImage.from_host(mi)
    if diffeo:
        filt = itkg.DiffeomorphicDemonsRegistrationFilter(f, m, iters, sigma_diff=sigma)
        filt.max_step_length = step
    else:
        filt = itkg.DemonsRegistrationFilter(f, m, iters, step)
    out = filt.compute()
    return out.data if host else out.download()


def smooth_pair(h, w, margin, seed, shift=(1.5, -1.0)):
    """Smooth fixed / moving images that are zero within `margin` of the edges
    (so the field stays zero there and no warped index leaves the image)."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    f = np.zeros((h, w))
    m = np.zeros((h, w))
    for _ in range(6):
        cy, cx = rng.uniform(margin + 8, h - margin - 8), rng.uniform(margin + 8, w - margin - 8)
        r = rng.uniform(4, 8)
        f += np.maximum(0.0, 1.0 - np.hypot(xx - cx, yy - cy) / r)
        m += np.maximum(0.0, 1.0 - np.hypot(xx - cx - shift[0], yy - cy - shift[1]) / r)
    return f.astype(np.float32), m.astype(np.float32)


@pytest.mark.parametrize("host", [False, True])
@pytest.mark.parametrize("name", DEMONS)
def test_demons_golden_bit_exact(gpu, golden, name, host):
    iters, step, diffeo, sigma = demons_meta(golden, name)
    got = run_demons(gpu, golden[f"dem_{name}__fixed"], golden[f"dem_{name}__moving"], iters, step, diffeo, sigma,
                     host=host)
    assert bits_equal(got, golden[f"dem_{name}__out"]), gpu.last_kernel()


@pytest.mark.parametrize("diffeo", [False, True])
def test_demons_against_oracle(gpu, diffeo):
    fixed, moving = smooth_pair(96, 130, 12, 3)
    if diffeo:
        want = oracle.diffeomorphic_demons(fixed, moving, 8, sigma_diff=1.3, max_step_length=0.5)
    else:
        want = oracle.demons_f32(fixed, moving, 8, 0.5)
    got = run_demons(gpu, fixed, moving, 8, 0.5, diffeo, 1.3)
    assert np.abs(want).max() > 0.1  # the field moved
    assert bits_equal(got, want)


def test_demons_offset_regions(gpu):
    """Fixed and moving regions at different indices: the warped index is read
    through the moving image's own region (registration_methods.rs:64-66)."""
    fixed, moving = smooth_pair(40, 50, 8, 4)
    big = np.zeros((44, 54), np.float32)  # the moving image's region (1, -4) + 54 x 44 covers the fixed one
    big[2:42, 2:52] = moving
    want = oracle.demons_f32(fixed, big, 5, 1.0, fixed_index=(3, -2), moving_index=(1, -4))
    got = run_demons(gpu, fixed, big, 5, 1.0, fixed_index=(3, -2), moving_index=(1, -4))
    assert np.abs(want).max() > 0.1
    assert bits_equal(got, want)


def test_syn_is_diffeomorphic_demons_of_the_iteration_sum(gpu):
    fixed, moving = smooth_pair(48, 64, 16, 5, shift=(0.5, 0.5))
    f = gpu.DeviceImage.from_host(gpu.Image(fixed))
    m = gpu.DeviceImage.from_host(gpu.Image(moving))
    got = gpu.SyNRegistrationMethod(f, m, iterations=(3, 2, 1)).compute().download()
    want = oracle.diffeomorphic_demons(fixed, moving, 6, sigma_diff=1.0)
    assert bits_equal(got, want)


def test_demons_warped_index_outside_is_refused(gpu):
    from itkg import _abi
    yy, xx = np.mgrid[0:6, 0:6]
    fixed = (xx + yy).astype(np.float32)
    ok = run_demons(gpu, fixed, fixed + 1.0, 2)
    assert bits_equal(ok, oracle.demons_f32(fixed, fixed + 1.0, 2))
    with pytest.raises(_abi.ItkgError) as ei:
        run_demons(gpu, fixed, fixed + 1.0, 4)
    assert ei.value.status == _abi.ERROR_INVALID_ARGUMENT


def run_n4(itkg, img, iters, sigma, thr, spacing=None, host=False, mri=False):
    im = itkg.Image(img, spacing=spacing)
    src = im if host else itkg.DeviceImage.from_host(im)
    f = itkg.MRIBiasFieldCorrectionFilter(src, iterations=iters) if mri else \
        itkg.N4BiasFieldCorrectionFilter(src, iters, sigma, thr)
    out = f.generate_region()
    return (out.data if host else out.download()), f.iterations_run


@pytest.mark.parametrize("host", [False, True])
@pytest.mark.parametrize("name", N4)
def test_n4_golden(gpu, golden, name, host):
    iters, sigma, thr, run, sp = n4_meta(golden, name)
    got, got_run = run_n4(gpu, golden[f"n4_{name}__in"], iters, sigma, thr, sp, host=host)
    want = golden[f"n4_{name}__out"]
    assert got_run == run
    assert normwise(got, want) <= 1e-6


@pytest.mark.parametrize("sigma,iters", [(30.0, 4), (8.0, 6), (2.5, 3)])
def test_n4_against_oracle(gpu, sigma, iters):
    rng = np.random.default_rng(int(sigma * 10))
    h, w = 200, 256
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    bias = 1.0 + 0.4 * (xx / w) - 0.2 * (yy / h) + 0.1 * np.sin(xx / 40.0)
    base = np.where((xx - 128) ** 2 / 90.0 ** 2 + (yy - 100) ** 2 / 70.0 ** 2 < 1.0, 120.0, 60.0)
    img = (base * bias + rng.normal(0, 2, base.shape)).astype(np.float32)
    want, run = oracle.n4(img, iters, sigma, 1e-3)
    got, got_run = run_n4(gpu, img, iters, sigma, 1e-3)
    assert got_run == run
    assert normwise(got, want) <= 1e-6
    # the device's ln / exp differ from the host's in the last bit at most:
    # nearly every f32 output is identical
    assert np.mean(got.view(np.uint32) == want.view(np.uint32)) > 0.99


def test_mri_bias_is_n4_with_sigma_20(gpu):
    img = np.full((4, 4), 5.0, np.float32)
    got, run = run_n4(gpu, img, 3, None, None, mri=True)
    want, wrun = oracle.n4(img, 3, 20.0, 1e-3)
    assert run == wrun and normwise(got, want) <= 1e-6
