"""Pin the oracle's Gaussian callers that iterate -- DemonsRegistrationFilter
(registration_methods.rs:39-100), DiffeomorphicDemonsRegistrationFilter
(:126-148) and N4BiasFieldCorrectionFilter (bias_correction.rs:45-83) --
against the `dem_*` / `n4_*` cases of tests/golden/golden.npz (the pure-Python
transcription in tests/golden/make_golden.py), and re-run the reference's own
tests of these filters (registration_methods.rs:487-503,
bias_correction.rs:131-150) on the oracle."""
import numpy as np
import pytest

import oracle

DEMONS = ["blob_3", "blob_6_step05", "blob_3_diffeo"]
N4 = ["default", "s2_aniso", "s1_one"]


def demons_meta(golden, name):
    m = golden[f"dem_{name}__meta"]
    return int(m[0]), float(m[1]), bool(m[2]), float(m[3])


def n4_meta(golden, name):
    m = golden[f"n4_{name}__meta"]
    return int(m[0]), float(m[1]), float(m[2]), int(m[3]), [float(m[4]), float(m[5])]


@pytest.mark.parametrize("name", DEMONS)
def test_demons_oracle_matches_golden(golden, name):
    iters, step, diffeo, sigma = demons_meta(golden, name)
    fixed, moving = golden[f"dem_{name}__fixed"], golden[f"dem_{name}__moving"]
    if diffeo:
        got = oracle.diffeomorphic_demons(fixed, moving, iters, sigma_diff=sigma, max_step_length=step)
    else:
        got = oracle.demons_f32(fixed, moving, iters, step)
    want = golden[f"dem_{name}__out"]
    assert got.shape == want.shape and np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("name", N4)
def test_n4_oracle_matches_golden(golden, name):
    iters, sigma, thr, run, sp = n4_meta(golden, name)
    got, got_run = oracle.n4(golden[f"n4_{name}__in"], iters, sigma, thr, spacing=sp)
    assert got_run == run
    assert np.array_equal(got.view(np.uint32), golden[f"n4_{name}__out"].view(np.uint32))


def checkerboard(w, h):
    """The reference's test image (registration_methods.rs:478-484)."""
    return np.array([[1.0 if (x + y) % 2 == 0 else 0.0 for x in range(w)] for y in range(h)], np.float32)


def test_demons_registration_runs():
    """registration_methods.rs:488-494: identical images, 5 iterations (a zero field)."""
    dx, dy = oracle.demons(checkerboard(8, 8), checkerboard(8, 8), 5)
    assert not dx.any() and not dy.any()


def test_syn_registration_runs():
    """registration_methods.rs:496-502: SyN = diffeomorphic demons with 20 + 10 + 5 iterations."""
    out = oracle.diffeomorphic_demons(checkerboard(8, 8), checkerboard(8, 8), 35)
    assert out.shape == (8, 8, 2) and not out.any()


def test_demons_warped_index_outside_moving_raises():
    """Where the warped index leaves the moving image the reference panics
    (Image::get_pixel, image.rs:122-125); the oracle raises."""
    yy, xx = np.mgrid[0:6, 0:6]
    fixed = (xx + yy).astype(np.float32)  # the field walks towards the first row
    oracle.demons(fixed, fixed + 1.0, 2)  # still inside after two iterations
    with pytest.raises(IndexError):
        oracle.demons(fixed, fixed + 1.0, 4)


def test_n4_constant_image_uniform():
    """bias_correction.rs:131-143: a constant image has no bias."""
    out, _ = oracle.n4(np.full((8, 8), 10.0, np.float32))
    assert np.all(np.abs(out - out.flat[0]) < 0.01)


def test_mri_bias_runs():
    """bias_correction.rs:145-150: MRIBiasFieldCorrectionFilter = N4 with sigma 20, 3 iterations."""
    out, run = oracle.n4(np.full((4, 4), 5.0, np.float32), iterations=3, sigma=20.0)
    assert out.shape == (4, 4) and 1 <= run <= 3
