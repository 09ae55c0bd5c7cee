"""Pin the oracle's in-crate callers of GaussianFilter -- SliceBySliceFilter
(spatial.rs:1284-1340), BSplineDownsampleFilter (spatial.rs:1128-1166) and
DisplacementFieldToBSplineFilter (spatial.rs:1484-1525) --
against the `cal_*` cases of tests/golden/golden.npz (the pure-Python
transcription in tests/golden/make_golden.py).  The reference has no tests of
its own for these filters."""
import numpy as np
import pytest

import oracle


def slice_meta(golden, name):
    m = golden[f"cal_{name}__meta"]
    sigma, sp = float(m[1]), [float(v) for v in m[2:5]]
    r = [int(v) for v in m[5:11]]
    return sigma, sp, (tuple(r[:3]), tuple(r[3:]))


@pytest.mark.parametrize("name", ["slices_s1p2", "slices_u8_s1"])
def test_slice_by_slice_oracle_matches_golden(golden, name):
    sigma, sp, req = slice_meta(golden, name)
    got = oracle.slice_by_slice(golden[f"cal_{name}__in"], sigma, sp, requested=req)
    want = golden[f"cal_{name}__out"]
    assert got.dtype == want.dtype and np.array_equal(got.view(np.uint8), want.view(np.uint8))


@pytest.mark.parametrize("name", ["bspline3d_odd", "bspline2d_aniso"])
def test_bspline_downsample_oracle_matches_golden(golden, name):
    x = golden[f"cal_{name}__in"]
    sp = [float(v) for v in golden[f"cal_{name}__meta"][2:]]
    got = oracle.bspline_downsample(x, sp)
    want = golden[f"cal_{name}__out"]
    assert got.shape == tuple((n + 1) // 2 for n in x.shape)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_slice_by_slice_leaves_z_alone():
    """A volume constant along x and y but varying along z is returned unchanged:
    the slices are smoothed independently."""
    z = np.arange(6, dtype=np.float32)[:, None, None] * np.ones((1, 5, 7), np.float32)
    out = oracle.slice_by_slice(z, 1.5)
    assert np.all(np.abs(out - z) <= 1e-6 * np.maximum(1.0, np.abs(z)))


def dfb_meta(golden, name):
    m = golden[f"cal_{name}__meta"]
    return float(m[1]), ((int(m[2]), int(m[3])), (int(m[4]), int(m[5])))


@pytest.mark.parametrize("name", ["dfbspline_s2", "dfbspline_sub_s1p5"])
def test_displacement_field_to_bspline_oracle_matches_golden(golden, name):
    sigma, req = dfb_meta(golden, name)
    got = oracle.displacement_field_to_bspline(golden[f"cal_{name}__in"], sigma, requested=req)
    assert np.array_equal(got.view(np.uint32), golden[f"cal_{name}__out"].view(np.uint32))


def test_displacement_field_to_bspline_clamps_at_the_request():
    """The Gaussian's largest region is the request: a sub-region result equals
    the whole-field filter run on the crop, not the crop of the whole-field result."""
    f = np.random.default_rng(3).standard_normal((20, 24, 2)).astype(np.float32)
    req = ((5, 4), (12, 10))
    sub = oracle.displacement_field_to_bspline(f, 1.5, requested=req)
    crop = np.ascontiguousarray(f[4:14, 5:17])
    assert np.array_equal(sub, oracle.displacement_field_to_bspline(crop, 1.5))
    whole = oracle.displacement_field_to_bspline(f, 1.5)
    assert not np.array_equal(sub, whole[4:14, 5:17])
