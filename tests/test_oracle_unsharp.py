"""Pin the oracle's UnsharpMaskFilter (oracle.unsharp_mask) before trusting it.

The reference has no test of its own for UnsharpMaskFilter (edges.rs:374-452),
so the oracle is pinned through its parts: the blur is the convolve_axis
family restatement (pinned by the `sep_*` cases and the reference's mean /
binomial tests), and the whole filter is checked bit-exact against the `ush_*`
cases of tests/golden/golden.npz, written by the independent pure-Python
transcription in tests/golden/make_golden.py.
"""
import math

import numpy as np
import pytest

import oracle

USH = ["f32_2d_s1", "f32_2d_sub_s1p3", "f32_3d_s0p8", "f32_1d_s2", "vec2d_s1", "u8_2d_s1p5"]


def ush_meta(golden, name):
    m = golden[f"ush_{name}__meta"]
    sigma, amount, threshold, comps = float(m[0]), float(m[1]), float(m[2]), int(m[3])
    rest = [int(v) for v in m[4:]]
    D = len(rest) // 2
    return sigma, amount, threshold, comps, (tuple(rest[:D]), tuple(rest[D:]))


@pytest.mark.parametrize("name", USH)
def test_unsharp_oracle_matches_golden(golden, name):
    sigma, amount, threshold, comps, req = ush_meta(golden, name)
    x = golden[f"ush_{name}__in"]
    got = oracle.unsharp_mask(x, sigma, amount, threshold, requested=req, comps=comps)
    want = golden[f"ush_{name}__out"]
    assert got.dtype == want.dtype and got.shape == want.shape
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))


@pytest.mark.parametrize("sigma", [0.2, 0.5, 1.0, 1.3, 2.0, 3.7, 6.0])
def test_unsharp_kernel(sigma):
    k = oracle.unsharp_kernel(sigma)
    r = math.ceil(3.0 * sigma)
    assert len(k) == 2 * r + 1
    assert np.array_equal(k, k[::-1])
    assert abs(k.sum() - 1.0) < 1e-12
    assert np.argmax(k) == r


def test_identity_cases():
    x = np.random.default_rng(5).random((9, 10, 11), dtype=np.float32)
    # no voxel passes an infinite threshold; amount 0 adds nothing
    assert np.array_equal(oracle.unsharp_mask(x, 1.0, 0.8, np.inf), x)
    assert np.array_equal(oracle.unsharp_mask(x, 1.0, 0.0, 0.0), x)


def test_sharpening_raises_contrast_at_a_step():
    x = np.zeros((1, 20), np.float32)
    x[:, 10:] = 1.0
    y = oracle.unsharp_mask(x, 1.0, 1.0, 0.0)
    assert y[0, 9] < 0.0 < 1.0 < y[0, 10]  # under- and overshoot either side of the edge
    # far from the edge: 0 stays 0; the f32 blur of ones is 1 - 2^-24, so 1 comes back 1 + 2^-23
    assert y[0, 0] == 0.0 and abs(float(y[0, -1]) - 1.0) <= 2.0 ** -23
