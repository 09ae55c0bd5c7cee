"""Batched execution (itkg_batch_*): many volumes of uneven sizes and sigmas,
planned once, replayed as one CUDA graph.  Every batched output must equal the
same request run alone through itkg_gaussian_generate_region (bit-exact, the
same kernels run), and the VJP items must equal itkg_gaussian_vjp."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _volumes(gpu, rng, n, lo=8, hi=48, comps=1, dim=3):
    out = []
    for _ in range(n):
        shape = tuple(int(v) for v in rng.integers(lo, hi + 1, dim))
        arr = rng.random(shape + ((comps,) if comps > 1 else ()), dtype=np.float32)
        sigma = float(rng.uniform(0.5, 4.0))
        out.append((arr, sigma))
    return out


@pytest.mark.parametrize("rounding", ["reference", "fma"])
@pytest.mark.parametrize("autotune", [True, False])
def test_batch_forward_equals_single_calls(gpu, rounding, autotune):
    rng = np.random.default_rng(123)
    rnd = gpu.ROUND_REFERENCE if rounding == "reference" else gpu.ROUND_FMA
    vols = _volumes(gpu, rng, 10)
    b = gpu.Batch()
    outs, devs = [], []
    for arr, sigma in vols:
        d = gpu.DeviceImage.from_host(gpu.Image(arr))
        devs.append(d)
        outs.append(b.add(d, sigma, rounding=rnd))
    b.plan(autotune=autotune)
    assert b.describe().strip()
    for rep in range(2):
        for o in outs:  # poison outputs so the replay must rewrite them
            from itkg import _abi
            sx, sy, sz = o.region.size
            nbytes = (sz - 1) * o.c.pitch[2] + (sy - 1) * o.c.pitch[1] + sx * o.c.pitch[0]
            _abi.check(_abi.lib().itkg_memset_device(ctypes.c_void_p(o.c.data), 0xFF, nbytes, None))
        b.run()
        gpu.Stream().synchronize()
        for (arr, sigma), o in zip(vols, outs):
            got = o.download()
            want = oracle.gaussian_f32(arr, sigma)
            if rnd == gpu.ROUND_REFERENCE:
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (arr.shape, sigma)
            else:
                assert np.abs(got - want).max() / np.abs(want).max() <= 1e-5


def test_batch_mixed_2d_vecpixel_and_3d(gpu):
    rng = np.random.default_rng(5)
    b = gpu.Batch()
    cases = []
    for _ in range(4):
        shape = tuple(int(v) for v in rng.integers(16, 80, 2))
        arr = rng.random(shape + (3,), dtype=np.float32)
        sigma = float(rng.uniform(0.5, 4.0))
        d = gpu.DeviceImage.from_host(gpu.Image(arr, components=3))
        cases.append((arr, sigma, 3, b.add(d, sigma, rounding=gpu.ROUND_REFERENCE)))
    for arr, sigma in _volumes(gpu, rng, 3):
        d = gpu.DeviceImage.from_host(gpu.Image(arr))
        cases.append((arr, sigma, 1, b.add(d, sigma, rounding=gpu.ROUND_REFERENCE)))
    b.plan()
    b.run()
    gpu.Stream().synchronize()
    for arr, sigma, comps, o in cases:
        want = oracle.gaussian_f32(arr, sigma, comps=comps)
        assert np.array_equal(o.download().view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("rounding", ["reference", "fma"])
def test_batch_2d_items_in_multi_request_tile_launches(gpu, rounding):
    """2-D items (1, 2 and 3 components, radii 1..12, sub-regions of images
    with offset indices, several items per kernel class) run as multi-request
    tile launches, one per class; each output equals the oracle (bit-exact in
    reference rounding) and replays rewrite it."""
    from itkg import _abi
    rnd = gpu.ROUND_REFERENCE if rounding == "reference" else gpu.ROUND_FMA
    rng = np.random.default_rng(77)
    b = gpu.Batch()
    cases = []
    for i in range(24):
        comps = (1, 2, 3)[i % 3]
        shape = tuple(int(v) for v in rng.integers(20, 300, 2))
        arr = rng.standard_normal(shape + ((comps,) if comps > 1 else ())).astype(np.float32)
        sigma = (0.6, 1.5, 2.2, 4.0)[i % 4]
        index = (int(rng.integers(-5, 5)), int(rng.integers(-5, 5)))
        img = gpu.Image(arr, index=index, components=comps)
        d = gpu.DeviceImage.from_host(img)
        req = None
        if i % 2:
            ri = (index[0] + shape[1] // 4, index[1] + shape[0] // 3)
            req = (ri, (shape[1] // 2, shape[0] // 2))
        o = b.add(d, sigma, rounding=rnd, requested=gpu.Region(*req) if req else None)
        cases.append((arr, sigma, comps, index, req, o))
    b.plan()
    plan = b.describe()
    assert "tile2d" in plan and "multi-request" in plan, plan
    for rep in range(2):
        for *_, o in cases:  # poison the outputs so the replay must rewrite them
            sx, sy = o.region.size[:2]
            nbytes = (sy - 1) * o.c.pitch[1] + sx * o.c.pitch[0]
            _abi.check(_abi.lib().itkg_memset_device(ctypes.c_void_p(o.c.data), 0xFF, nbytes, None))
        b.run()
        gpu.Stream().synchronize()
        for arr, sigma, comps, index, req, o in cases:
            want = oracle.gaussian_f32(arr, sigma, comps=comps, index=index, requested=req)
            got = o.download()
            if rnd == gpu.ROUND_REFERENCE:
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (arr.shape, sigma, req)
            else:
                assert np.abs(got - want).max() / np.abs(want).max() <= 1e-5


def test_batch_vjp_items_match_single_vjp(gpu):
    from itkg import _abi
    L = _abi.lib()
    rng = np.random.default_rng(9)
    n = 3
    sb = ctypes.c_void_p()
    _abi.check(L.itkg_device_alloc(8 * n, ctypes.byref(sb)))
    _abi.check(L.itkg_memset_device(sb, 0, 8 * n, None))
    b = gpu.Batch()
    items = []
    for i, (arr, sigma) in enumerate(_volumes(gpu, rng, n)):
        ybar = rng.standard_normal(arr.shape).astype(np.float32)
        dx = gpu.DeviceImage.from_host(gpu.Image(arr))
        dy = gpu.DeviceImage.from_host(gpu.Image(ybar))
        xb = b.add_vjp(dx, dy, sigma, sigma_bar_dev=sb.value + 8 * i)
        items.append((dx, dy, sigma, xb))
    b.plan()
    b.run()
    gpu.Stream().synchronize()
    host = (ctypes.c_double * n)()
    _abi.check(L.itkg_memcpy(ctypes.cast(host, ctypes.c_void_p), sb, 8 * n, 1, None))
    _abi.check(L.itkg_stream_synchronize(None))
    for i, (dx, dy, sigma, xb) in enumerate(items):
        want_x, want_s = gpu.vjp(dx, dy, sigma)
        assert np.array_equal(xb.download(), want_x.download())
        assert host[i] == pytest.approx(want_s, rel=1e-12, abs=1e-12)
    L.itkg_device_free(sb)
