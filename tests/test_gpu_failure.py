"""Failure paths and concurrent callers, with no GPU fault provoked.

  - A bounded wait that runs out: a test hook lowers the wait limit of the
    kernels' waits on tile loads to one clock cycle on small, valid loads.
    Each kernel that gives up records it in the calling thread's device fault
    word, lets every load it issued land (under the default limit) and
    returns; a device-buffer call leaves the word set (itkg_device_fault
    reports and clears it), a host-buffer call returns ITKG_ERROR_TIMEOUT.
    With the limit restored the next call is bit-exact again.
  - An allocation failure: a test hook makes the next device scratch
    allocation fail; the call returns ITKG_ERROR_OUT_OF_MEMORY and the next
    call works.
  - Concurrent callers: GaussianFilter is Sync in the reference
    (src/filters/gaussian.rs:43-47, S: Sync); four host threads, each on its
    own stream, call generate_region at once and get the oracle's bytes.
"""
import ctypes
import threading

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def _fault(L, clear):
    f = ctypes.c_uint32(0)
    from itkg import _abi
    _abi.check(L.itkg_device_fault(1 if clear else 0, ctypes.byref(f)))
    return f.value


@pytest.fixture
def wait_limit_one_cycle(gpu):
    from itkg import _abi
    L = _abi.lib()
    _fault(L, True)
    L.itkg_debug_set_wait_limit(1)
    try:
        yield L
    finally:
        L.itkg_debug_set_wait_limit(0)
        _fault(L, True)


@pytest.mark.parametrize("algo", ["two_pass", "fused", "one_trip"])
def test_wait_that_runs_out_sets_fault_word_then_recovers(gpu, wait_limit_one_cycle, algo):
    L = wait_limit_one_cycle
    algorithm = {"two_pass": gpu.ALGO_TWO_PASS, "fused": gpu.ALGO_FUSED, "one_trip": gpu.ALGO_ONE_TRIP}[algo]
    rng = np.random.default_rng(1)
    x = rng.random((48, 64, 96), dtype=np.float32)
    dev = gpu.DeviceImage.from_host(gpu.Image(x))
    f = gpu.GaussianFilter(dev, 1.5, rounding=gpu.ROUND_REFERENCE, algorithm=algorithm)
    out = f.generate_region(dev.region)
    out.download()  # synchronises
    assert _fault(L, False) == 1, gpu.last_kernel()
    assert _fault(L, True) == 1
    assert _fault(L, False) == 0
    # a host-buffer call reads the word itself and fails with a timeout
    from itkg import _abi
    with pytest.raises(_abi.ItkgError) as ei:
        gpu.GaussianFilter(gpu.Image(x), 1.5, rounding=gpu.ROUND_REFERENCE,
                           algorithm=algorithm).generate_region(gpu.Image(x).region)
    assert ei.value.status == _abi.ERROR_TIMEOUT
    assert _fault(L, False) == 0  # the failing call cleared it
    # the default limit back: bit-exact, no fault
    L.itkg_debug_set_wait_limit(0)
    got = f.generate_region(dev.region).download()
    assert _fault(L, False) == 0
    assert bits_equal(got, oracle.gaussian_f32(x, 1.5))


def test_vjp_wait_that_runs_out_sets_fault_word(gpu, wait_limit_one_cycle):
    L = wait_limit_one_cycle
    rng = np.random.default_rng(2)
    x = rng.random((40, 48, 64), dtype=np.float32)
    y = rng.standard_normal((40, 48, 64)).astype(np.float32)
    dx = gpu.DeviceImage.from_host(gpu.Image(x))
    dy = gpu.DeviceImage.from_host(gpu.Image(y))
    xb, _ = gpu.vjp(dx, dy, 2.0)
    xb.download()
    assert _fault(L, True) == 1, gpu.last_kernel()
    L.itkg_debug_set_wait_limit(0)
    xb, _ = gpu.vjp(dx, dy, 2.0)
    want = oracle.gaussian_adjoint_f64(y.astype(np.float64), 2.0)
    got = xb.download().astype(np.float64)
    assert _fault(L, False) == 0
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()


def test_fault_word_is_per_thread(gpu, wait_limit_one_cycle):
    """A wait given up under one thread's call does not show in another
    thread's fault word."""
    L = wait_limit_one_cycle
    x = np.random.default_rng(3).random((32, 40, 64), dtype=np.float32)
    dev = gpu.DeviceImage.from_host(gpu.Image(x))
    gpu.GaussianFilter(dev, 1.5, algorithm=gpu.ALGO_TWO_PASS).generate_region(dev.region).download()
    seen = {}

    def other():
        seen["fault"] = _fault(L, False)

    t = threading.Thread(target=other)
    t.start()
    t.join()
    assert seen["fault"] == 0
    assert _fault(L, True) == 1


@pytest.mark.parametrize("after", [0, 1])
def test_injected_allocation_failure(gpu, after):
    from itkg import _abi
    L = _abi.lib()
    rng = np.random.default_rng(4)
    x = rng.random((40, 50, 60), dtype=np.float32)
    img = gpu.Image(x)
    want = oracle.gaussian_f32(x, 1.8)
    # host buffers: the call allocates staging and intermediate scratch
    n0 = L.itkg_scratch_alloc_counter()
    L.itkg_debug_fail_scratch_alloc(after)
    try:
        with pytest.raises(_abi.ItkgError) as ei:
            gpu.GaussianFilter(img, 1.8).generate_region(img.region)
        assert ei.value.status == _abi.ERROR_OUT_OF_MEMORY
        assert "injected" in L.itkg_last_error().decode()
    finally:
        L.itkg_debug_fail_scratch_alloc(-1)
    assert L.itkg_scratch_alloc_counter() - n0 == after
    got = gpu.GaussianFilter(img, 1.8).generate_region(img.region).data
    assert bits_equal(got, want)
    # device buffers: the x-y + z kernels take their intermediate from scratch
    dev = gpu.DeviceImage.from_host(img)
    L.itkg_debug_fail_scratch_alloc(0)
    try:
        with pytest.raises(_abi.ItkgError) as ei:
            gpu.GaussianFilter(dev, 1.8, algorithm=gpu.ALGO_TWO_PASS).generate_region(dev.region)
        assert ei.value.status == _abi.ERROR_OUT_OF_MEMORY
    finally:
        L.itkg_debug_fail_scratch_alloc(-1)
    got = gpu.GaussianFilter(dev, 1.8, algorithm=gpu.ALGO_TWO_PASS).generate_region(dev.region).download()
    assert bits_equal(got, want)


def test_four_threads_concurrent_generate_region(gpu):
    from itkg import _abi
    L = _abi.lib()
    rng = np.random.default_rng(5)
    vols = [rng.random((40 + 8 * i, 56, 72), dtype=np.float32) for i in range(4)]
    sigmas = [1.0, 1.5, 2.0, 2.5]
    wants = [oracle.gaussian_f32(v, s) for v, s in zip(vols, sigmas)]
    results, errors = {}, []
    barrier = threading.Barrier(4)

    def worker(i):
        try:
            h = ctypes.c_void_p()
            _abi.check(L.itkg_stream_create(ctypes.byref(h)))
            stream = gpu.Stream(h.value)
            dev = gpu.DeviceImage.from_host(gpu.Image(vols[i]), stream)
            outs = []
            barrier.wait()
            for rep in range(6):
                algo = [gpu.ALGO_AUTO, gpu.ALGO_FUSED, gpu.ALGO_PER_AXIS][rep % 3]
                f = gpu.GaussianFilter(dev, sigmas[i], algorithm=algo)
                outs.append(f.generate_region(dev.region, stream=stream).download(stream))
                # host-buffer calls from every thread at once too
                outs.append(gpu.GaussianFilter(gpu.Image(vols[i]), sigmas[i]).generate_region(
                    gpu.Image(vols[i]).region).data)
            stream.synchronize()
            results[i] = outs
            _abi.check(L.itkg_stream_destroy(h))
        except Exception as e:  # reported on the main thread
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for i in range(4):
        for got in results[i]:
            assert bits_equal(got, wants[i]), i
