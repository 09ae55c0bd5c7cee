#!/usr/bin/env python
"""Benchmark of the GB300 Gaussian path (GaussianFilter::generate_region).

Workload (default): plain 3-D forward, Image<f32,3> 256x256x256, spacing 1,
values = 32 seeded Gaussian blobs + N(0, 0.05) noise, sigma 2.0 (r = 6),
full-region output, FMA rounding (<= 1e-5 normwise of the reference).

A step = the filter over each of 8 such volumes (8 generate_region calls on
8 distinct device buffer pairs, 1 GiB in total, so every step streams from
HBM rather than L2).  `value` = voxels/s over the timed steps with inputs
resident in HBM; `e2e` = the same metric through the C ABI with host
(pinned) buffers, host<->device copies inside the timed region.

--impl reference times the reference algorithm on the host cores instead: the
C restatement of itk-rs's rayon path (serial index build + parallel loop over
output voxels), on a bounded slab of the same workload per step.

--workload selects another line (the default above is fwd3d):
  fwd2d        2-D Image<f32> 512x512, sigma 1.5, 64 images per step
  ct16         CT Image<i16> 512x512x384 -> f32 / bf16 / f16
  batch        64 volumes + 256 RGB images in one graph (batch_vjp: with the VJP)
  vjp_stack    multi-scale loss VJP, 8 x 192^3, sigma {1, 2, 4, 8}
  mean3d       MeanFilter radius 2        binomial3d  BinomialBlurFilter 4 rounds
  recursive3d  RecursiveGaussianFilter (and gradient magnitude), f64 lines
  unsharp3d    UnsharpMaskFilter, both roundings and Image<u8>
  callers3d    SliceBySliceFilter and BSplineDownsampleFilter
  registration2d  DiffeomorphicDemons and N4 bias correction, 512^2
  u8_3d        GaussianFilter<Image<u8>> 256^3 in u8 pixel arithmetic

Prints ONE JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "itk-rs_gb300"))

METRIC = "Gaussian voxels/s & %HBM peak: batched fwd+VJP vs plain fwd, 1 GB300, ≤1e-5 rel"
SHAPE = (256, 256, 256)
SIGMA = 2.0
NVOL = 8
BYTES_PER_VOXEL = 8  # f32 in + f32 out (compulsory traffic)
FALLBACK_HBM_GBS = 6800.0


from itkg.workloads import blobs_volume, ct_volume  # noqa: E402  (seeded synthetic inputs)


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel_key):
    """DRAM bytes per launch from the committed ncu summary, if captured."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get(kernel_key)
    except Exception:
        return None


class Clocks:
    """Samples nvidia-smi while running; summary() gives the clocks record."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.proc = None
        self.device = device

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.05)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        rows = []
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[3:7]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r)
                          if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": rows[0][1],
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# reference arm: the reference algorithm on the host cores
# ---------------------------------------------------------------------------
def cpu_sample_rate(vol, budget_s, threads):
    """Voxels/s of the reference algorithm (C restatement, `threads` workers)
    on a slab of full-xy slices of `vol`, sized to about `budget_s` seconds."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    nz, ny, nx = vol.shape
    z0 = nz // 2

    def run(s):
        req = ((0, 0, z0), (nx, ny, s))
        t = time.perf_counter()
        oracle.gaussian_f32_mt(vol, SIGMA, requested=req, nthreads=threads)
        return time.perf_counter() - t

    t1 = run(2)
    per_slice = max(t1 / 2, 1e-4)
    s = int(max(1, min(nz // 2 - 1, budget_s / per_slice)))
    return s, run


# ---------------------------------------------------------------------------
# Replicas across ranks (one process per GPU, no data exchange)
# ---------------------------------------------------------------------------
def max_over_ranks(value, dist, device):
    """The largest of every rank's `value` (a float), e.g. the timed region's
    duration: the job is as slow as its slowest replica."""
    import torch
    if dist is None:
        return float(value)
    t = torch.tensor([float(value)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world, units_per_rank, elapsed_s):
    """Whole-job throughput of `world` replicas, each processing
    `units_per_rank` units, timed by the slowest one (weak scaling)."""
    return world * units_per_rank / elapsed_s


def reports(rank):
    """Only rank 0 prints the JSON line."""
    return rank == 0


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if not reports(rank):  # under torchrun only rank 0 times the CPU reference
        return 0
    threads = os.cpu_count() or 1
    vol = blobs_volume(SHAPE, 0)
    budget = max(0.02, min(2.0, 150.0 / max(args.steps + args.warmup, 1)))
    s, run = cpu_sample_rate(vol, budget, threads)
    for _ in range(args.warmup):
        run(s)
    times = [run(s) for _ in range(args.steps)]
    vox = SHAPE[1] * SHAPE[2] * s
    value = vox * len(times) / sum(times)
    sample = f"{SHAPE[2]}x{SHAPE[1]}x{s} slab (z from {SHAPE[0] // 2}) of the 256^3 volume per step"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "voxels/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "3-D forward Image<f32,3> 256^3 sigma 2 (blobs+noise)",
                   "sigma": SIGMA, "shape": list(SHAPE)},
        "cpu_baseline": {"value": value, "unit": "voxels/s", "cores": threads, "kind": "port",
                         "sample": sample + "; C restatement of the reference rayon path"},
        "e2e": {"value": value, "unit": "voxels/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def gpu_arm(args):
    import torch
    import itkg
    from itkg import _abi

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    _abi.check(_abi.lib().itkg_set_device(local))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    rounding = itkg.ROUND_REFERENCE if args.rounding == "reference" else itkg.ROUND_FMA
    L = _abi.lib()
    stream = torch.cuda.Stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)

    vol = blobs_volume(SHAPE, 0)
    region = itkg.Region((0, 0, 0), tuple(reversed(SHAPE)))
    ins, outs = [], []
    host_img = itkg.Image(vol)
    for i in range(NVOL):
        d = itkg.DeviceImage(region)
        d.upload(vol)
        ins.append(d)
        outs.append(itkg.DeviceImage(region))
    prm = _abi.itkg_gaussian_params()
    prm.sigma = SIGMA
    prm.rounding = rounding
    prm.algorithm = {"auto": itkg.ALGO_AUTO, "fused": itkg.ALGO_FUSED,
                     "per_axis": itkg.ALGO_PER_AXIS, "two_pass": itkg.ALGO_TWO_PASS,
                     "one_trip": itkg.ALGO_ONE_TRIP}[args.algo]
    lg = region.to_c()
    req = region.to_c()
    in_c = [ctypes.byref(d.c) for d in ins]
    out_c = [ctypes.byref(d.c) for d in outs]
    lg_r, req_r, prm_r = ctypes.byref(lg), ctypes.byref(req), ctypes.byref(prm)
    gen = L.itkg_gaussian_generate_region

    def step(ev=None):
        for i in range(NVOL):
            if ev is not None:
                ev[i][0].record(stream)
            st = gen(in_c[i], lg_r, req_r, prm_r, out_c[i], sptr)
            if st != 0:
                raise _abi.ItkgError(st, L.itkg_last_error().decode())
            if ev is not None:
                ev[i][1].record(stream)

    # accuracy of one output vs the oracle (normwise, and bit-exactness)
    with torch.cuda.stream(stream):
        step()
    stream.synchronize()
    kernel = L.itkg_last_kernel().decode()
    got = outs[0].download()
    acc = {}
    if args.check:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        want = oracle.gaussian_f32_mt(vol, SIGMA)
        err = np.abs(got.astype(np.float64) - want)
        acc = {"normwise_rel_vs_ref_f32": float(err.max() / np.abs(want).max()),
               "max_abs_vs_ref_f32": float(err.max()),
               "bit_exact_vs_ref_f32": bool(np.array_equal(got.view(np.uint32), want.view(np.uint32)))}

    for _ in range(args.warmup):
        step()
    stream.synchronize()

    clocks = Clocks(local)
    clocks.start()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = L.itkg_launch_counter()
    t0.record(stream)
    for k in range(args.steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    launches = L.itkg_launch_counter() - launches0
    if dist is not None:
        dist.barrier()
    clk = clocks.stop()
    elapsed_ms = t0.elapsed_time(t1)
    elapsed_ms = max_over_ranks(elapsed_ms, dist, "cuda")
    # the same calls with an event pair around each (an event between two
    # calls stops the next call's kernels from starting while the previous
    # call's last kernel drains): the call's duration on its own
    ev = [[[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
           for _ in range(NVOL)] for _ in range(max(1, args.steps // 4))]
    for row in ev:
        step(row)
    torch.cuda.synchronize()
    isolated_call_us = statistics.mean(e[0].elapsed_time(e[1]) for row in ev for e in row) * 1e3

    nvox = SHAPE[0] * SHAPE[1] * SHAPE[2]
    value = job_throughput(world, args.steps * NVOL * nvox, elapsed_ms * 1e-3)
    # average call duration over the timed region (calls back to back, as a
    # user's loop issues them)
    avg_launch_s = elapsed_ms * 1e-3 / (args.steps * NVOL)
    peak, peak_kind = measured_peak()
    achieved = nvox * BYTES_PER_VOXEL / avg_launch_s / 1e9

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        nbytes = vol.nbytes
        hp_in = ctypes.c_void_p()
        hp_out = ctypes.c_void_p()
        _abi.check(L.itkg_host_alloc_pinned(nbytes, ctypes.byref(hp_in)))
        _abi.check(L.itkg_host_alloc_pinned(nbytes, ctypes.byref(hp_out)))
        ctypes.memmove(hp_in.value, vol.ctypes.data, nbytes)
        hin = host_img.to_c()
        hin.data = hp_in.value
        hout = host_img.to_c()
        hout.data = hp_out.value
        for _ in range(2):
            _abi.check(gen(ctypes.byref(hin), lg_r, req_r, prm_r, ctypes.byref(hout), sptr))
        if dist is not None:
            dist.barrier()
        ts = time.perf_counter()
        for _ in range(args.e2e_steps):
            _abi.check(gen(ctypes.byref(hin), lg_r, req_r, prm_r, ctypes.byref(hout), sptr))
        te = time.perf_counter() - ts
        te = max_over_ranks(te, dist, "cuda")
        res = np.frombuffer((ctypes.c_char * nbytes).from_address(hp_out.value), dtype=np.float32)
        if not np.array_equal(res.reshape(SHAPE).view(np.uint32), got.view(np.uint32)):
            raise RuntimeError("e2e result differs from the device-resident result")
        L.itkg_host_free_pinned(hp_in)
        L.itkg_host_free_pinned(hp_out)
        e2e = {"value": job_throughput(world, args.e2e_steps * nvox, te), "unit": "voxels/s",
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "steps": args.e2e_steps}

    cpu = None
    if rank == 0 and world == 1 and args.cpu_seconds > 0:
        threads = os.cpu_count() or 1
        s, run = cpu_sample_rate(vol, args.cpu_seconds, threads)
        t = run(s)
        cpu = {"value": SHAPE[1] * SHAPE[2] * s / t, "unit": "voxels/s", "cores": threads,
               "kind": "port",
               "sample": f"{SHAPE[2]}x{SHAPE[1]}x{s} slab of the 256^3 volume, {t:.1f} s; "
                         "C restatement of the reference rayon path"}

    # the metric's second half: batched forward + VJP against the plain per-volume calls
    batch = None
    if rank == 0 and world == 1 and args.batch_steps > 0:
        sp = itkg.Stream(stream.cuda_stream)
        bm = batch_measure(itkg, L, stream, sp, True, args.batch_steps, 3)
        batch = {"value": bm["value"], "unit": "voxels/s (forward + VJP voxel-passes)",
                 "ms_per_step": bm["ms_per_step"], "workload": bm["config"]["workload"],
                 "batch_launches_per_step": bm["config"]["batch_launches_per_step"],
                 "plain_per_volume": bm["plain_per_volume"],
                 "batched_over_plain": bm["batched_over_plain"],
                 "accuracy": bm["accuracy"]}

    if reports(rank):
        line = {
            "metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "3-D forward Image<f32,3> 256^3 sigma 2 (r=6), blobs+noise",
                       "volumes_per_step": NVOL, "sigma": SIGMA, "shape": list(SHAPE),
                       "rounding": args.rounding, "algorithm": args.algo, "kernel": kernel,
                       "l2": "8 rotating 128 MiB in/out buffer pairs per step (1 GiB > L2)",
                       "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": ncu_traffic(kernel),
                         "per": ("call: xy_pass + z_pass kernels" if kernel.startswith("z_pass")
                                 else "call: one kernel"),
                         "algorithmic_bytes_per_launch": nvox * BYTES_PER_VOXEL,
                         "avg_launch_us": avg_launch_s * 1e6,
                         "avg_launch_how": "timed region / calls (CUDA events on the launching stream)",
                         "isolated_call_us": isolated_call_us,
                         "frac_of_8TBs": achieved / 8000.0},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
            "accuracy": acc, "clocks": clk, "batch_fwd_vjp": batch,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# Other configurations (parity/extra lines; not the default bench line)
# ---------------------------------------------------------------------------
def _timed(stream, fn, steps, warmup):
    """Mean ms per call of fn() on `stream`, CUDA events, after warm-up."""
    import torch
    for _ in range(warmup):
        fn()
    stream.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(steps):
        fn()
    t1.record(stream)
    t1.synchronize()
    return t0.elapsed_time(t1) / steps


def _normwise(a, ref):
    ref = np.asarray(ref, np.float64)
    return float(np.abs(np.asarray(a, np.float64) - ref).max() / max(np.abs(ref).max(), 1e-300))


def _gen_call(L, f, req, outimg, sp):
    """One generate_region call of filter f into outimg on stream sp, as a closure."""
    from itkg import _abi
    p = f.params()
    lg = f._leaf().largest_region().to_c()
    rq = req.to_c()
    src = f._leaf().to_c()
    return lambda: _abi.check(L.itkg_gaussian_generate_region(
        ctypes.byref(src), ctypes.byref(lg), ctypes.byref(rq), ctypes.byref(p),
        ctypes.byref(outimg.c), sp.ptr))


def batch_measure(itkg, L, stream, sp, vjp, steps, warmup):
    """The batch workload: 64 Image<f32,3> with dims U{32..320} and sigma
    U[0.5, 4] (plus, forward only, 256 RGB Image<VecPixel<f32,3>,2> with sides
    U{64..1024}), as one planned batch replayed as a CUDA graph, against the
    plain per-volume calls a user makes without the batch API: the library's
    default generate_region (and, with vjp, the default gaussian_vjp) per
    volume, in a loop on the same stream.  Returns the JSON fields."""
    from itkg import _abi
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    rng = np.random.default_rng(0)
    vols = []
    for i in range(64):
        shape = tuple(int(v) for v in rng.integers(32, 321, 3))
        vols.append((rng.random(shape, dtype=np.float32), float(rng.uniform(0.5, 4.0)), 1))
    for i in range(0 if vjp else 256):
        shape = tuple(int(v) for v in rng.integers(64, 1025, 2))
        vols.append((rng.random(shape + (3,), dtype=np.float32), float(rng.uniform(0.5, 4.0)), 3))
    outs, calls = [], []
    b = itkg.Batch()
    vjp_items = []
    sb = ctypes.c_void_p()
    if vjp:
        _abi.check(L.itkg_device_alloc(8 * len(vols), ctypes.byref(sb)))
    nvox = 0
    for i, (arr, sigma, comps) in enumerate(vols):
        d = itkg.DeviceImage.from_host(itkg.Image(arr, components=comps))
        o = itkg.DeviceImage(d.region, itkg.F32, comps)
        outs.append(o)
        nvox += arr.size // comps
        b.add(d, sigma, out=o, rounding=itkg.ROUND_FMA)
        plain = itkg.GaussianFilter(d, sigma, rounding=itkg.ROUND_FMA, algorithm=itkg.ALGO_AUTO)
        calls.append(_gen_call(L, plain, d.region, o, sp))
        if vjp:
            yb = itkg.DeviceImage.from_host(itkg.Image(rng.standard_normal(arr.shape).astype(np.float32)))
            xb = b.add_vjp(d, yb, sigma, sigma_bar_dev=sb.value + 8 * i)
            vjp_items.append((d, yb, sigma, xb, i))
    b.plan(stream=sp)
    ms_batch = _timed(stream, lambda: b.run(sp), steps, warmup)
    launches0 = L.itkg_launch_counter()
    b.run(sp)
    stream.synchronize()
    batch_launches = L.itkg_launch_counter() - launches0

    def plain_all():
        for c in calls:
            c()
        for d, yb, sigma, xb, i in vjp_items:
            p = _abi.itkg_gaussian_params()
            p.sigma = sigma
            p.rounding = itkg.ROUND_FMA
            p.algorithm = itkg.ALGO_AUTO  # the library's default VJP kernels per volume
            _abi.check(L.itkg_gaussian_vjp(ctypes.byref(d.c), ctypes.byref(yb.c), ctypes.byref(p),
                                           ctypes.byref(xb.c),
                                           ctypes.cast(ctypes.c_void_p(sb.value + 8 * i), ctypes.POINTER(ctypes.c_double)),
                                           4, sp.ptr))
    ms_plain = _timed(stream, plain_all, max(1, steps // 2), max(1, warmup // 2))
    launches0 = L.itkg_launch_counter()
    plain_all()
    stream.synchronize()
    plain_launches = L.itkg_launch_counter() - launches0
    units = nvox * (2 if vjp else 1)
    got = outs[0].download()
    err = _normwise(got, oracle.gaussian_f32(vols[0][0], vols[0][1], comps=vols[0][2]))
    if sb.value:
        L.itkg_device_free(sb)
    return {"value": units / (ms_batch * 1e-3), "ms_per_step": ms_batch, "dtype": "f32",
            "config": {"workload": ("64 Image<f32,3> U{32..320}^3 + 256 RGB 2-D U{64..1024}^2, sigma U[0.5,4], one graph"
                                    if not vjp else
                                    "64 Image<f32,3> U{32..320}^3, sigma U[0.5,4]: forward + VJP (x and sigma), one graph"),
                       "voxels": nvox, "plan": b.describe().strip().splitlines()[:12],
                       "batch_launches_per_step": int(batch_launches)},
            "plain_per_volume": {"value": units / (ms_plain * 1e-3), "ms_per_step": ms_plain,
                                 "launches_per_step": int(plain_launches),
                                 "kernel": "default generate_region per volume" +
                                           (" + default gaussian_vjp per volume" if vjp else "")},
            "batched_over_plain": ms_plain / ms_batch,
            "accuracy": {"normwise_rel_vs_ref_f32_item0": err}}


def extra_workload(args):
    """One JSON line for a workload other than the default (see --workload)."""
    import torch
    import itkg
    from itkg import _abi
    torch.cuda.set_device(0)
    L = _abi.lib()
    stream = torch.cuda.Stream()
    sp = itkg.Stream(stream.cuda_stream)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    peak, _ = measured_peak()
    rng = np.random.default_rng(0)
    out = {"metric": METRIC, "unit": "voxels/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "higher_is_better": True, "data": "synthetic",
           "vs_baseline": None}

    def gen(f, req, outimg):
        p = f.params()
        lg = f._leaf().largest_region().to_c()
        rq = req.to_c()
        src = f._leaf().to_c()
        return lambda: _abi.check(L.itkg_gaussian_generate_region(
            ctypes.byref(src), ctypes.byref(lg), ctypes.byref(rq), ctypes.byref(p),
            ctypes.byref(outimg.c), sp.ptr))

    if args.workload == "fwd2d":
        # 2-D workload: Image<f32,2> 512x512, U[0,1), sigma 1.5 (r = 5)
        n = 64
        imgs = [rng.random((512, 512), dtype=np.float32) for _ in range(4)]
        devs = [itkg.DeviceImage.from_host(itkg.Image(imgs[i % 4])) for i in range(n)]
        outs = [itkg.DeviceImage(devs[0].region) for _ in range(n)]
        calls = [gen(itkg.GaussianFilter(d, 1.5, rounding=itkg.ROUND_FMA), d.region, o)
                 for d, o in zip(devs, outs)]
        ms = _timed(stream, lambda: [c() for c in calls], args.steps, args.warmup)
        kernel = itkg.last_kernel()
        got = outs[0].download()
        err = _normwise(got, oracle.gaussian_f32(imgs[0], 1.5))
        vox = n * 512 * 512
        # host time of one call (argument checks, plan, launch), the GPU not waited for
        stream.synchronize()
        t0 = time.perf_counter()
        for c in calls:
            c()
        host_us = (time.perf_counter() - t0) / n * 1e6
        stream.synchronize()
        # the same 64 images as one planned batch (a CUDA graph replayed per step)
        b = itkg.Batch()
        for d, o in zip(devs, outs):
            b.add(d, 1.5, out=o, rounding=itkg.ROUND_FMA)
        b.plan(stream=sp)
        ms_b = _timed(stream, lambda: b.run(sp), args.steps, args.warmup)
        out.update({"value": vox / (ms * 1e-3), "ms_per_step": ms, "dtype": "f32",
                    "config": {"workload": "2-D forward Image<f32,2> 512x512 sigma 1.5, 64 images per step",
                               "kernel": kernel, "host_us_per_call": host_us},
                    "roofline": {"bound": "hbm", "achieved": vox * 8 / (ms * 1e-3) / 1e9, "peak": peak,
                                 "unit": "GB/s", "frac": vox * 8 / (ms * 1e-3) / 1e9 / peak},
                    "batched": {"value": vox / (ms_b * 1e-3), "ms_per_step": ms_b,
                                "achieved_GBs": vox * 8 / (ms_b * 1e-3) / 1e9,
                                "how": "itkg.Batch of the 64 calls, one graph replay per step"},
                    "accuracy": {"normwise_rel_vs_ref_f32": err}})
    elif args.workload == "ct16":
        # CT workload: Image<i16,3> 512x512x384 CT-like, spacing (0.7,0.7,2.5), sigma 1.5 mm
        ct = ct_volume((384, 512, 512), seed=0)
        spacing = (0.7, 0.7, 2.5)
        dev = itkg.DeviceImage.from_host(itkg.Image(ct, spacing=spacing))
        lines = {}
        sub = ct[180:204, 200:264, 200:264].astype(np.float64)  # FP64 check on a block
        ref64 = oracle.gaussian_f64(sub, 1.5, spacing=list(spacing))
        for name, code, bpv in [("f32", itkg.F32, 6), ("bf16", itkg.BF16, 4), ("f16", itkg.F16, 4)]:
            o = itkg.DeviceImage(dev.region, code, 1, spacing)
            f = itkg.GaussianFilter(itkg.CastFilter(dev, itkg.F32), 1.5, rounding=itkg.ROUND_FMA)
            call = gen(f, dev.region, o)
            ms = _timed(stream, call, args.steps, args.warmup)
            kern = itkg.last_kernel()
            # accuracy: same block through the filter vs FP64 oracle
            sdev = itkg.DeviceImage.from_host(itkg.Image(np.ascontiguousarray(ct[180:204, 200:264, 200:264]), spacing=spacing))
            so = itkg.GaussianFilter(itkg.CastFilter(sdev, itkg.F32), 1.5, rounding=itkg.ROUND_FMA) \
                .generate_region(sdev.region, out_dtype=code).download()
            got = (so.astype(np.uint32) << 16).view(np.float32) if code == itkg.BF16 else so.astype(np.float32)
            nvox = ct.size
            lines[name] = {"voxels_per_s": nvox / (ms * 1e-3), "ms": ms, "kernel": kern,
                           "GBs": nvox * bpv / (ms * 1e-3) / 1e9,
                           "normwise_rel_vs_fp64": _normwise(got, ref64),
                           "max_abs_vs_fp64": float(np.abs(got - ref64).max())}
        out.update({"value": lines["f32"]["voxels_per_s"], "ms_per_step": lines["f32"]["ms"],
                    "dtype": "i16->f32", "config": {"workload": "CT i16 512x512x384, spacing (0.7,0.7,2.5), sigma 1.5 mm, r=(7,7,2)",
                                                   "outputs": lines}})
    elif args.workload in ("batch", "batch_vjp"):
        out.update(batch_measure(itkg, L, stream, sp, args.workload == "batch_vjp", args.steps, args.warmup))
    elif args.workload == "vjp_stack":
        # multi-scale VJP workload: 8 x 192^3 blobs+noise, sigma {1,2,4,8}; loss sum_l |G_l x - t|^2
        n = 8
        shape = (192, 192, 192)
        xs = [blobs_volume(shape, 100 + i) for i in range(n)]
        ts = [blobs_volume(shape, 200 + i) for i in range(n)]
        dx = [itkg.DeviceImage.from_host(itkg.Image(a)) for a in xs]
        dt = [itkg.DeviceImage.from_host(itkg.Image(a)) for a in ts]
        sigmas = [1.0, 2.0, 4.0, 8.0]
        xbar = [itkg.DeviceImage(dx[0].region) for _ in range(n)]
        sig_arr = (ctypes.c_double * len(sigmas))(*sigmas)
        sb = ctypes.c_void_p()
        _abi.check(L.itkg_device_alloc(8 * len(sigmas) * n, ctypes.byref(sb)))

        def step():
            # L_i = sum_l |G_l x_i - t_i|^2: loss gradient w.r.t. x_i and each sigma_l, the
            # scale stack recomputed level by level (dL/dsigma kept on the device)
            for i in range(n):
                _abi.check(L.itkg_gaussian_scale_stack_loss_vjp(
                    ctypes.byref(dx[i].c), ctypes.byref(dt[i].c), sig_arr, len(sigmas),
                    ctypes.byref(xbar[i].c), None,
                    ctypes.cast(ctypes.c_void_p(sb.value + 8 * len(sigmas) * i), ctypes.POINTER(ctypes.c_double)),
                    4, sp.ptr))
        ms = _timed(stream, step, max(1, args.steps // 4), 1)
        kernel = L.itkg_last_kernel().decode()
        L.itkg_device_free(sb)
        vl = n * len(sigmas) * int(np.prod(shape))
        out.update({"value": vl / (ms * 1e-3), "unit": "voxel-levels/s", "ms_per_step": ms,
                    "dtype": "f32",
                    "config": {"workload": "8 x 192^3 blobs+noise, targets a second seeded set, sigma {1,2,4,8}: "
                                           "loss sum_l |G_l x - t|^2, dL/dx and dL/dsigma_l, stack recomputed",
                               "kernel": kernel,
                               "note": "levels with radius <= 12 use the two-pass forward and VJP kernels; "
                                       "sigma 8 (radius 24) the per-axis passes"}})
    elif args.workload in ("mean3d", "binomial3d"):
        # the convolve_axis family on the 256^3 blobs volume of the default workload
        vol = blobs_volume(SHAPE, 0)
        if args.workload == "mean3d":
            radius = 2
            make = lambda src: itkg.MeanFilter(src, radius, rounding=itkg.ROUND_FMA)
            kernels, reps = [oracle.box_kernel(radius)] * 3, 1
            desc = "MeanFilter radius 2 (5-tap box per axis), Image<f32,3> 256^3 blobs+noise, 8 volumes per step"
            passes = 1
        else:
            reps = 4
            make = lambda src: itkg.BinomialBlurFilter(src, reps, rounding=itkg.ROUND_FMA)
            kernels = [oracle.BINOMIAL_KERNEL] * 3
            desc = "BinomialBlurFilter 4 rounds ([1,2,1]/4, 12 passes), Image<f32,3> 256^3 blobs+noise, 8 volumes per step"
            passes = 3 * reps
        devs = [itkg.DeviceImage.from_host(itkg.Image(vol)) for _ in range(NVOL)]
        outs = [itkg.DeviceImage(devs[0].region) for _ in range(NVOL)]
        filters = [make(d) for d in devs]
        prms = [f.separable_params() for f in filters]
        lg = devs[0].region.to_c()
        rq = devs[0].region.to_c()

        def step():
            for f, p, d, o in zip(filters, prms, devs, outs):
                _abi.check(L.itkg_separable_generate_region(ctypes.byref(d.c), ctypes.byref(lg), ctypes.byref(rq),
                                                            ctypes.byref(p), ctypes.byref(o.c), sp.ptr))
        launches0 = L.itkg_launch_counter()
        step()
        torch.cuda.synchronize()
        per_call_launches = (L.itkg_launch_counter() - launches0) // NVOL
        kern = itkg.last_kernel()
        ms = _timed(stream, step, args.steps, args.warmup)
        nvox = int(np.prod(SHAPE))
        err = _normwise(outs[0].download(), oracle.separable_f32_mt(vol, kernels, reps))
        call_s = ms * 1e-3 / NVOL
        achieved = nvox * BYTES_PER_VOXEL / call_s / 1e9
        cpu = None
        if args.cpu_seconds > 0:
            threads = os.cpu_count() or 1
            nz, ny, nx = vol.shape

            def run(sl):
                t = time.perf_counter()
                oracle.separable_f32_mt(vol, kernels, reps, requested=((0, 0, nz // 2), (nx, ny, sl)),
                                        nthreads=threads)
                return time.perf_counter() - t
            per = max(run(2) / 2, 1e-4)
            sl = int(max(1, min(nz // 2 - 1, args.cpu_seconds / per)))
            cpu = {"value": nx * ny * sl / run(sl), "unit": "voxels/s", "cores": threads, "kind": "port",
                   "sample": f"{sl} output slices of 256x256 (same filter, C restatement, {threads} threads)"}
        out.update({"value": NVOL * nvox / (ms * 1e-3), "ms_per_step": ms, "dtype": "f32",
                    "config": {"workload": desc, "kernel": kern, "launches_per_call": int(per_call_launches),
                               "l2": "8 distinct 64 MiB input/output pairs per step (1 GiB > L2)"},
                    "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                 "frac": achieved / peak, "per_pass_GBs": achieved * passes,
                                 "note": "8 B per voxel per call; per-axis passes each move ~8 B per voxel"},
                    "cpu_baseline": cpu,
                    "accuracy": {"normwise_rel_vs_ref_f32": err}})
    elif args.workload == "recursive3d":
        # RecursiveGaussianFilter sigma 2 on the 256^3 blobs volume: f64 bit-exact and f64 with FMA
        vol = blobs_volume(SHAPE, 0)
        nvox = int(np.prod(SHAPE))
        n = 4
        devs = [itkg.DeviceImage.from_host(itkg.Image(vol)) for _ in range(n)]
        outs = [itkg.DeviceImage(devs[0].region) for _ in range(n)]
        lg = devs[0].region.to_c()
        rq = devs[0].region.to_c()
        lines = {}
        want = oracle.recursive_gaussian_f32(vol, SIGMA)
        for name, rnd in (("f64_reference", itkg.ROUND_REFERENCE), ("f64_fma", itkg.ROUND_FMA)):
            p = _abi.itkg_recursive_params()
            p.sigma, p.axis, p.rounding = SIGMA, -1, rnd

            def step(p=p):
                for d, o in zip(devs, outs):
                    _abi.check(L.itkg_recursive_gaussian_generate_region(
                        ctypes.byref(d.c), ctypes.byref(lg), ctypes.byref(rq), ctypes.byref(p),
                        ctypes.byref(o.c), sp.ptr))
            ms = _timed(stream, step, max(2, args.steps // 8), args.warmup)
            got = outs[0].download()
            lines[name] = {"voxels_per_s": n * nvox / (ms * 1e-3), "ms_per_call": ms / n,
                           "kernel": itkg.last_kernel(), "normwise_rel_vs_ref": _normwise(got, want),
                           "bit_exact": bool(np.array_equal(got.view(np.uint32), want.view(np.uint32)))}
        # a derivative user: GradientMagnitudeRecursiveGaussianFilter (smoothing + gradient stencil)
        p = _abi.itkg_recursive_derivative_params()
        p.sigma, p.kind, p.rounding = SIGMA, 0, itkg.ROUND_REFERENCE

        def step_gm(p=p):
            for d, o in zip(devs, outs):
                _abi.check(L.itkg_recursive_gaussian_derivative_generate_region(
                    ctypes.byref(d.c), ctypes.byref(lg), ctypes.byref(rq), ctypes.byref(p),
                    ctypes.byref(o.c), sp.ptr))
        ms = _timed(stream, step_gm, max(2, args.steps // 8), args.warmup)
        gm = outs[0].download()
        want_gm = oracle.recursive_derivative(vol, SIGMA, oracle.REC_GRADIENT_MAGNITUDE)
        lines["gradient_magnitude_f64_reference"] = {
            "voxels_per_s": n * nvox / (ms * 1e-3), "ms_per_call": ms / n, "kernel": itkg.last_kernel(),
            "bit_exact": bool(np.array_equal(gm.view(np.uint32), want_gm.view(np.uint32)))}
        cpu = None
        if args.cpu_seconds > 0:
            sub = vol[:, :64, :64]  # the recursion is sequential per line: time a 256 x 64 x 64 block
            t = time.perf_counter()
            oracle.recursive_gaussian_f32(sub, SIGMA)
            dt = time.perf_counter() - t
            cpu = {"value": sub.size / dt, "unit": "voxels/s", "cores": 1, "kind": "port",
                   "sample": "256x64x64 block, C restatement (the reference runs its lines sequentially)"}
        out.update({"value": lines["f64_reference"]["voxels_per_s"], "ms_per_step": lines["f64_reference"]["ms_per_call"] * n,
                    "dtype": "f64", "config": {"workload": "RecursiveGaussianFilter sigma 2, Image<f32,3> 256^3 blobs+noise, 4 volumes per step",
                                               "variants": lines},
                    "cpu_baseline": cpu})
    elif args.workload == "unsharp3d":
        # UnsharpMaskFilter sigma 1.5 (radius 5 on every axis), amount 0.5, threshold 0
        vol = blobs_volume(SHAPE, 0)
        nvox = int(np.prod(SHAPE))
        usig, amount = 1.5, 0.5
        devs = [itkg.DeviceImage.from_host(itkg.Image(vol)) for _ in range(NVOL)]
        outs = [itkg.DeviceImage(devs[0].region) for _ in range(NVOL)]
        lg = devs[0].region.to_c()
        rq = devs[0].region.to_c()
        want = oracle.unsharp_mask(vol, usig, amount, 0.0)
        lines = {}
        for name, rnd in (("reference", itkg.ROUND_REFERENCE), ("fma", itkg.ROUND_FMA)):
            p = _abi.itkg_unsharp_params()
            p.sigma, p.amount, p.threshold, p.rounding = usig, amount, 0.0, rnd

            def step(p=p):
                for d, o in zip(devs, outs):
                    _abi.check(L.itkg_unsharp_mask_generate_region(ctypes.byref(d.c), ctypes.byref(lg),
                                                                   ctypes.byref(rq), ctypes.byref(p),
                                                                   ctypes.byref(o.c), sp.ptr))
            launches0 = L.itkg_launch_counter()
            step()
            torch.cuda.synchronize()
            per_call = (L.itkg_launch_counter() - launches0) // NVOL
            ms = _timed(stream, step, args.steps, args.warmup)
            got = outs[0].download()
            call_s = ms * 1e-3 / NVOL
            lines[name] = {"voxels_per_s": NVOL * nvox / (ms * 1e-3), "ms_per_call": ms / NVOL,
                           "kernel": itkg.last_kernel(), "launches_per_call": int(per_call),
                           "achieved_GBs": nvox * BYTES_PER_VOXEL / call_s / 1e9,
                           "normwise_rel_vs_ref": _normwise(got, want),
                           "bit_exact": bool(np.array_equal(got.view(np.uint32), want.view(np.uint32)))}
        cpu = None
        if args.cpu_seconds > 0:
            # the blur dominates the CPU cost: time the family restatement on a slab of output slices
            threads = os.cpu_count() or 1
            nz, ny, nx = vol.shape
            k = [oracle.unsharp_kernel(usig)] * 3

            def run(sl):
                t = time.perf_counter()
                oracle.separable_f32_mt(vol, k, 1, requested=((0, 0, nz // 2), (nx, ny, sl)), nthreads=threads)
                return time.perf_counter() - t
            per = max(run(2) / 2, 1e-4)
            sl = int(max(1, min(nz // 2 - 1, args.cpu_seconds / per)))
            cpu = {"value": nx * ny * sl / run(sl), "unit": "voxels/s", "cores": threads, "kind": "port",
                   "sample": f"the blur of {sl} output slices of 256x256 (C restatement, {threads} threads; "
                             "the point-wise step is not timed)"}
        # Image<u8, 3>: the blobs volume scaled to 0..255 (u8 pixel arithmetic, bit-exact)
        vol8 = np.clip(np.rint(vol * 100.0), 0, 255).astype(np.uint8)
        d8 = [itkg.DeviceImage.from_host(itkg.Image(vol8)) for _ in range(NVOL)]
        o8 = [itkg.DeviceImage(d8[0].region, itkg.U8) for _ in range(NVOL)]
        p8 = _abi.itkg_unsharp_params()
        p8.sigma, p8.amount, p8.threshold, p8.rounding = usig, amount, 0.0, itkg.ROUND_REFERENCE

        def step8():
            for d, o in zip(d8, o8):
                _abi.check(L.itkg_unsharp_mask_generate_region(ctypes.byref(d.c), ctypes.byref(lg), ctypes.byref(rq),
                                                               ctypes.byref(p8), ctypes.byref(o.c), sp.ptr))
        ms8 = _timed(stream, step8, args.steps, args.warmup)
        got8 = o8[0].download()
        lines["u8_reference"] = {"voxels_per_s": NVOL * nvox / (ms8 * 1e-3), "ms_per_call": ms8 / NVOL,
                                 "kernel": itkg.last_kernel(),
                                 "bit_exact": bool(np.array_equal(got8, oracle.unsharp_mask(vol8, usig, amount, 0.0)))}
        best = lines["fma"]
        out.update({"value": best["voxels_per_s"], "ms_per_step": best["ms_per_call"] * NVOL, "dtype": "f32",
                    "config": {"workload": "UnsharpMaskFilter sigma 1.5 amount 0.5, Image<f32,3> 256^3 blobs+noise, "
                                           "8 volumes per step",
                               "variants": lines,
                               "l2": "8 distinct 64 MiB input/output pairs per step (1 GiB > L2)"},
                    "roofline": {"bound": "hbm", "achieved": best["achieved_GBs"], "peak": peak, "unit": "GB/s",
                                 "frac": best["achieved_GBs"] / peak,
                                 "note": "algorithmic 8 B per voxel per call (read the input, write the output)"},
                    "cpu_baseline": cpu})
    elif args.workload == "u8_3d":
        # GaussianFilter<Image<u8>> (u8 pixel arithmetic), 256^3 u8 from the
        # blobs volume scaled to 0..255, sigma 2: two-pass kernels and per-axis passes
        vol = np.clip(blobs_volume(SHAPE, 0) * 120.0, 0, 255).astype(np.uint8)
        nvox = int(np.prod(SHAPE))
        devs = [itkg.DeviceImage.from_host(itkg.Image(vol)) for _ in range(NVOL)]
        region = devs[0].region
        want = oracle.gaussian_u8(vol, SIGMA)
        lines = {}
        for name, algo in (("two_pass", itkg.ALGO_AUTO), ("per_axis", itkg.ALGO_PER_AXIS)):
            outs = [itkg.DeviceImage(region, itkg.U8, 1) for _ in range(NVOL)]
            calls = [_gen_call(L, itkg.GaussianFilter(d, SIGMA, arithmetic=itkg.ARITH_PIXEL_U8, algorithm=algo),
                               region, o, sp) for d, o in zip(devs, outs)]
            ms = _timed(stream, lambda: [c() for c in calls], args.steps, args.warmup)
            got = outs[0].download()
            lines[name] = {"voxels_per_s": NVOL * nvox / (ms * 1e-3), "us_per_call": ms / NVOL * 1e3,
                           "kernel": itkg.last_kernel(), "bit_exact": bool(np.array_equal(got, want))}
        best = lines["two_pass"]
        out.update({"value": best["voxels_per_s"], "ms_per_step": best["us_per_call"] * NVOL * 1e-3, "dtype": "u8",
                    "config": {"workload": "GaussianFilter<Image<u8,3>> 256^3 sigma 2, u8 pixel arithmetic "
                                           "(wrapping u8 adds of round(x*w)), 8 volumes per step",
                               "variants": lines},
                    "roofline": {"bound": "fp32 issue (three instructions per tap and voxel)",
                                 "achieved": nvox * 2 / (best["us_per_call"] * 1e-6) / 1e9, "peak": peak,
                                 "unit": "GB/s", "frac": nvox * 2 / (best["us_per_call"] * 1e-6) / 1e9 / peak,
                                 "note": "algorithmic 2 B per voxel (u8 in, u8 out)"}})
    elif args.workload == "callers3d":
        # the in-crate callers of GaussianFilter on the 256^3 blobs volume
        vol = blobs_volume(SHAPE, 0)
        nvox = int(np.prod(SHAPE))
        devs = [itkg.DeviceImage.from_host(itkg.Image(vol)) for _ in range(NVOL)]
        region = devs[0].region
        lines = {}
        for name, rnd in (("reference", itkg.ROUND_REFERENCE), ("fma", itkg.ROUND_FMA)):
            sl = [itkg.SliceBySliceFilter(d, SIGMA, rounding=rnd) for d in devs]
            outs = [itkg.DeviceImage(region) for _ in range(NVOL)]
            prm = sl[0].params()
            rq = region.to_c()

            def step_sl():
                for d, o in zip(devs, outs):
                    _abi.check(L.itkg_slice_by_slice_generate_region(ctypes.byref(d.c), ctypes.byref(rq),
                                                                     ctypes.byref(prm), ctypes.byref(o.c), sp.ptr))
            ms = _timed(stream, step_sl, args.steps, args.warmup)
            got = outs[0].download()
            want = oracle.slice_by_slice(vol, SIGMA)
            lines[f"slice_by_slice_sigma2_{name}"] = {
                "voxels_per_s": NVOL * nvox / (ms * 1e-3), "ms_per_call": ms / NVOL, "kernel": itkg.last_kernel(),
                "normwise_rel_vs_ref": _normwise(got, want),
                "bit_exact": bool(np.array_equal(got.view(np.uint32), want.view(np.uint32)))}
            bs = [itkg.BSplineDownsampleFilter(d, rounding=rnd) for d in devs]
            half = bs[0].largest_region()
            bouts = [itkg.DeviceImage(half) for _ in range(NVOL)]
            bprm = bs[0].params()
            lg = region.to_c()

            def step_bs():
                for d, o in zip(devs, bouts):
                    _abi.check(L.itkg_bspline_downsample_generate_region(ctypes.byref(d.c), ctypes.byref(lg),
                                                                         ctypes.byref(bprm), ctypes.byref(o.c),
                                                                         sp.ptr))
            ms = _timed(stream, step_bs, args.steps, args.warmup)
            got = bouts[0].download()
            want = oracle.bspline_downsample(vol)
            lines[f"bspline_downsample_{name}"] = {
                "input_voxels_per_s": NVOL * nvox / (ms * 1e-3), "ms_per_call": ms / NVOL,
                "kernel": itkg.last_kernel(), "normwise_rel_vs_ref": _normwise(got, want),
                "bit_exact": bool(np.array_equal(got.view(np.uint32), want.view(np.uint32)))}
        best = lines["slice_by_slice_sigma2_fma"]
        achieved = nvox * BYTES_PER_VOXEL / (best["ms_per_call"] * 1e-3) / 1e9
        out.update({"value": best["voxels_per_s"], "ms_per_step": best["ms_per_call"] * NVOL, "dtype": "f32",
                    "config": {"workload": "SliceBySliceFilter sigma 2 and BSplineDownsampleFilter, Image<f32,3> "
                                           "256^3 blobs+noise, 8 volumes per step",
                               "variants": lines,
                               "l2": "8 distinct 64 MiB input/output pairs per step (1 GiB > L2)"},
                    "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                 "frac": achieved / peak,
                                 "note": "SliceBySlice, algorithmic 8 B per voxel per call (the fused 2-D kernel over every slice)"}})
    elif args.workload == "registration2d":
        # the Gaussian callers that iterate: diffeomorphic demons (30 iterations,
        # max step 0.5, sigma_diff 1) and N4 bias correction (4 iterations, sigma 30)
        from itkg.workloads import biased_image, registration_pair
        fixed, moving = registration_pair((512, 512), 0)
        img = biased_image((512, 512), 0)
        fd = itkg.DeviceImage.from_host(itkg.Image(fixed))
        md = itkg.DeviceImage.from_host(itkg.Image(moving))
        idv = itkg.DeviceImage.from_host(itkg.Image(img))
        lines = {}
        dem = itkg.DiffeomorphicDemonsRegistrationFilter(fd, md, 30, sigma_diff=1.0)
        dem.max_step_length = 0.5
        n4f = itkg.N4BiasFieldCorrectionFilter(idv, 4, 30.0, 1e-3)
        for name, fn, ref in (
                ("diffeomorphic_demons_512sq_30it", lambda: dem.compute(sp),
                 lambda: oracle.diffeomorphic_demons(fixed, moving, 30, sigma_diff=1.0, max_step_length=0.5)),
                ("n4_512sq_4it_sigma30", lambda: n4f.generate_region(None, sp),
                 lambda: oracle.n4(img, 4, 30.0, 1e-3)[0])):
            for _ in range(max(1, args.warmup)):
                res = fn()
            stream.synchronize()
            n = max(1, args.steps // 20)
            t0 = time.perf_counter()
            for _ in range(n):
                res = fn()
            stream.synchronize()
            dt = (time.perf_counter() - t0) / n
            got = res.download()
            tc = time.perf_counter()
            want = ref()
            cpu = time.perf_counter() - tc
            lines[name] = {"ms_per_call": dt * 1e3, "pixels_per_s": 512 * 512 / dt, "kernel": itkg.last_kernel(),
                           "normwise_rel_vs_oracle": _normwise(got, want),
                           "bit_exact": bool(np.array_equal(got.view(np.uint32), want.view(np.uint32))),
                           "cpu_port_ms_1_core": cpu * 1e3}
        d = lines["diffeomorphic_demons_512sq_30it"]
        out.update({"value": d["pixels_per_s"], "unit": "pixels/s", "ms_per_step": d["ms_per_call"], "dtype": "f64+f32",
                    "config": {"workload": "DiffeomorphicDemonsRegistrationFilter 512^2 (30 iterations) and "
                                           "N4BiasFieldCorrectionFilter 512^2 (4 iterations, sigma 30), synthetic",
                               "variants": lines,
                               "timing": "host clock around synchronous calls (each call reads a result back)"}})
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["itkg", "reference"], default="itkg")
    ap.add_argument("--workload", choices=["fwd3d", "fwd2d", "ct16", "batch", "batch_vjp", "vjp_stack",
                                           "mean3d", "binomial3d", "recursive3d", "unsharp3d", "callers3d",
                                           "registration2d", "u8_3d"],
                    default="fwd3d")
    ap.add_argument("--rounding", choices=["fma", "reference"], default="fma")
    ap.add_argument("--algo", choices=["auto", "fused", "per_axis", "two_pass", "one_trip"], default="auto")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--batch-steps", type=int, default=10,
                    help="steps of the batched forward + VJP measurement added to the default line (0: skip)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-check", dest="check", action="store_false")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload != "fwd3d":
        return extra_workload(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
