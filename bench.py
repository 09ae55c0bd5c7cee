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


def blobs_volume(shape, seed, nblobs=32, noise=0.05):
    """Sum of `nblobs` seeded Gaussian blobs (centres uniform in the volume,
    amplitude U[0.5, 2], std U[4, 24] voxels) plus N(0, noise)."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z = np.arange(nz, dtype=np.float32)[:, None, None]
    y = np.arange(ny, dtype=np.float32)[None, :, None]
    x = np.arange(nx, dtype=np.float32)[None, None, :]
    vol = np.zeros(shape, np.float32)
    for _ in range(nblobs):
        cz, cy, cx = rng.uniform(0, nz), rng.uniform(0, ny), rng.uniform(0, nx)
        amp = rng.uniform(0.5, 2.0)
        sd = rng.uniform(4.0, 24.0)
        k = np.float32(-0.5 / (sd * sd))
        gz = np.exp(k * (z - cz) ** 2)
        gy = np.exp(k * (y - cy) ** 2)
        gx = np.exp(k * (x - cx) ** 2)
        vol += np.float32(amp) * (gz * gy * gx)
    vol += rng.normal(0.0, noise, shape).astype(np.float32)
    return vol


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


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
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
                     "per_axis": itkg.ALGO_PER_AXIS}[args.algo]
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
    ev = [[[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
           for _ in range(NVOL)] for _ in range(args.steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = L.itkg_launch_counter()
    t0.record(stream)
    for k in range(args.steps):
        step(ev[k])
    t1.record(stream)
    torch.cuda.synchronize()
    launches = L.itkg_launch_counter() - launches0
    if dist is not None:
        dist.barrier()
    clk = clocks.stop()
    elapsed_ms = t0.elapsed_time(t1)
    per_launch_ms = [e[0].elapsed_time(e[1]) for row in ev for e in row]
    if dist is not None:
        t = torch.tensor([elapsed_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())

    nvox = SHAPE[0] * SHAPE[1] * SHAPE[2]
    value = world * args.steps * NVOL * nvox / (elapsed_ms * 1e-3)
    avg_launch_s = statistics.mean(per_launch_ms) * 1e-3
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
        if dist is not None:
            t = torch.tensor([te], device="cuda", dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            te = float(t.item())
        res = np.frombuffer((ctypes.c_char * nbytes).from_address(hp_out.value), dtype=np.float32)
        if not np.array_equal(res.reshape(SHAPE).view(np.uint32), got.view(np.uint32)):
            raise RuntimeError("e2e result differs from the device-resident result")
        L.itkg_host_free_pinned(hp_in)
        L.itkg_host_free_pinned(hp_out)
        e2e = {"value": world * args.e2e_steps * nvox / te, "unit": "voxels/s",
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

    if rank == 0:
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
                         "algorithmic_bytes_per_launch": nvox * BYTES_PER_VOXEL,
                         "avg_launch_us": avg_launch_s * 1e6,
                         "frac_of_8TBs": achieved / 8000.0},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
            "accuracy": acc, "clocks": clk,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["itkg", "reference"], default="itkg")
    ap.add_argument("--rounding", choices=["fma", "reference"], default="fma")
    ap.add_argument("--algo", choices=["auto", "fused", "per_axis"], default="auto")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-check", dest="check", action="store_false")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
