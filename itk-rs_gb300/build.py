"""Build recipe for libitkg.so (sm_103a).  Run: python itk-rs_gb300/build.py

Compiles every CUDA / C++ translation unit under csrc/ in parallel with nvcc
(one -gencode: compute_103a -> sm_103a) and links one shared library into
itk-rs_gb300/lib/.  Objects go to itk-rs_gb300/_build/.  Rebuilds only what is
older than its sources or headers.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libitkg.so")
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off for the host compiler: host-side coefficients (the
# recursive Gaussian's, the kernels' f64 weights and edge tables) must round
# every product and sum separately as the reference does; gcc on aarch64 would
# otherwise fuse them into FMAs and the coefficients would differ by an ulp
# between an x86 and an Arm host.
COMMON = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", os.path.join(ROOT, "include"), "-I", CSRC]
# -fmad=false: ptxas must not contract a separate multiply and add into an FMA
# (the reference-rounding kernels rely on two roundings per tap); FMA-rounding
# code uses explicit fma instructions, which the flag does not touch.
CUFLAGS = ARCH + ["-lineinfo", "--expt-relaxed-constexpr", "-fmad=false", "-Xptxas", "-warn-spills"]


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(CSRC, "*.cuh"))
            + [os.path.join(ROOT, "include", "itkg.h")])


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + _headers()):
        return obj, None
    cmd = [NVCC] + COMMON + (CUFLAGS if src.endswith(".cu") else ARCH) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"$ {' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    objs, errs = [], []
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        for obj, err in ex.map(_compile, srcs):
            objs.append(obj)
            if err:
                errs.append(err)
    if errs:
        raise RuntimeError("itkg build failed:\n" + "\n".join(errs))
    if _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"itkg link failed:\n$ {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


HOST_TEST_SRC = os.path.join(ROOT, "tests", "cpp", "test_pipeline.cpp")
HOST_TEST_BIN = os.path.join(OBJ, "test_pipeline")


def build_host_tests(verbose: bool = False) -> str:
    """Compile the C++ host-mirror test program against libitkg.so."""
    lib = build()
    deps = [HOST_TEST_SRC, lib, os.path.join(HERE, "host", "itk_gauss.hpp")]
    if _stale(HOST_TEST_BIN, deps):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I",
               os.path.join(HERE, "host"), HOST_TEST_SRC, "-o", HOST_TEST_BIN, "-L", LIBDIR,
               "-litkg", f"-Wl,-rpath,{LIBDIR}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host test build failed:\n$ {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(HOST_TEST_BIN)
    return HOST_TEST_BIN


if __name__ == "__main__":
    build(verbose=True)
    build_host_tests(verbose=True)
    sys.exit(0)
