"""Runs the C++ host-mirror test program (tests/cpp/test_pipeline.cpp), which
re-states the reference's pipeline tests against itk-rs_gb300/host/itk_gauss.hpp."""
import importlib.util
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build_mod():
    spec = importlib.util.spec_from_file_location(
        "itkg_build", os.path.join(ROOT, "itk-rs_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_host_mirror_compiles():
    exe = _build_mod().build_host_tests()
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_host_mirror_pipeline_tests(gpu):
    exe = _build_mod().build_host_tests()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAIL" not in r.stdout


def test_python_filters_region_logic():
    """Host-side geometry of the Python mirror's filters (no device needed)."""
    import numpy as np
    import itkg
    img = itkg.Image(np.zeros((9, 10, 11), np.float32), index=(2, -1, 0))
    u = itkg.UnsharpMaskFilter(img, 1.2)  # radius ceil(3.6) = 4
    out = itkg.Region((4, 0, 1), (3, 2, 2))
    assert u.input_region_for_output(out) == itkg.Region((2, -1, 0), (9, 7, 7))
    assert u.with_amount(0.9).amount == 0.9
    assert itkg.SliceBySliceFilter(img, 2.0).input_region_for_output(out) == out
    b = itkg.BSplineDownsampleFilter(img)
    assert b.largest_region() == itkg.Region((2, -1, 0), (6, 5, 5))
    assert b.spacing == (2.0, 2.0, 2.0)
    assert b.input_region_for_output(out) == img.region
    assert len(itkg.unsharp_kernel(1.2)) == 9
