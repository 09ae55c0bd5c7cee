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
