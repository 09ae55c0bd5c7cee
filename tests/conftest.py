import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "itk-rs_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103) and libitkg.so built for it")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "golden.npz")))


@pytest.fixture(scope="session")
def itkg_lib():
    """libitkg.so, built in-tree if missing (nvcc cross-compiles without a GPU)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "itkg_build", os.path.join(ROOT, "itk-rs_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import itkg
    return itkg._abi.lib()


@pytest.fixture(scope="session")
def gpu(itkg_lib):
    import itkg
    if itkg.device_count() < 1:
        pytest.fail("GPU test requested but no CUDA device is visible")
    return itkg
