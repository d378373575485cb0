import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "sarlab-tdc_gb300"
for p in (str(ROOT), str(PKG), str(Path(__file__).resolve().parent)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine through its C ABI")


@pytest.fixture(scope="session")
def engine_lib():
    """Build (if stale) and load libtdc_gb300.so."""
    import importlib

    spec = importlib.util.spec_from_file_location("tdc_pkg_build", PKG / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import _tdc_capi

    return _tdc_capi.lib()


@pytest.fixture(scope="session")
def cuda_device(engine_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")
