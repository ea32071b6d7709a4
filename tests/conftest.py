"""Shared test setup: import paths and the `gpu` marker.

`-m "not gpu"` runs the oracle's known-answer tests, the host logic and the
C-ABI symbol checks on CPU; `-m gpu` runs the parity tests through the C ABI
on a GPU.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "custom-gpgpu-rasterizer_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path through the C ABI)")


@pytest.fixture(scope="session")
def gbr_lib():
    import build as gbr_build  # custom-gpgpu-rasterizer_gb300/build.py
    gbr_build.build()
    import gbr
    return gbr


@pytest.fixture(scope="session")
def cuda_device():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is available")
    torch.cuda.init()
    return torch.device("cuda:0")
