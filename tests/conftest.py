import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsray_gpu.so")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def small_scene_path():
    from sray_gb300 import scenegen
    return scenegen.write_scene("small")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads the native library; GPU tests only."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without CUDA")
    from sray_gb300 import build, gpu
    build.build()
    return gpu
