import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "mglet-base_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import binding
    binding.build()
    return binding


@pytest.fixture(scope="session")
def gpu_lib():
    import torch  # noqa: F401  (fails the test early on a box without CUDA)
    from mglet_gb300 import build, gpu
    build.build()
    return gpu
