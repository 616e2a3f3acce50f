import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libbem_gb300.so on cuda:0)")


@pytest.fixture(scope="session")
def bemlib():
    """The product library, built in-tree when missing (nvcc only)."""
    from bem_gpu_clean_cpp_gb300 import build
    build.build()
    import bem_gpu_clean_cpp_gb300 as bem
    bem.lib()
    return bem


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle
