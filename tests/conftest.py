"""Shared test set-up: import paths, the gpu marker, and one-time builds of
the CPU oracle (always) and of libcl2pt.so (GPU tests only)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "cocoa-cosmolike-core_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libcl2pt.so")


@pytest.fixture(scope="session")
def oracle_built():
    import oracle
    oracle.build(ref=False)
    return True


@pytest.fixture(scope="session")
def gpu_lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cl2pt import build, lib
    build.build()
    return lib.load()
