"""Test configuration.

Markers:
  gpu -- needs a CUDA device; these are the parity tests proper and call the
         library through its C ABI (directly or via the torch binding).
Everything else runs on CPU: the oracle against the golden fixtures, the
host-side logic, and that libgbnufft.so loads and exports its C ABI.
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "jax-finufft_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def pytest_collection_modifyitems(config, items):
    import torch

    if torch.cuda.is_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build, cpu_nufft

    if not os.path.exists(build.library_path()):
        build.build()
    return cpu_nufft.lib()


@pytest.fixture(scope="session")
def native():
    """The CUDA library; on a GPU machine a missing build is an error."""
    from jax_finufft_gb300 import _native

    return _native.load()
