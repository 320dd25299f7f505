"""Shared test configuration.  `gpu` tests need a CUDA device and the built native libraries."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _ensure_built():
    """Build the engine and the oracle if this checkout has not built them for this machine."""
    import __graft_entry__
    lib = os.path.join(ROOT, "cuda_voxelizer_gb300", "_lib", "libcvx.so")
    oracle_build = __graft_entry__._load("oracle/build.py", "_oracle_build_check")
    if not os.path.exists(lib) or oracle_build.foreign_binary(lib):
        __graft_entry__.build()


_ensure_built()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)
