import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running parity case")


_GPU = None


def has_gpu() -> bool:
    """True when the CUDA driver reports at least one device (no torch import)."""
    global _GPU
    if _GPU is None:
        try:
            import ctypes
            cu = ctypes.CDLL("libcuda.so.1")
            n = ctypes.c_int(0)
            _GPU = cu.cuInit(0) == 0 and cu.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
        except OSError:
            _GPU = False
    return _GPU


def pytest_collection_modifyitems(config, items):
    if has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)
