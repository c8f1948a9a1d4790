import ctypes
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _gpu_present() -> bool:
    try:
        cu = ctypes.CDLL("libcuda.so.1")
    except OSError:
        return False
    if cu.cuInit(0) != 0:
        return False
    n = ctypes.c_int(0)
    return cu.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0


HAVE_GPU = _gpu_present()


def pytest_collection_modifyitems(config, items):
    if HAVE_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA device visible")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)
