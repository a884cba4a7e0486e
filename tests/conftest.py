import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    arrays = np.load(os.path.join(GOLDEN, "reference_kat.npz"))
    with open(os.path.join(GOLDEN, "reference_kat.json")) as f:
        meta = json.load(f)
    return arrays, meta


@pytest.fixture(scope="session")
def lib():
    from block_ipt_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("gpu test collected on a host without CUDA")
    return torch


def _load_cudart():
    import ctypes
    for name in ("libcudart.so", "/usr/local/cuda/lib64/libcudart.so", "libcudart.so.13",
                 "libcudart.so.12"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    raise OSError("libcudart not found")


def device_to_host(ptr, array):
    """cudaMemcpy(array <- device ptr); array is a numpy buffer."""
    import ctypes
    rt = _load_cudart()
    rc = rt.cudaMemcpy(ctypes.c_void_p(array.ctypes.data), ptr, ctypes.c_size_t(array.nbytes), 2)
    assert rc == 0, rc
    return array
