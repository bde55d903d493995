"""Without a usable CUDA device the GPU entry points fail loudly with
CHL_ERR_CUDA: there is no CPU fallback behind the C ABI."""
import ctypes

import numpy as np
import pytest


def _has_device():
    for name in ("libcuda.so.1", "libcuda.so"):
        try:
            cu = ctypes.CDLL(name)
        except OSError:
            continue
        if cu.cuInit(0) != 0:
            return False
        count = ctypes.c_int(0)
        return cu.cuDeviceGetCount(ctypes.byref(count)) == 0 and count.value > 0
    return False


def test_gpu_entry_points_fail_without_a_device(P):
    if _has_device():
        pytest.skip("a CUDA device is present")
    g = P.Graph.grid(12, 12, seed=2)
    order = np.arange(g.get_n(), dtype=np.uint32)
    with pytest.raises(P.CHLError) as e:
        P.build(g, order)
    assert e.value.status == P.CHL_ERR_CUDA
