"""Host-side argument handling of the Python binding (no GPU needed).

One C call passes a single on_device flag for all of its pointers, so the binding
allocates default outputs on the side of the input and rejects calls that mix host
arrays and CUDA tensors before anything reaches the library.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "ithaca-sem_gb300"))


class _FakeCuda:
    is_cuda = True


def test_default_output_follows_host_input():
    from ithaca_gpu.operators import _like
    out = _like(np.zeros(3), 5, np.float32)
    assert isinstance(out, np.ndarray) and out.shape == (5,) and out.dtype == np.float32


def test_mixed_host_and_device_arrays_are_rejected():
    from ithaca_gpu.operators import _same_side
    _same_side(np.zeros(2), None, np.zeros(3))
    _same_side(_FakeCuda(), None, _FakeCuda())
    with pytest.raises(ValueError):
        _same_side(np.zeros(2), _FakeCuda())
