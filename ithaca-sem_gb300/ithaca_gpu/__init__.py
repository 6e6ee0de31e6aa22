"""GB300 (sm_103a) implementation of ITHACA-SEM's spectral/hp Helmholtz + CG + POD path.

The compute lives in lib/libithaca_gpu.so behind the C ABI of include/ithaca_gpu.h;
this package is the Python host side (ctypes bindings, mesh generation, POD driver,
autograd function). There is no CPU fallback.
"""
from . import _capi
from ._capi import GpuError


def load():
    """Loads the shared library (raises if it has not been built)."""
    return _capi.lib()


__all__ = ["load", "GpuError"]
