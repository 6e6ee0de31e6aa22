"""The C-ABI library builds, loads without a GPU, and exports every declared symbol."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "ithaca-sem_gb300"))
    import build as gpu_build
    gpu_build.build()
    from ithaca_gpu import _capi
    return _capi.lib()


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(ithaca_gpu_\w+)\s*\(", src))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "ithaca_gpu_helmholtz" in names and "ithaca_gpu_cg_solve" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header():
    from ithaca_gpu import _capi
    assert set(declared_symbols()) <= set(_capi.SIGNATURES), set(declared_symbols()) - set(_capi.SIGNATURES)


def test_host_only_calls_work_without_gpu(lib):
    """Basis tables and error reporting need no device."""
    import numpy as np
    from ithaca_gpu.operators import basis_modA
    from oracle import basis as obasis
    z, w, D, B, DB = basis_modA(7, 8)
    b = obasis.Basis1D(7, 8)
    assert np.max(np.abs(z - b.z)) < 1e-15 and np.max(np.abs(B - b.B)) < 1e-14
    assert np.max(np.abs(D - b.D)) / np.max(np.abs(b.D)) < 1e-13
    from ithaca_gpu._capi import GpuError, call
    with pytest.raises(GpuError):
        call("ithaca_gpu_basis_modA", 0, 0, None, None, None, None, None)
