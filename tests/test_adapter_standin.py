"""The Nektar++ adapter classes (ithaca-sem_gb300/adapter: the Collections "GPU"
operators and the IterativeFullGPU / IterativeStaticCondGPU global systems) compiled and
linked here against stand-in headers with the reference's signatures
(tests/adapter_standin, Collections/Operator.h:45-175, MultiRegions/GlobalLinSys.h:62-160,
AssemblyMap.h:80-308), and driven through the reference's factories.

CPU: the adapter compiles with -Wall -Wextra, links with every library symbol resolved
(-Wl,--no-undefined against libithaca_gpu.so), registers 30 operator keys (5 operators x
the six shapes) and the two systems, and turns a library error into NekError. GPU: a Helmholtz
apply and HelmSolves through the factory-made objects match the oracle.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from cases import quad_case, rel_err
from oracle import ops as oops
from oracle import solve as osolve

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(ROOT, "ithaca-sem_gb300", "adapter")
STANDIN = os.path.join(ROOT, "tests", "adapter_standin")
LIBDIR = os.path.join(ROOT, "ithaca-sem_gb300", "lib")


@pytest.fixture(scope="module")
def adapter(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    import sys
    sys.path.insert(0, os.path.join(ROOT, "ithaca-sem_gb300"))
    import build as gpu_build
    gpu_build.build()
    out = tmp_path_factory.mktemp("adapter")
    objs = []
    for src in ("CollectionsGPU.cpp", "GlobalLinSysGPU.cpp", os.path.join(STANDIN, "adapter_probe.cpp")):
        path = src if os.path.isabs(src) else os.path.join(ADAPTER, src)
        obj = str(out / (os.path.basename(path) + ".o"))
        r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-fPIC", "-I" + STANDIN,
                            "-I" + os.path.join(ROOT, "include"), "-c", path, "-o", obj], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        objs.append(obj)
    so = str(out / "libadapter_probe.so")
    r = subprocess.run(["g++", "-shared", "-o", so] + objs + ["-Wl,--no-undefined", "-L" + LIBDIR, "-lithaca_gpu",
                                                            "-Wl,-rpath," + LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(so)
    return lib


def test_adapter_registers_operators_and_systems(adapter):
    v = [ctypes.c_int() for _ in range(4)]
    adapter.probe_registry(*[ctypes.byref(x) for x in v])
    nops, nsys, full, sc = (x.value for x in v)
    assert nops == 30 and nsys == 2 and full == 1 and sc == 1


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _helmholtz(adapter, c, lam, u, shape=4):
    out = np.zeros(c.E * c.nm)
    msg = ctypes.create_string_buffer(512)
    rc = adapter.probe_helmholtz(shape, c.n, c.Q, c.E, _dp(np.ascontiguousarray(c.jac)), _dp(np.ascontiguousarray(c.df)),
                                 ctypes.c_double(lam), _dp(u), _dp(out), msg, 512)
    return rc, out, msg.value.decode()


def test_adapter_reports_library_errors_as_nekerror(adapter):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the operator is created")
    c = quad_case(2, 2, 3)
    rc, _, msg = _helmholtz(adapter, c, 1.0, np.ones(c.E * c.nm))
    assert rc == 1 and msg.startswith("ithaca_gpu:")


@pytest.mark.gpu
def test_adapter_helmholtz_matches_oracle(adapter):
    c = quad_case(6, 5, 7)
    u = np.random.default_rng(3).uniform(-1, 1, c.E * c.nm)
    rc, out, msg = _helmholtz(adapter, c, 1.5, u)
    assert rc == 0, msg
    ref = oops.helmholtz(c.basis, 2, c.jac.reshape(c.E, -1), c.df, 1.5, u).reshape(-1)
    assert rel_err(out, ref) < 1e-12


@pytest.mark.gpu
def test_adapter_triangle_helmholtz_matches_oracle(adapter):
    """A triangle collection (eTriangle = 3) through the same adapter class."""
    from cases import tri_case
    from oracle import tri as otri
    c = tri_case(4, 3, 6)
    u = np.random.default_rng(4).uniform(-1, 1, c.E * c.nm)
    rc, out, msg = _helmholtz(adapter, c, 0.8, u, shape=3)
    assert rc == 0, msg
    assert rel_err(out, otri.helmholtz(c.basis, c.jac.reshape(c.E, -1), c.df, 0.8, u)) < 1e-12


@pytest.mark.gpu
def test_adapter_3d_collapsed_helmholtz_match_oracle(adapter):
    """Tetrahedron (5), pyramid (6) and prism (7) collections through the adapter."""
    from cases import prism_case, pyr_case, tet_case
    from oracle import prism as oprism
    from oracle import pyr as opyr
    from oracle import tet as otet
    for c, shape, mod in ((tet_case(1, 1, 1, 5), 5, otet), (pyr_case(1, 1, 1, 5), 6, opyr),
                          (prism_case(1, 1, 1, 5), 7, oprism)):
        u = np.random.default_rng(shape).uniform(-1, 1, c.E * c.nm)
        rc, out, msg = _helmholtz(adapter, c, 0.6, u, shape=shape)
        assert rc == 0, msg
        assert rel_err(out, mod.helmholtz(c.basis, c.jac.reshape(c.E, -1), c.df, 0.6, u)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["IterativeFullGPU", "IterativeStaticCondGPU"])
def test_adapter_global_systems_match_oracle(adapter, name):
    c = quad_case(8, 6, 6)
    amap = c.mesh.assembly(c.n)
    jac = c.jac.reshape(c.E, -1)
    f = (np.sin(np.pi * c.X[0]) * np.sin(np.pi * c.X[1])).reshape(-1)
    loc = -oops.iproduct(c.basis, 2, jac, f).reshape(-1)
    out = np.zeros(c.E * c.nm)
    msg = ctypes.create_string_buffer(512)
    l2g = np.ascontiguousarray(amap.l2g, dtype=np.int32)
    rc = adapter.probe_solve(name.encode(), 4, c.n, c.Q, c.E, _dp(np.ascontiguousarray(c.jac)),
                             _dp(np.ascontiguousarray(c.df)), ctypes.c_double(1.0),
                             l2g.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(amap.sign), amap.nglobal,
                             amap.ndir, ctypes.c_double(1e-12), _dp(loc), _dp(out), msg, 512)
    assert rc == 0, msg.value.decode()
    xo, _ = osolve.helmsolve(c.basis, 2, jac, c.df, 1.0, amap, f, tol=1e-12)
    assert rel_err(out, xo.reshape(-1)) < 1e-9
