"""The compiled CPU port (oracle/cport, the timed CPU baseline and the reference arm of
the benchmark) against golden vectors from the reference's own compiled kernels.

Fixtures: tests/golden/*.npz (tests/golden/make_golden.py, from oracle/_ref). Operators to
1e-13 relative (FP64 on both sides, different summation order); the CG recurrence to the
same iteration count and the solution to 1e-12.
"""
import os

import numpy as np
import pytest

from cases import rel_err

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-13


@pytest.fixture(scope="module")
def cport():
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.run(["make", "-s", "-C", os.path.join(root, "oracle", "cport")], check=True)
    from oracle import cportbind
    return cportbind


def load(name):
    return np.load(os.path.join(G, name))


@pytest.mark.parametrize("fname,dim,n", [("mesh_quad.npz", 2, 7), ("mesh_hex.npz", 3, 5)])
@pytest.mark.parametrize("nthreads", [1, 3])
def test_cport_operators_match_reference(cport, fname, dim, n, nthreads):
    g = load(fname)
    Q = n + 1
    E = g["u"].size // n ** dim
    jac, df, u, f = g["jac"], g["df"], g["u"], g["f"]
    assert rel_err(cport.bwdtrans(dim, n, Q, E, u, nthreads), g["bwd"]) < TOL
    assert rel_err(cport.iproduct(dim, n, Q, E, jac, True, f, nthreads), g["iprod"]) < TOL
    d = cport.physderiv(dim, n, Q, E, df, True, f, nthreads)
    for k in range(dim):
        assert rel_err(d[k], g["deriv"][k]) < TOL
    out = cport.helmholtz(dim, n, Q, E, jac, df, True, 1.0, u, nthreads)
    assert rel_err(out, g["helm"]) < TOL


@pytest.mark.parametrize("name", ["regular", "deformed"])
def test_cport_reference_quad_collection_case(cport, name):
    """TestQuadHelmholtz_MatrixFree_UniformP[_Deformed] (TestQuadCollection.cpp:2612-2782)."""
    g = load("unit_quad.npz")
    n, Q, E = 5, 6, 10
    deformed = name == "deformed"
    out = cport.helmholtz(2, n, Q, E, g[f"{name}_jac"], g[f"{name}_df"], deformed, float(g[f"{name}_lambda"]),
                          np.ones(E * n * n))
    assert rel_err(out, g[f"{name}_out"]) < TOL


def test_cport_reference_hex_collection_case(cport):
    """TestHexHelmholtz_MatrixFree_UniformP_Deformed (TestHexCollection.cpp:3649-3746)."""
    g = load("unit_hex.npz")
    n, Q, E = 4, 5, 10
    out = cport.helmholtz(3, n, Q, E, g["jac"], g["df"], True, float(g["lam"]), np.ones(E * n ** 3))
    assert rel_err(out, g["out"]) < TOL


@pytest.mark.parametrize("nthreads", [1, 4])
def test_cport_cg_matches_reference_recurrence(cport, nthreads):
    """NekLinSysIterCG recurrence (NekLinSysIterCG.cpp:104-263): the same iteration count
    as the reference build and the solution to 1e-12."""
    g = load("cg_quad.npz")
    n, Q = 5, 6
    E = g["l2g"].size // (n * n)
    x, it, eps = cport.cg_solve(2, n, Q, E, g["jac"], g["df"], True, 1.0, g["l2g"], g["sign"], int(g["nglobal"]),
                                int(g["ndir"]), g["dinv"], g["rhs"], 1e-12, 5000, nthreads)
    assert it == int(g["iterations"])
    nd = int(g["ndir"])
    assert rel_err(x[nd:], g["x"][nd:]) < 1e-12


@pytest.mark.parametrize("tag,deformed", [("mesh", True), ("reg", False)])
def test_cport_triangle_helmholtz(cport, tag, deformed):
    """The port's triangle Helmholtz (HelmholtzTriImpl restated) against the reference kernels."""
    from oracle import tri as otri
    g = load("tri.npz")
    n = int(g[f"{tag}_n"])
    tb = otri.TriBasis(n)
    u = g[f"{tag}_u"]
    E = u.size // tb.nc
    out = cport.tri_helmholtz(tb, E, g[f"{tag}_jac"], g[f"{tag}_df"], deformed, 1.3, u, nthreads=2)
    assert rel_err(out, g[f"{tag}_helm"]) < TOL
