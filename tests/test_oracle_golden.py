"""The numpy oracle against golden vectors produced by the reference's own compiled code.

Fixtures: tests/golden/*.npz, written by tests/golden/make_golden.py from
oracle/_ref (reference Polylib.cpp + MatrixFreeOps kernels compiled in place).
Tolerance: 1e-13 relative (both sides are FP64; only the summation order differs).
"""
import os

import numpy as np
import pytest

from cases import rel_err
from oracle import basis as obasis
from oracle import geom as ogeom
from oracle import ops as oops
from oracle import polylib
from oracle import solve as osolve

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-13


def load(name):
    return np.load(os.path.join(G, name))


@pytest.mark.parametrize("n", range(2, 11))
def test_basis_tables(n):
    g = load("basis.npz")
    Q = n + 1
    b = obasis.Basis1D(n, Q)
    assert np.max(np.abs(b.z - g[f"z{n}"])) < 1e-15
    assert np.max(np.abs(b.w - g[f"w{n}"])) < 1e-15
    assert rel_err(b.D, g[f"D{n}"]) < TOL
    assert rel_err(b.B, g[f"B{n}"]) < TOL
    assert rel_err(b.DB, g[f"DB{n}"]) < TOL


def test_gll_quadrature_exactness():
    for Q in range(3, 12):
        z, w = polylib.gll(Q)
        for k in range(0, 2 * Q - 2):  # GLL is exact to degree 2Q - 3
            exact = 0.0 if k % 2 else 2.0 / (k + 1)
            assert abs(np.dot(w, z ** k) - exact) < 1e-13


@pytest.mark.parametrize("name", ["regular", "deformed"])
def test_reference_quad_collection_case(name):
    """TestQuadHelmholtz_MatrixFree_UniformP[_Deformed] inputs, reference-kernel outputs."""
    g = load("unit_quad.npz")
    n, Q, E = 5, 6, 10
    b = obasis.Basis1D(n, Q)
    jac = g[f"{name}_jac"]
    out = oops.helmholtz(b, 2, jac.reshape(E, -1), g[f"{name}_df"], float(g[f"{name}_lambda"]), np.ones(E * n * n))
    assert rel_err(out, g[f"{name}_out"]) < TOL


def test_reference_hex_collection_case():
    g = load("unit_hex.npz")
    n, Q, E = 4, 5, 10
    b = obasis.Basis1D(n, Q)
    out = oops.helmholtz(b, 3, g["jac"].reshape(E, -1), g["df"], float(g["lam"]), np.ones(E * n ** 3))
    assert rel_err(out, g["out"]) < TOL


@pytest.mark.parametrize("fname,n,dim", [("mesh_quad.npz", 7, 2), ("mesh_hex.npz", 5, 3)])
def test_all_operators_on_seeded_mesh(fname, n, dim):
    g = load(fname)
    Q = n + 1
    b = obasis.Basis1D(n, Q)
    E = g["X"].shape[1]
    jac = g["jac"].reshape(E, -1)
    assert rel_err(oops.bwdtrans(b, dim, g["u"]), g["bwd"]) < TOL
    assert rel_err(oops.iproduct(b, dim, jac, g["f"]), g["iprod"]) < TOL
    for d, r in zip(oops.physderiv(b, dim, g["df"], g["f"]), g["deriv"]):
        assert rel_err(d, r) < TOL
    assert rel_err(oops.helmholtz(b, dim, jac, g["df"], 1.0, g["u"]), g["helm"]) < TOL
    # geometry restatement reproduces the stored factors
    j2, df2 = ogeom.geom_factors(g["X"], b.D2, dim)
    assert rel_err(j2, g["jac"]) < TOL and rel_err(df2, g["df"]) < TOL


def test_reference_cg_recurrence():
    g = load("cg_quad.npz")
    n, Q = 5, 6
    b = obasis.Basis1D(n, Q)
    E = g["l2g"].size // (n * n)
    m = osolve.Map(g["l2g"], g["sign"], int(g["nglobal"]), int(g["ndir"]))
    jac = g["jac"].reshape(E, -1)
    dinv = osolve.jacobi_inverse(b, 2, jac, g["df"], 1.0, m)
    assert rel_err(dinv, g["dinv"]) < TOL
    x, it, eps, _ = osolve.cg(lambda v: osolve.global_apply(b, 2, jac, g["df"], 1.0, m, v), dinv, g["rhs"],
                              m.ndir, tol=1e-12)
    assert it == int(g["iterations"])
    assert rel_err(x[m.ndir:], g["x"][m.ndir:]) < 1e-11


def test_bilinear_jacobian_is_analytic():
    """J of a straight-sided quad equals the determinant of the analytic bilinear map."""
    from ithaca_gpu.mesh import QuadMesh
    mesh = QuadMesh(2, 2, jitter=0.2, seed=3)
    Q = 6
    b = obasis.Basis1D(5, Q)
    X = mesh.coords(Q)
    jac, df = ogeom.geom_factors(X, b.D2, 2)
    z = b.z
    xi0, xi1 = np.meshgrid(z, z, indexing="xy")  # [j, i]
    for e in range(mesh.E):
        v = mesh.V[mesh.EV[e]]
        dx0 = 0.25 * ((1 - xi1)[..., None] * (v[1] - v[0]) + (1 + xi1)[..., None] * (v[2] - v[3]))
        dx1 = 0.25 * ((1 - xi0)[..., None] * (v[3] - v[0]) + (1 + xi0)[..., None] * (v[2] - v[1]))
        det = dx0[..., 0] * dx1[..., 1] - dx0[..., 1] * dx1[..., 0]
        assert np.max(np.abs(jac[e] - det.reshape(-1))) < 1e-13


@pytest.mark.parametrize("fname,n,dim", [("mesh_quad.npz", 7, 2), ("mesh_hex.npz", 5, 3)])
def test_iproduct_deriv_composes_the_laplacian(fname, n, dim):
    """IProductWRTDerivBase of the physical gradient is the Laplacian part of the
    Helmholtz operator, which the golden vectors pin to the compiled reference kernels:
    sum_k (d phi / d x_k, d u / d x_k) = L u (lambda = 0)."""
    g = load(fname)
    b = obasis.Basis1D(n, n + 1)
    E = g["X"].shape[1]
    jac = g["jac"].reshape(E, -1)
    grads = oops.physderiv(b, dim, g["df"], oops.bwdtrans(b, dim, g["u"]))
    lap = oops.iproduct_deriv(b, dim, jac, g["df"], grads)
    assert rel_err(lap, oops.helmholtz(b, dim, jac, g["df"], 0.0, g["u"])) < 1e-12
