"""Solve-level known answers stored with the reference's regression tests.

library/Demos/MultiRegions/Tests/Helmholtz3D_CG_Hex.tst runs the Helmholtz3D demo on
Helmholtz3D_Hex_P6.xml: the unit cube as 2 x 2 x 2 hexahedra, ModifiedA with 6 modes
(GLL, 7 points), lambda = 1, Dirichlet u = sin(pi x/2) sin(pi y/2) sin(pi z/2) on the
whole boundary, forcing f = -(lambda + 3 pi^2 / 4) u, and stores the errors of the
discrete solution against that exact solution: L2 = 1.11818e-07 and Linf = 5.66374e-07
(tolerance 1e-12). The Dirichlet data enter as the boundary-constrained projections of
the boundary expansions (oracle/bc.py); the reference solves directly (static
condensation), the CG here runs to 1e-14 so that the two discrete solutions agree far
below the tolerance. The CPU test runs the oracle; the GPU test the library's HelmSolve.
"""
import numpy as np
import pytest

from cases import hex_dirichlet
from oracle import basis as obasis
from oracle import geom as ogeom
from oracle import ops as oops
from oracle import solve as osolve

L2_REF, LINF_REF, TOL = 1.11818e-07, 5.66374e-07, 1e-12
LAM = 1.0


def _exact(x, y, z):
    return np.sin(0.5 * np.pi * x) * np.sin(0.5 * np.pi * y) * np.sin(0.5 * np.pi * z)


def _problem():
    from ithaca_gpu.mesh import HexMesh
    n, Q = 6, 7
    mesh = HexMesh(2, 2, 2)
    b = obasis.Basis1D(n, Q)
    X = mesh.coords(Q)
    jac, df = ogeom.geom_factors(X, b.D2, 3)
    amap = mesh.assembly(n)
    u = _exact(X[0], X[1], X[2]).reshape(-1)
    f = -(LAM + 0.75 * np.pi ** 2) * u
    xd = hex_dirichlet(mesh, amap, b, X, _exact)
    return mesh, b, X, jac.reshape(mesh.E, -1), df, amap, u, f, xd


def _errors(b, jac, coeffs, u, E):
    uh = oops.bwdtrans(b, 3, coeffs).reshape(E, -1)
    w3 = np.einsum("k,j,i->kji", b.w, b.w, b.w).reshape(-1)
    err = uh - u.reshape(E, -1)
    return np.sqrt(np.sum(jac * w3[None, :] * err ** 2)), np.max(np.abs(err))


def test_helmholtz3d_cg_hex_oracle():
    mesh, b, X, jac, df, amap, u, f, xd = _problem()
    coeffs, _ = osolve.helmsolve(b, 3, jac, df, LAM, amap, f, tol=1e-14, dirichlet=xd)
    l2, linf = _errors(b, jac, coeffs, u, mesh.E)
    assert abs(l2 - L2_REF) < TOL, l2
    assert abs(linf - LINF_REF) < TOL, linf


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_helmholtz3d_cg_hex_gpu(mode):
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU
    mesh, b, X, jac, df, amap, u, f, xd = _problem()
    ctx = Context(0)
    coll = Collection(ctx, "hex", b.n, b.Q, mesh.E, jac.reshape(-1), df, deformed=True)
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    coeffs, res = sysg.helmsolve(LAM, f, dirichlet=xd, tol=1e-14, mode=mode)
    l2, linf = _errors(b, jac, coeffs, u, mesh.E)
    assert abs(l2 - L2_REF) < TOL, l2
    assert abs(linf - LINF_REF) < TOL, linf
