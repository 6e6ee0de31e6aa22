"""The 2-D known answer stored with the reference's regression tests, read through the
library's session reader.

library/Demos/MultiRegions/Tests/Helmholtz2D_CG_P7_PreconDiagonal.tst runs the
Helmholtz2D demo with Preconditioner=Diagonal on Helmholtz2D_P7_Periodic.xml: 4 x 4
quads of [0, 1.5]^2 (edges given with mixed orientations), 7 ModifiedA modes, lambda = 1,
periodic in y, Dirichlet u = sin(4 pi x/3 + pi/2) sin(4 pi y/3 + pi/2) at x = 0 and 1.5,
GlobalSysSoln = IterativeStaticCond, default tolerance 1e-9. It stores L2 = 6.82374e-07
and Linf = 9.43919e-07 (tolerance 1e-8) and 17 CG iterations (tolerance 2).

The session is read from the reference tree where it exists (CPU test) and otherwise from
tests/golden/session_helmholtz2d_p7_periodic.json, written from it by
tests/golden/make_session_fixtures.py. The oracle (CPU) and the library (GPU) run the
statically condensed solve (the session's GlobalSysSoln) and the full system.
"""
import json
import os

import numpy as np
import pytest

from oracle import basis as obasis
from oracle import bc as obc
from oracle import geom as ogeom
from oracle import ops as oops
from oracle import solve as osolve
from oracle import statcond as osc

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "session_helmholtz2d_p7_periodic.json")
REF_XML = os.path.join(os.environ.get("ITHACA_REFERENCE", "/root/reference"),
                       "library/Demos/MultiRegions/Tests/Helmholtz2D_P7_Periodic.xml")
L2_REF, LINF_REF, TOL = 6.82374e-07, 9.43919e-07, 1e-8
ITERS_REF, ITERS_TOL = 17, 2


def _session():
    from ithaca_gpu.session import Session
    return Session.from_dict(json.load(open(FIXTURE))["session"])


def _problem():
    from ithaca_gpu.session import QuadSessionMesh
    s = _session()
    mesh = QuadSessionMesh(s)
    n = s.nummodes()
    Q = n + 1
    b = obasis.Basis1D(n, Q)
    X = mesh.coords(Q)
    jac, df = ogeom.geom_factors(X, b.D2, 2)
    amap = mesh.assembly(n)
    exact = s.function("ExactSolution")
    u = exact(X[0], X[1]).reshape(-1)
    f = s.function("Forcing")(X[0], X[1]).reshape(-1)
    dvals = mesh.dirichlet_coefficients(n, exact, amap)
    return s, mesh, b, X, jac.reshape(mesh.E, -1), df, amap, u, f, dvals


def _errors(b, jac, coeffs, u, E):
    uh = oops.bwdtrans(b, 2, coeffs).reshape(E, -1)
    err = uh - u.reshape(E, -1)
    return np.sqrt(np.sum(jac * np.outer(b.w, b.w).reshape(-1)[None, :] * err ** 2)), np.max(np.abs(err))


@pytest.mark.skipif(not os.path.exists(REF_XML), reason="reference tree not present")
def test_reader_matches_fixture():
    from ithaca_gpu.session import read_session
    s = read_session(REF_XML)
    assert json.loads(json.dumps(s.to_dict())) == json.load(open(FIXTURE))["session"]
    assert s.solverinfo["GlobalSysSoln"] == "IterativeStaticCond" and s.parameters["Lambda"] == 1.0


def test_mesh_periodic_and_dirichlet_structure():
    s, mesh, b, X, jac, df, amap, u, f, dvals = _problem()
    assert mesh.E == 16 and len(mesh.periodic_pairs) == 4 and len(mesh.dirichlet_edges) == 8
    assert np.all(jac > 0)
    # the periodic identification removes the top row of vertex and edge dofs:
    # 5 x 4 vertices, (4 x 4 horizontal + 5 x 4 vertical) edges x 5 modes, 16 x 25 interior
    assert amap.nglobal == 20 + 36 * 5 + 16 * 25
    # Dirichlet data: the session's edge projection equals the oracle's boundary-constrained one
    exact = s.function("ExactSolution")
    z = b.z
    for e in sorted(mesh.dirichlet_edges):
        va, vb = mesh.EDGES[e]
        pts = np.outer(0.5 * (1 - z), mesh.V[va]) + np.outer(0.5 * (1 + z), mesh.V[vb])
        c = obc.seg_fwd_bnd(b, exact(pts[:, 0], pts[:, 1]))
        assert abs(dvals[mesh._newid[mesh._vnum[mesh._vrep[va]]]] - c[0]) < 1e-15
    # a constant is reproduced exactly by the Dirichlet projection
    ones = mesh.dirichlet_coefficients(b.n, lambda x, y: np.ones_like(x), amap)
    verts = [mesh._newid[mesh._vnum[c]] for c in set(mesh._vrep[np.concatenate([mesh.EDGES[e] for e in mesh.dirichlet_edges])])]
    assert np.allclose(ones[verts], 1.0) and np.allclose(np.delete(ones, verts), 0.0, atol=1e-14)


def test_known_answer_oracle_static_condensation():
    s, mesh, b, X, jac, df, amap, u, f, dvals = _problem()
    lam = s.parameters["Lambda"]
    coeffs, it, _ = osc.helmsolve(b, 2, jac, df, lam, amap, f, tol=1e-9, dirichlet=dvals)
    l2, linf = _errors(b, jac, coeffs, u, mesh.E)
    assert abs(l2 - L2_REF) < TOL and abs(linf - LINF_REF) < TOL, (l2, linf)
    assert abs(it - ITERS_REF) <= ITERS_TOL, it
    full, _ = osolve.helmsolve(b, 2, jac, df, lam, amap, f, tol=1e-12, dirichlet=dvals)
    l2f, linff = _errors(b, jac, full.reshape(-1), u, mesh.E)
    assert abs(l2f - L2_REF) < TOL and abs(linff - LINF_REF) < TOL


@pytest.mark.gpu
def test_known_answer_gpu():
    from ithaca_gpu.operators import (Collection, Context, GlobalLinSysIterativeFullGPU,
                                      GlobalLinSysIterativeStaticCondGPU, geom_factors)
    s, mesh, b, X, jac, df, amap, u, f, dvals = _problem()
    lam = s.parameters["Lambda"]
    ctx = Context(0)
    jg, dfg = geom_factors(ctx, "quad", b.Q, X)
    coll = Collection(ctx, "quad", b.n, b.Q, mesh.E, jg, dfg)
    sc = GlobalLinSysIterativeStaticCondGPU(coll, amap)
    coeffs, res = sc.helmsolve(lam, f, dirichlet=dvals, tol=1e-9)
    l2, linf = _errors(b, jac, coeffs, u, mesh.E)
    assert abs(l2 - L2_REF) < TOL and abs(linf - LINF_REF) < TOL, (l2, linf)
    assert abs(res.iterations - ITERS_REF) <= ITERS_TOL, res.iterations
    full, resf = GlobalLinSysIterativeFullGPU(coll, amap).helmsolve(lam, f, dirichlet=dvals, tol=1e-12)
    l2f, linff = _errors(b, jac, full, u, mesh.E)
    assert abs(l2f - L2_REF) < TOL and abs(linff - LINF_REF) < TOL, (l2f, linff)
    ctx.close()
