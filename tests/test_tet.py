"""Tetrahedra: tables and operators (CPU oracle + GPU kernels).

Pinning: tests/golden/tet.npz holds outputs of the reference's own tetrahedron kernels
(MatrixFreeOps BwdTransTetKernel / IProductTetKernel / PhysDerivTetKernel and the
HelmholtzTetImpl / IProductWRTDerivBaseTetImpl compositions, Polylib zwgrjm / Dgrjm with
alpha 1 and 2), including the MatrixFree cases of
library/UnitTests/Collections/TestTetCollection.cpp; made by tests/golden/make_tet_golden.py.
The oracle (oracle/tet.py) is held to them; the GPU to the oracle at every order (FP64
1e-12, FP32 2e-5 relative, max-norm) and to the fixtures directly.
"""
import os

import numpy as np
import pytest

from cases import rel_err, tet_case
from oracle import tet as otet

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "tet.npz"))
TOL64 = 1e-12
TOL32 = 2e-5
NAMES = ("z0", "w0", "D0", "B0", "DB0", "z1", "w1", "D1", "B1", "DB1", "z2", "w2", "D2", "B2", "DB2")


@pytest.mark.parametrize("n", range(2, 11))
def test_tables_match_reference(n):
    from ithaca_gpu.operators import basis_tet, basis_tri
    a, b = basis_tri(n)
    c = basis_tet(n)
    tb = otet.TetBasis(n)
    orc = [tb.z0, tb.w0, tb.D0, tb.B0.ravel(), tb.DB0.ravel(), tb.z1, tb.w1, tb.D1, tb.B1.ravel(), tb.DB1.ravel(),
           tb.z2, tb.w2, tb.D2, tb.B2.ravel(), tb.DB2.ravel()]
    for name, lib, o in zip(NAMES, list(a) + list(b) + list(c), orc):
        ref = GOLD[f"t{n}_{name}"]
        scale = max(np.abs(ref).max(), 1.0)
        assert np.abs(lib - ref).max() < 2e-13 * scale * n, (name, np.abs(lib - ref).max())
        assert np.abs(o - ref).max() < 2e-13 * scale * n, (name, np.abs(o - ref).max())


def test_oracle_unit_cases():
    tb = otet.TetBasis(4)
    assert rel_err(otet.bwdtrans(tb, GOLD["unit_bwd_in"]), GOLD["unit_bwd_out"]) < 1e-14
    c = np.zeros(tb.nc)
    c[[0, 1, tb.n, tb.n * (tb.n + 1) // 2]] = 1.0   # the four vertex modes: 1 everywhere
    assert np.abs(otet.bwdtrans(tb, c) - 1.0).max() < 1e-14
    for tag in ("undeformed", "deformed"):
        J, df, f = GOLD[f"unit_ipr_{tag}_jac"], GOLD[f"unit_ipr_{tag}_df"], GOLD[f"unit_ipr_{tag}_f"]
        assert rel_err(otet.iproduct(tb, J, f), GOLD[f"unit_ipr_{tag}_out"]) < 1e-13
        assert rel_err(np.stack(otet.physderiv(tb, df, f)).reshape(3, -1), GOLD[f"unit_deriv_{tag}_out"]) < 1e-13
    u = np.ones(10 * tb.nc)
    out = otet.helmholtz(tb, GOLD["unit_helm_jac"], GOLD["unit_helm_df"], float(GOLD["unit_helm_lambda"]), u)
    assert rel_err(out, GOLD["unit_helm_out"]) < 1e-13


@pytest.mark.parametrize("tag", ["mesh", "reg"])
def test_oracle_mesh_cases(tag):
    n = int(GOLD[f"{tag}_n"])
    tb = otet.TetBasis(n)
    J, df, u = GOLD[f"{tag}_jac"], GOLD[f"{tag}_df"], GOLD[f"{tag}_u"]
    E = u.size // tb.nc
    Jp = J.reshape(E, -1)
    f, g, h = GOLD[f"{tag}_f"], GOLD[f"{tag}_g"], GOLD[f"{tag}_h"]
    assert rel_err(otet.bwdtrans(tb, u), GOLD[f"{tag}_bwd"]) < 1e-13
    assert rel_err(otet.iproduct(tb, Jp, f), GOLD[f"{tag}_iprod"]) < 1e-13
    assert rel_err(np.stack(otet.physderiv(tb, df, f)).reshape(3, -1), GOLD[f"{tag}_deriv"]) < 1e-13
    assert rel_err(otet.iproduct_deriv(tb, Jp, df, [f, g, h]), GOLD[f"{tag}_iprd"]) < 1e-13
    assert rel_err(otet.helmholtz(tb, Jp, df, 1.3, u), GOLD[f"{tag}_helm"]) < 1e-13


def test_geometry_straight_equals_affine():
    c = tet_case(2, 1, 1, 4, curve=0.0)
    J, df = otet.geom_factors(c.basis, c.X)
    Jr, dfr = otet.straight_tet_geometry(c.mesh.V[c.mesh.EV])
    assert rel_err(J.reshape(c.E, -1), np.repeat(Jr[:, None], c.nq, 1)) < 1e-12
    assert rel_err(df.reshape(9, c.E, -1), np.repeat(dfr[:, :, None], c.nq, 2)) < 1e-12
    assert np.all(Jr > 0)
    assert abs(np.sum(J.reshape(c.E, -1) * c.basis.weights()[None]) - 1.0) < 1e-13


# ---------------------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def ctx():
    from ithaca_gpu.operators import Context
    c = Context(0)
    yield c
    c.close()


def _coll(ctx, c, precision="fp64"):
    from ithaca_gpu.operators import Collection
    return Collection(ctx, "tet", c.n, c.Q, c.E, c.jac, c.df, deformed=c.deformed, precision=precision)


CASES = [(n, True) for n in range(2, 11)] + [(4, False), (7, False)]


@pytest.mark.gpu
@pytest.mark.parametrize("n,deformed", CASES)
def test_gpu_operators_match_oracle(ctx, n, deformed):
    c = tet_case(1, 1, 1, n, deformed=deformed)
    J = c.jac.reshape(c.E, -1) if deformed else c.jac
    rng = np.random.default_rng(n)
    u = rng.uniform(-1, 1, c.E * c.nm)
    f, g, h = (rng.uniform(-1, 1, c.E * c.nq) for _ in range(3))
    ref = {"bwd": otet.bwdtrans(c.basis, u), "ipr": otet.iproduct(c.basis, J, f),
           "deriv": otet.physderiv(c.basis, c.df, f), "iprd": otet.iproduct_deriv(c.basis, J, c.df, [f, g, h])}
    for prec, tol in (("fp64", TOL64), ("fp32", TOL32)):
        coll = _coll(ctx, c, prec)
        dt = np.float64 if prec == "fp64" else np.float32
        uu, ff, gg, hh = (x.astype(dt) for x in (u, f, g, h))
        assert coll.Ndof() == c.E * c.nm
        assert rel_err(coll.bwdtrans(uu), ref["bwd"]) < tol
        assert rel_err(coll.iproduct(ff), ref["ipr"]) < tol
        d = coll.physderiv(ff)
        assert max(rel_err(d[k], ref["deriv"][k]) for k in range(3)) < tol
        assert rel_err(coll.iproduct_deriv([ff, gg, hh]), ref["iprd"]) < tol
        for lam in (0.0, 1.0, 10.0):
            assert rel_err(coll.helmholtz(lam, uu), otet.helmholtz(c.basis, J, c.df, lam, u)) < tol, (prec, lam)
        if prec == "fp64":
            assert rel_err(coll.helmholtz_diag(2.0), otet.helmholtz_diag(c.basis, c.E, J, c.df, 2.0)) < tol
        coll.close()


@pytest.mark.gpu
def test_gpu_reference_fixtures(ctx):
    from ithaca_gpu.operators import Collection
    E = 10
    coll = Collection(ctx, "tet", 4, 5, E, GOLD["unit_helm_jac"], GOLD["unit_helm_df"], deformed=False)
    out = coll.helmholtz(float(GOLD["unit_helm_lambda"]), np.ones(E * 20))
    assert rel_err(out, GOLD["unit_helm_out"]) < TOL64
    for tag, deformed in (("mesh", True), ("reg", False)):
        n = int(GOLD[f"{tag}_n"])
        nc = n * (n + 1) * (n + 2) // 6
        E = GOLD[f"{tag}_u"].size // nc
        coll = Collection(ctx, "tet", n, n + 1, E, GOLD[f"{tag}_jac"], GOLD[f"{tag}_df"], deformed=deformed)
        f, g, h, u = GOLD[f"{tag}_f"], GOLD[f"{tag}_g"], GOLD[f"{tag}_h"], GOLD[f"{tag}_u"]
        assert rel_err(coll.bwdtrans(u), GOLD[f"{tag}_bwd"]) < TOL64
        assert rel_err(coll.iproduct(f), GOLD[f"{tag}_iprod"]) < TOL64
        assert rel_err(np.stack(coll.physderiv(f)), GOLD[f"{tag}_deriv"]) < TOL64
        assert rel_err(coll.iproduct_deriv([f, g, h]), GOLD[f"{tag}_iprd"]) < TOL64
        assert rel_err(coll.helmholtz(1.3, u), GOLD[f"{tag}_helm"]) < TOL64


@pytest.mark.gpu
def test_gpu_geometry(ctx):
    from ithaca_gpu.operators import geom_factors
    c = tet_case(2, 2, 1, 5)
    jac, df = geom_factors(ctx, "tet", c.Q, c.X)
    assert rel_err(jac, c.jac) < 1e-12
    assert rel_err(df, c.df) < 1e-12


_XI = np.array([[-1.0, -1, -1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]])


@pytest.mark.parametrize("n", [3, 4, 6])
def test_assembly_is_conforming(n):
    """A global vector expands to the same values on both sides of every shared face."""
    c = tet_case(2, 2, 1, n, jitter=0.2)
    amap = c.mesh.assembly(n)
    x = np.random.default_rng(5).uniform(-1, 1, amap.nglobal)
    loc = (amap.sign * x[amap.l2g]).reshape(c.E, -1)
    EV = c.mesh.EV
    faces = {}
    for e in range(c.E):
        for f in ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)):
            g = tuple(sorted(EV[e, list(f)]))
            faces.setdefault(g, []).append(e)
    lam = np.array([(a, b) for a in (0.1, 0.3, 0.55) for b in (0.15, 0.35) if a + b < 0.9])
    bary = np.stack([1 - lam.sum(1), lam[:, 0], lam[:, 1]], axis=1)   # w.r.t. the sorted global ids
    checked = 0
    for g, els in faces.items():
        if len(els) != 2:
            continue
        vals = []
        for e in els:
            loc_idx = [int(np.flatnonzero(EV[e] == gv)[0]) for gv in g]
            xi = bary @ _XI[loc_idx]
            xi = 0.999999999 * xi + 1e-9 * _XI.mean(0)
            vals.append(otet.modal_values(n, xi[:, 0], xi[:, 1], xi[:, 2]) @ loc[e])
        assert np.abs(vals[0] - vals[1]).max() < 1e-7, g
        checked += 1
    assert checked > 0


def _oracle_solve(c, amap, lam, rhs, tol):
    from oracle import solve as osolve
    m = osolve.Map.of(amap)
    J = c.jac.reshape(c.E, -1) if c.deformed else c.jac

    def apply(v):
        vv = v.copy()
        vv[:m.ndir] = 0
        return m.assemble(otet.helmholtz(c.basis, J, c.df, lam, m.gather(vv)))
    d = np.zeros(m.nglobal)
    np.add.at(d, m.l2g, otet.helmholtz_diag(c.basis, c.E, J, c.df, lam).reshape(-1))
    return osolve.cg(apply, 1.0 / d[m.ndir:], rhs, m.ndir, tol)


def _manufactured(c, amap, lam):
    from oracle import solve as osolve
    X = c.X
    u = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1]) * np.sin(np.pi * X[2])).reshape(-1)
    f = -(lam + 3 * np.pi ** 2) * u
    J = c.jac.reshape(c.E, -1) if c.deformed else c.jac
    rhs = -osolve.Map.of(amap).assemble(otet.iproduct(c.basis, J, f))
    return u, f, rhs


def test_oracle_manufactured_solution_converges():
    from oracle import solve as osolve
    errs = []
    for n in (3, 5):
        c = tet_case(2, 2, 2, n, curve=0.0, jitter=0.0)
        amap = c.mesh.assembly(n)
        u, f, rhs = _manufactured(c, amap, 1.0)
        x, it, _, _ = _oracle_solve(c, amap, 1.0, rhs, 1e-12)
        uh = otet.bwdtrans(c.basis, osolve.Map.of(amap).gather(x))
        errs.append(np.abs(uh.reshape(-1) - u).max())
    assert errs[1] < errs[0] / 10, errs


@pytest.mark.gpu
@pytest.mark.parametrize("n", [3, 5])
def test_gpu_cg_matches_oracle(ctx, n):
    from ithaca_gpu.operators import GlobalLinSysIterativeFullGPU, GlobalLinSysIterativeStaticCondGPU
    from oracle import solve as osolve
    c = tet_case(2, 2, 1, n)
    amap = c.mesh.assembly(n)
    coll = _coll(ctx, c)
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    rhs = np.random.default_rng(8).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    x, res = sysg.solve(1.2, rhs, tol=1e-12)
    xo, it_o, _, _ = _oracle_solve(c, amap, 1.2, rhs, 1e-12)
    assert abs(res.iterations - it_o) <= max(2, it_o // 50), (res.iterations, it_o)
    assert rel_err(x[amap.ndir:], xo[amap.ndir:]) < 1e-10
    xm, rm = sysg.solve(1.2, rhs, tol=1e-10, mode="mixed")
    assert rm.rel_residual < 1e-10
    u, f, rhs2 = _manufactured(c, amap, 1.0)
    loc, _ = sysg.helmsolve(1.0, f, tol=1e-12)
    xo2, _, _, _ = _oracle_solve(c, amap, 1.0, rhs2, 1e-12)
    assert rel_err(loc, osolve.Map.of(amap).gather(xo2)) < 1e-10
    sc = GlobalLinSysIterativeStaticCondGPU(coll, amap)
    assert sc.info()["nint_local"] == (n - 2) * (n - 3) * (n - 4) // 6
    loc_sc, _ = sc.helmsolve(1.0, f, tol=1e-12)
    assert rel_err(loc_sc, loc) < 1e-9
    sc.close()
    sysg.close()
    coll.close()
