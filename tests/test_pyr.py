"""Pyramids: tables, operators, assembly and solves (CPU oracle + GPU kernels).

Pinning: tests/golden/pyr.npz holds outputs of the reference's own pyramid kernels
(MatrixFreeOps BwdTransPyrKernel / IProductPyrKernel / PhysDerivPyrKernel and the
HelmholtzPyrImpl / IProductWRTDerivBasePyrImpl compositions, Polylib zwgrjm / Dgrjm with
alpha 2 and the eModifiedPyr_C rows), including the MatrixFree Helmholtz case of
library/UnitTests/Collections/TestPyrCollection.cpp; made by tests/golden/make_pyr_golden.py.
The oracle (oracle/pyr.py) is held to them; the GPU to the oracle at every order (FP64
1e-12, FP32 2e-5 relative, max-norm) and to the fixtures directly.
"""
import os

import numpy as np
import pytest

from cases import pyr_case, rel_err
from oracle import pyr as opyr

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "pyr.npz"))
TOL64 = 1e-12
TOL32 = 2e-5


@pytest.mark.parametrize("n", range(2, 11))
def test_tables_match_reference(n):
    from ithaca_gpu.operators import basis_pyr
    lib = basis_pyr(n)
    yb = opyr.PyrBasis(n)
    for name, a, o in zip(("z2", "w2", "D2", "B2", "DB2"), lib, (yb.z2, yb.w2, yb.D2, yb.B2.ravel(), yb.DB2.ravel())):
        ref = GOLD[f"t{n}_{name}"]
        scale = max(np.abs(ref).max(), 1.0)
        assert np.abs(a - ref).max() < 2e-13 * scale * n, (name, np.abs(a - ref).max())
        assert np.abs(o - ref).max() < 2e-13 * scale * n, (name, np.abs(o - ref).max())


def test_oracle_unit_cases():
    yb = opyr.PyrBasis(4)
    assert rel_err(opyr.bwdtrans(yb, np.ones(yb.nc)), GOLD["unit_bwd_out"]) < 1e-14
    u = np.ones(10 * yb.nc)
    out = opyr.helmholtz(yb, GOLD["unit_helm_jac"], GOLD["unit_helm_df"], float(GOLD["unit_helm_lambda"]), u)
    assert rel_err(out, GOLD["unit_helm_out"]) < 1e-13
    # the five vertex modes sum to 1
    c = np.zeros(yb.nc)
    verts = [yb.modes.index(v) for v in ((0, 0, 0), (0, 0, 1), (1, 0, 0), (1, 1, 0), (0, 1, 0))]
    c[verts] = 1.0
    assert np.abs(opyr.bwdtrans(yb, c) - 1.0).max() < 1e-14


@pytest.mark.parametrize("tag", ["mesh", "reg"])
def test_oracle_mesh_cases(tag):
    n = int(GOLD[f"{tag}_n"])
    yb = opyr.PyrBasis(n)
    J, df, u = GOLD[f"{tag}_jac"], GOLD[f"{tag}_df"], GOLD[f"{tag}_u"]
    E = u.size // yb.nc
    Jp = J.reshape(E, -1)
    f, g, h = GOLD[f"{tag}_f"], GOLD[f"{tag}_g"], GOLD[f"{tag}_h"]
    assert rel_err(opyr.bwdtrans(yb, u), GOLD[f"{tag}_bwd"]) < 1e-13
    assert rel_err(opyr.iproduct(yb, Jp, f), GOLD[f"{tag}_iprod"]) < 1e-13
    assert rel_err(np.stack(opyr.physderiv(yb, df, f)).reshape(3, -1), GOLD[f"{tag}_deriv"]) < 1e-13
    assert rel_err(opyr.iproduct_deriv(yb, Jp, df, [f, g, h]), GOLD[f"{tag}_iprd"]) < 1e-13
    assert rel_err(opyr.helmholtz(yb, Jp, df, 1.3, u), GOLD[f"{tag}_helm"]) < 1e-13


_XI = np.array([[-1.0, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1]])
_FACES = ((0, 1, 2, 3), (0, 1, 4), (1, 2, 4), (3, 2, 4), (0, 3, 4))


@pytest.mark.parametrize("n", [3, 4, 6])
def test_assembly_is_conforming(n):
    """Both sides of every shared (triangular or quadrilateral) face agree."""
    c = pyr_case(2, 1, 1, n)
    amap = c.mesh.assembly(n)
    x = np.random.default_rng(6).uniform(-1, 1, amap.nglobal)
    loc = (amap.sign * x[amap.l2g]).reshape(c.E, -1)
    EV = c.mesh.EV
    faces = {}
    for e in range(c.E):
        for f in _FACES:
            faces.setdefault(tuple(sorted(EV[e, list(f)])), []).append((e, f))
    checked = 0
    s_ = np.linspace(0.15, 0.85, 4)
    S, T = (a.ravel() for a in np.meshgrid(s_, s_, indexing="ij"))
    w4 = np.stack([(1 - S) * (1 - T), S * (1 - T), S * T, (1 - S) * T], axis=1)   # bilinear weights
    for g, occ in faces.items():
        if len(occ) != 2:
            continue
        wts = np.random.default_rng(len(g)).dirichlet(np.ones(3), size=6)    # barycentric, sorted ids
        vals = []
        ref_cyc = [EV[occ[0][0], v] for v in occ[0][1]]
        for e, f in occ:
            loc_idx = list(f)
            gl = list(EV[e, loc_idx])
            if len(f) == 3:
                lam = np.stack([wts[:, list(g).index(v)] for v in gl], axis=1)
                xi = lam @ _XI[loc_idx]
            else:
                # the same bilinear points of the (straight) face, in this element's cyclic order
                st = np.zeros((S.size, 4))
                st[:, [gl.index(v) for v in ref_cyc]] = w4
                xi = st @ _XI[loc_idx]
            xi = 0.999999999 * xi + 1e-9 * _XI.mean(0)
            vals.append(opyr.modal_values(n, xi[:, 0], xi[:, 1], xi[:, 2]) @ loc[e])
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
        return m.assemble(opyr.helmholtz(c.basis, J, c.df, lam, m.gather(vv)))
    d = np.zeros(m.nglobal)
    np.add.at(d, m.l2g, opyr.helmholtz_diag(c.basis, c.E, J, c.df, lam).reshape(-1))
    return osolve.cg(apply, 1.0 / d[m.ndir:], rhs, m.ndir, tol)


def _manufactured(c, amap, lam):
    from oracle import solve as osolve
    X = c.X
    u = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1]) * np.sin(np.pi * X[2])).reshape(-1)
    f = -(lam + 3 * np.pi ** 2) * u
    J = c.jac.reshape(c.E, -1) if c.deformed else c.jac
    rhs = -osolve.Map.of(amap).assemble(opyr.iproduct(c.basis, J, f))
    return u, f, rhs


def test_oracle_manufactured_solution_converges():
    from oracle import solve as osolve
    errs = []
    for n in (3, 5):
        c = pyr_case(2, 2, 2, n, deformed=False)
        amap = c.mesh.assembly(n)
        u, f, rhs = _manufactured(c, amap, 1.0)
        x, it, _, _ = _oracle_solve(c, amap, 1.0, rhs, 1e-12)
        uh = opyr.bwdtrans(c.basis, osolve.Map.of(amap).gather(x))
        errs.append(np.abs(uh.reshape(-1) - u).max())
    assert errs[1] < errs[0] / 10, errs


# ---------------------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def ctx():
    from ithaca_gpu.operators import Context
    c = Context(0)
    yield c
    c.close()


def _coll(ctx, c, precision="fp64"):
    from ithaca_gpu.operators import Collection
    return Collection(ctx, "pyr", c.n, c.Q, c.E, c.jac, c.df, deformed=c.deformed, precision=precision)


CASES = [(n, True) for n in range(2, 11)] + [(4, False), (7, False)]


@pytest.mark.gpu
@pytest.mark.parametrize("n,deformed", CASES)
def test_gpu_operators_match_oracle(ctx, n, deformed):
    c = pyr_case(1, 1, 1, n, deformed=deformed)
    J = c.jac.reshape(c.E, -1) if deformed else c.jac
    rng = np.random.default_rng(n)
    u = rng.uniform(-1, 1, c.E * c.nm)
    f, g, h = (rng.uniform(-1, 1, c.E * c.nq) for _ in range(3))
    ref = {"bwd": opyr.bwdtrans(c.basis, u), "ipr": opyr.iproduct(c.basis, J, f),
           "deriv": opyr.physderiv(c.basis, c.df, f),
           "iprd": opyr.iproduct_deriv(c.basis, J, c.df, [f, g, h])}
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
            assert rel_err(coll.helmholtz(lam, uu), opyr.helmholtz(c.basis, J, c.df, lam, u)) < tol, (prec, lam)
        if prec == "fp64":
            assert rel_err(coll.helmholtz_diag(2.0), opyr.helmholtz_diag(c.basis, c.E, J, c.df, 2.0)) < tol
        coll.close()


@pytest.mark.gpu
def test_gpu_reference_fixtures(ctx):
    from ithaca_gpu.operators import Collection
    E, n = 10, 4
    coll = Collection(ctx, "pyr", n, n + 1, E, GOLD["unit_helm_jac"], GOLD["unit_helm_df"], deformed=False)
    out = coll.helmholtz(float(GOLD["unit_helm_lambda"]), np.ones(E * n * (n + 1) * (2 * n + 1) // 6))
    assert rel_err(out, GOLD["unit_helm_out"]) < TOL64
    for tag, deformed in (("mesh", True), ("reg", False)):
        n = int(GOLD[f"{tag}_n"])
        nc = n * (n + 1) * (2 * n + 1) // 6
        E = GOLD[f"{tag}_u"].size // nc
        coll = Collection(ctx, "pyr", n, n + 1, E, GOLD[f"{tag}_jac"], GOLD[f"{tag}_df"], deformed=deformed)
        f, g, h, u = GOLD[f"{tag}_f"], GOLD[f"{tag}_g"], GOLD[f"{tag}_h"], GOLD[f"{tag}_u"]
        assert rel_err(coll.bwdtrans(u), GOLD[f"{tag}_bwd"]) < TOL64
        assert rel_err(coll.iproduct(f), GOLD[f"{tag}_iprod"]) < TOL64
        assert rel_err(np.stack(coll.physderiv(f)), GOLD[f"{tag}_deriv"]) < TOL64
        assert rel_err(coll.iproduct_deriv([f, g, h]), GOLD[f"{tag}_iprd"]) < TOL64
        assert rel_err(coll.helmholtz(1.3, u), GOLD[f"{tag}_helm"]) < TOL64


@pytest.mark.gpu
def test_gpu_geometry(ctx):
    from ithaca_gpu.operators import geom_factors
    c = pyr_case(2, 1, 2, 5)
    jac, df = geom_factors(ctx, "pyr", c.Q, c.X)
    assert rel_err(jac, c.jac) < 1e-12
    assert rel_err(df, c.df) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("n", [3, 5])
def test_gpu_cg_matches_oracle(ctx, n):
    from ithaca_gpu.operators import GlobalLinSysIterativeFullGPU, GlobalLinSysIterativeStaticCondGPU
    from oracle import solve as osolve
    c = pyr_case(2, 2, 1, n)
    amap = c.mesh.assembly(n)
    coll = _coll(ctx, c)
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    rhs = np.random.default_rng(9).uniform(-1, 1, amap.nglobal)
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
    assert sc.info()["nint_local"] == sum(1 for (p, q, r) in c.basis.modes if p >= 2 and q >= 2 and r >= 1)
    loc_sc, _ = sc.helmsolve(1.0, f, tol=1e-12)
    assert rel_err(loc_sc, loc) < 1e-9
    sc.close()
    sysg.close()
    coll.close()
