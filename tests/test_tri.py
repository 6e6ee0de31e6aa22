"""Triangles: tables, operators, assembly and solves (CPU oracle + GPU kernels).

Pinning: tests/golden/tri.npz holds outputs of the reference's own triangle kernels
(MatrixFreeOps BwdTransTriKernel / IProductTriKernel / PhysDerivTriKernel and the
HelmholtzTriImpl / IProductWRTDerivBaseTriImpl compositions, Polylib zwgrjm / Dgrjm),
including the MatrixFree cases of library/UnitTests/Collections/TestTriCollection.cpp;
made by tests/golden/make_tri_golden.py. The oracle (oracle/tri.py) is checked against
them, then the GPU against the oracle at every order (FP64 1e-12, FP32 2e-5 relative,
the max-norm of the difference over that of the reference value) and against the
fixtures directly.
"""
import os

import numpy as np
import pytest

from cases import rel_err, tri_case
from oracle import solve as osolve
from oracle import tri as otri

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "tri.npz"))
TOL64 = 1e-12
TOL32 = 2e-5


# ---------------------------------------------------------------------------- CPU
@pytest.mark.parametrize("n", range(2, 13))
def test_tables_match_reference(n):
    """Library host tables and the oracle's against Polylib / Basis (eModified_B)."""
    from ithaca_gpu.operators import basis_tri
    lib_a, lib_b = basis_tri(n)
    tb = otri.TriBasis(n)
    orc = [tb.z0, tb.w0, tb.D0, tb.B0.ravel(), tb.DB0.ravel(), tb.z1, tb.w1, tb.D1, tb.B1.ravel(), tb.DB1.ravel()]
    names = ["z0", "w0", "D0", "B0", "DB0", "z1", "w1", "D1", "B1", "DB1"]
    for name, lib, o in zip(names, list(lib_a) + list(lib_b), orc):
        ref = GOLD[f"t{n}_{name}"]
        scale = max(np.abs(ref).max(), 1.0)
        assert np.abs(lib - ref).max() < 1e-13 * scale * n, (name, np.abs(lib - ref).max())
        assert np.abs(o - ref).max() < 1e-13 * scale * n, (name, np.abs(o - ref).max())


def test_oracle_unit_cases():
    """The TestTriCollection.cpp MatrixFree cases through the oracle."""
    tb4, tb2 = otri.TriBasis(4), otri.TriBasis(2)
    assert rel_err(otri.bwdtrans(tb4, GOLD["unit_bwd_in"]), GOLD["unit_bwd_out"]) < 1e-14
    # all coefficients 1 on the standard triangle: a known polynomial; bwd of the three
    # vertex modes alone is 1 everywhere (partition of unity with the top-vertex term)
    c = np.zeros(tb4.nc)
    c[[0, 1, tb4.n]] = 1.0
    assert np.abs(otri.bwdtrans(tb4, c) - 1.0).max() < 1e-14
    for tag in ("undeformed", "deformed"):
        out = otri.iproduct(tb4, GOLD[f"unit_ipr_{tag}_jac"], GOLD[f"unit_ipr_{tag}_f"])
        assert rel_err(out, GOLD[f"unit_ipr_{tag}_out"]) < 1e-13
        d = otri.physderiv(tb2, GOLD[f"unit_deriv_{tag}_df"], GOLD[f"unit_deriv_{tag}_f"])
        assert rel_err(np.stack(d).reshape(2, -1), GOLD[f"unit_deriv_{tag}_out"]) < 1e-13
    E = 10
    u = np.ones(E * tb4.nc)
    out = otri.helmholtz(tb4, GOLD["unit_helm_jac"], GOLD["unit_helm_df"], float(GOLD["unit_helm_lambda"]), u)
    assert rel_err(out, GOLD["unit_helm_out"]) < 1e-13


@pytest.mark.parametrize("tag", ["mesh", "reg"])
def test_oracle_mesh_cases(tag):
    n = int(GOLD[f"{tag}_n"])
    tb = otri.TriBasis(n)
    J, df = GOLD[f"{tag}_jac"], GOLD[f"{tag}_df"]
    E = GOLD[f"{tag}_u"].size // tb.nc
    Jp = J.reshape(E, -1)
    f, g, u = GOLD[f"{tag}_f"], GOLD[f"{tag}_g"], GOLD[f"{tag}_u"]
    assert rel_err(otri.bwdtrans(tb, u), GOLD[f"{tag}_bwd"]) < 1e-13
    assert rel_err(otri.iproduct(tb, Jp, f), GOLD[f"{tag}_iprod"]) < 1e-13
    assert rel_err(np.stack(otri.physderiv(tb, df, f)).reshape(2, -1), GOLD[f"{tag}_deriv"]) < 1e-13
    assert rel_err(otri.iproduct_deriv(tb, Jp, df, [f, g]), GOLD[f"{tag}_iprd"]) < 1e-13
    assert rel_err(otri.helmholtz(tb, Jp, df, 1.3, u), GOLD[f"{tag}_helm"]) < 1e-13


def test_geometry_straight_equals_affine():
    c = tri_case(3, 2, 5, curve=0.0)
    J, df = otri.geom_factors(c.basis, c.X)
    Jr, dfr = otri.straight_tri_geometry(c.mesh.V[c.mesh.EV])
    assert rel_err(J.reshape(c.E, -1), np.repeat(Jr[:, None], c.nq, 1)) < 1e-12
    assert rel_err(df.reshape(4, c.E, -1), np.repeat(dfr[:, :, None], c.nq, 2)) < 1e-12
    # area of the unit square
    assert abs(np.sum(J.reshape(c.E, -1) * np.outer(c.basis.w1h, c.basis.w0).reshape(1, -1)) - 1.0) < 1e-13


@pytest.mark.parametrize("n", [3, 4, 7])
def test_assembly_is_conforming(n):
    """A global vector expands to the same values on both sides of every shared edge
    (signed edge modes, collapsed top vertex), with rotated local vertex orders."""
    c = tri_case(3, 3, n)
    amap = c.mesh.assembly(n)
    x = np.random.default_rng(2).uniform(-1, 1, amap.nglobal)
    loc = (amap.sign * x[amap.l2g]).reshape(c.E, -1)
    EV = c.mesh.EV
    s = np.linspace(-0.9, 0.9, 7)
    edges = {}
    for e in range(c.E):
        for ed, (a, b) in enumerate(((0, 1), (1, 2), (0, 2))):
            va, vb = EV[e, a], EV[e, b]
            edges.setdefault((min(va, vb), max(va, vb)), []).append((e, ed, va < vb))
    checked = 0
    for key, occ in edges.items():
        vals = []
        for e, ed, fwd in occ:
            t = s if fwd else -s
            eta = [(t, -np.ones_like(t)), (np.ones_like(t), t), (-np.ones_like(t), t)][ed]
            vals.append(otri.modal_values(n, *eta) @ loc[e])
        if len(vals) == 2:
            assert np.abs(vals[0] - vals[1]).max() < 1e-12, key
            checked += 1
    assert checked > 0


def _oracle_solve(c, amap, lam, rhs, tol):
    m = osolve.Map.of(amap)
    J = c.jac.reshape(c.E, -1) if c.deformed else c.jac

    def apply(v):
        vv = v.copy()
        vv[:m.ndir] = 0
        return m.assemble(otri.helmholtz(c.basis, J, c.df, lam, m.gather(vv)))
    d = np.zeros(m.nglobal)
    np.add.at(d, m.l2g, otri.helmholtz_diag(c.basis, c.E, J, c.df, lam).reshape(-1))
    return osolve.cg(apply, 1.0 / d[m.ndir:], rhs, m.ndir, tol)


def _manufactured(c, amap, lam):
    u = (np.sin(np.pi * c.X[0]) * np.sin(np.pi * c.X[1])).reshape(-1)
    f = -(lam + 2 * np.pi ** 2) * u
    J = c.jac.reshape(c.E, -1) if c.deformed else c.jac
    m = osolve.Map.of(amap)
    rhs = -m.assemble(otri.iproduct(c.basis, J, f))
    return u, f, rhs


def test_oracle_manufactured_solution_converges():
    """sin(pi x) sin(pi y) with homogeneous Dirichlet data: the error falls spectrally."""
    errs = []
    for n in (4, 6, 8):
        c = tri_case(3, 3, n)
        amap = c.mesh.assembly(n)
        u, f, rhs = _manufactured(c, amap, 1.0)
        x, it, _, _ = _oracle_solve(c, amap, 1.0, rhs, 1e-12)
        uh = otri.bwdtrans(c.basis, osolve.Map.of(amap).gather(x))
        errs.append(np.abs(uh.reshape(-1) - u).max())
    assert errs[0] < 1e-2 and errs[1] < errs[0] / 20 and errs[2] < errs[1] / 20, errs


# ---------------------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def ctx():
    from ithaca_gpu.operators import Context
    c = Context(0)
    yield c
    c.close()


def _coll(ctx, c, precision="fp64"):
    from ithaca_gpu.operators import Collection
    return Collection(ctx, "tri", c.n, c.Q, c.E, c.jac, c.df, deformed=c.deformed, precision=precision)


CASES = [(n, True) for n in range(2, 13)] + [(4, False), (7, False), (10, False), (12, False)]


@pytest.mark.gpu
@pytest.mark.parametrize("n,deformed", CASES)
def test_gpu_operators_match_oracle(ctx, n, deformed):
    c = tri_case(3, 2, n, deformed=deformed)
    J = c.jac.reshape(c.E, -1) if deformed else c.jac
    rng = np.random.default_rng(n)
    u = rng.uniform(-1, 1, c.E * c.nm)
    f = rng.uniform(-1, 1, c.E * c.nq)
    g = rng.uniform(-1, 1, c.E * c.nq)
    for prec, tol in (("fp64", TOL64), ("fp32", TOL32)):
        coll = _coll(ctx, c, prec)
        dt = np.float64 if prec == "fp64" else np.float32
        uu, ff, gg = u.astype(dt), f.astype(dt), g.astype(dt)
        assert coll.Ndof() == c.E * c.nm
        assert rel_err(coll.bwdtrans(uu), otri.bwdtrans(c.basis, u)) < tol
        assert rel_err(coll.iproduct(ff), otri.iproduct(c.basis, J, f)) < tol
        d0, d1 = coll.physderiv(ff)
        r0, r1 = otri.physderiv(c.basis, c.df, f)
        assert max(rel_err(d0, r0), rel_err(d1, r1)) < tol
        assert rel_err(coll.iproduct_deriv([ff, gg]), otri.iproduct_deriv(c.basis, J, c.df, [f, g])) < tol
        for lam in (0.0, 1.0, 10.0):
            assert rel_err(coll.helmholtz(lam, uu), otri.helmholtz(c.basis, J, c.df, lam, u)) < tol, (prec, lam)
        if prec == "fp64":
            assert rel_err(coll.helmholtz_diag(2.0), otri.helmholtz_diag(c.basis, c.E, J, c.df, 2.0)) < tol
        coll.close()


@pytest.mark.gpu
def test_gpu_reference_fixtures(ctx):
    """The GPU against the reference's own kernels directly."""
    from ithaca_gpu.operators import Collection
    E = 10
    coll = Collection(ctx, "tri", 4, 5, E, GOLD["unit_helm_jac"], GOLD["unit_helm_df"], deformed=False)
    out = coll.helmholtz(float(GOLD["unit_helm_lambda"]), np.ones(E * 10))
    assert rel_err(out, GOLD["unit_helm_out"]) < TOL64
    for tag, deformed in (("mesh", True), ("reg", False)):
        n = int(GOLD[f"{tag}_n"])
        E = GOLD[f"{tag}_u"].size // (n * (n + 1) // 2)
        coll = Collection(ctx, "tri", n, n + 1, E, GOLD[f"{tag}_jac"], GOLD[f"{tag}_df"], deformed=deformed)
        f, g, u = GOLD[f"{tag}_f"], GOLD[f"{tag}_g"], GOLD[f"{tag}_u"]
        assert rel_err(coll.bwdtrans(u), GOLD[f"{tag}_bwd"]) < TOL64
        assert rel_err(coll.iproduct(f), GOLD[f"{tag}_iprod"]) < TOL64
        assert rel_err(np.stack(coll.physderiv(f)), GOLD[f"{tag}_deriv"]) < TOL64
        assert rel_err(coll.iproduct_deriv([f, g]), GOLD[f"{tag}_iprd"]) < TOL64
        assert rel_err(coll.helmholtz(1.3, u), GOLD[f"{tag}_helm"]) < TOL64


@pytest.mark.gpu
def test_gpu_geometry(ctx):
    from ithaca_gpu.operators import geom_factors
    c = tri_case(4, 3, 6)
    jac, df = geom_factors(ctx, "tri", c.Q, c.X)
    assert rel_err(jac, c.jac) < 1e-12
    assert rel_err(df, c.df) < 1e-12
    bad = c.X.copy()
    bad[0, 0] = bad[0, 0][::-1].copy()  # a folded element
    with pytest.raises(Exception):
        geom_factors(ctx, "tri", c.Q, bad)


@pytest.mark.gpu
@pytest.mark.parametrize("n,deformed", [(3, True), (6, True), (9, True), (5, False)])
def test_gpu_cg_matches_oracle(ctx, n, deformed):
    from ithaca_gpu.operators import GlobalLinSysIterativeFullGPU
    c = tri_case(4, 3, n, deformed=deformed)
    amap = c.mesh.assembly(n)
    coll = _coll(ctx, c)
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    rhs = np.random.default_rng(7).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    x, res = sysg.solve(1.5, rhs, tol=1e-12)
    xo, it_o, _, _ = _oracle_solve(c, amap, 1.5, rhs, 1e-12)
    assert abs(res.iterations - it_o) <= max(2, it_o // 50), (res.iterations, it_o)
    assert rel_err(x[amap.ndir:], xo[amap.ndir:]) < 1e-10
    xm, rm = sysg.solve(1.5, rhs, tol=1e-10, mode="mixed")
    assert rm.rel_residual < 1e-10
    assert rel_err(xm[amap.ndir:], xo[amap.ndir:]) < 1e-7
    sysg.close()
    coll.close()


@pytest.mark.gpu
def test_gpu_helmsolve_manufactured(ctx):
    """HelmSolve on curved triangles: GPU = oracle, and close to the exact solution."""
    from ithaca_gpu.operators import GlobalLinSysIterativeFullGPU, GlobalLinSysIterativeStaticCondGPU
    n = 7
    c = tri_case(4, 4, n)
    amap = c.mesh.assembly(n)
    u, f, rhs = _manufactured(c, amap, 1.0)
    coll = _coll(ctx, c)
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    loc, res = sysg.helmsolve(1.0, f, tol=1e-12)
    xo, _, _, _ = _oracle_solve(c, amap, 1.0, rhs, 1e-12)
    lo = osolve.Map.of(amap).gather(xo)
    assert rel_err(loc, lo) < 1e-10
    uh = coll.bwdtrans(loc)
    assert np.abs(uh - u).max() < 1e-4  # P = 6 on 32 curved triangles
    sc = GlobalLinSysIterativeStaticCondGPU(coll, amap)
    info = sc.info()
    assert info["nint_local"] == (n - 2) * (n - 3) // 2  # interior modes per element
    loc_sc, res_sc = sc.helmsolve(1.0, f, tol=1e-12)
    assert rel_err(loc_sc, lo) < 1e-9
    assert res_sc.iterations < res.iterations
    sc.close()
    sysg.close()
    coll.close()


@pytest.mark.gpu
def test_gpu_varcoeff(ctx):
    """An isotropic coefficient kappa(x) per point on deformed triangles."""
    from ithaca_gpu.operators import GlobalLinSysIterativeFullGPU
    n = 5
    c = tri_case(3, 3, n)
    amap = c.mesh.assembly(n)
    coll = _coll(ctx, c)
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    kappa = 1.0 + 0.5 * np.sin(3 * c.X[0]) * np.cos(2 * c.X[1])
    sysg.set_varcoeff(kappa.reshape(-1))
    x = np.random.default_rng(3).uniform(-1, 1, amap.nglobal)
    x[:amap.ndir] = 0
    m = osolve.Map.of(amap)
    ref = m.assemble(otri.helmholtz(c.basis, c.jac.reshape(c.E, -1), c.df, 0.7, m.gather(x), kappa=kappa))
    y = sysg.apply(0.7, x)
    assert rel_err(y[amap.ndir:], ref[amap.ndir:]) < 1e-12
    with pytest.raises(Exception):
        sysg.set_varcoeff_tensor(np.ones((3, c.E * c.nq)))
    sysg.close()
    coll.close()
