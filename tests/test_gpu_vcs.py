"""The ROM incompressible solver's HelmSolve callers on the GPU
(VelocityCorrectionScheme_ROM::v_SolveViscous / v_SolvePressure,
solvers/IncNavierStokesSolver/EquationSystems/VelocityCorrectionScheme_ROM.cpp:1522-1567)
against the oracle's restatement: per-field lambda = 1 / (aii_dt diff_coeff), Dirichlet
lift, BwdTrans of every field, lambda = 0 for the pressure."""
import numpy as np
import pytest

from cases import hex_case, quad_case, rel_err
from oracle import solve as osolve

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from ithaca_gpu.operators import Context
    c = Context(0)
    yield c
    c.close()


def _system(ctx, c, amap=None):
    from ithaca_gpu.operators import Collection, GlobalLinSysIterativeFullGPU
    coll = Collection(ctx, c.shape, c.n, c.Q, c.E, c.jac, c.df, deformed=c.deformed)
    amap = amap if amap is not None else c.mesh.assembly(c.n)
    return coll, amap, GlobalLinSysIterativeFullGPU(coll, amap)


def _fields(c, amap, seed):
    rng = np.random.default_rng(seed)
    X = c.X.reshape(c.dim, -1)
    f0 = np.sin(np.pi * X[0]) * np.cos(np.pi * X[1])
    f1 = np.cos(2 * X[0]) * X[1] ** 2 + 0.3
    d0 = rng.uniform(-1, 1, amap.ndir)
    return [np.ascontiguousarray(f0), np.ascontiguousarray(f1)], [d0, None]


@pytest.mark.parametrize("on_device", [False, True])
def test_solve_viscous_matches_oracle(ctx, on_device):
    from ithaca_gpu.vcs import VelocityCorrectionGPU
    c = quad_case(6, 5, 7)
    coll, amap, sys_ = _system(ctx, c)
    forcing, dirichlet = _fields(c, amap, 4)
    diff, aii_dt = [0.01, 0.025], 0.1
    jac = c.jac.reshape(c.E, -1)
    co, ph, its = osolve.solve_viscous(c.basis, 2, jac, c.df, amap, forcing, aii_dt, diff, dirichlet, tol=1e-12)
    vcs = VelocityCorrectionGPU(sys_, diff)
    if on_device:
        import torch
        fd = [torch.from_numpy(f).cuda() for f in forcing]
        dd = [torch.from_numpy(dirichlet[0]).cuda(), None]
        coeffs, phys, res = vcs.solve_viscous(fd, aii_dt, dirichlet=dd, tol=1e-12)
        coeffs = [x.cpu().numpy() for x in coeffs]
        phys = [x.cpu().numpy() for x in phys]
    else:
        coeffs, phys, res = vcs.solve_viscous(forcing, aii_dt, dirichlet=dirichlet, tol=1e-12)
    for i in range(2):
        assert rel_err(coeffs[i], co[i]) < 1e-10, i
        assert rel_err(phys[i], ph[i]) < 1e-10, i
        # to 1e-12 the residual is near the FP64 floor of this mass-dominated system
        # (lambda = 400, 1000), and the reduction order moves the count by a few
        assert abs(res[i].iterations - its[i]) <= 3, (res[i].iterations, its[i])
        assert res[i].rel_residual < 1e-11
    # the Dirichlet data of field 0 are its boundary coefficients; field 1 is homogeneous
    first = {}
    for l, g in enumerate(amap.l2g):
        first.setdefault(g, l)
    for g in range(amap.ndir):
        assert abs(coeffs[0][first[g]] * amap.sign[first[g]] - dirichlet[0][g]) < 1e-13
        assert coeffs[1][first[g]] == 0.0


def test_solve_viscous_curved_hex_mixed(ctx):
    """One field on curved hexes in mixed precision: the same answer to the FP64 tolerance."""
    from ithaca_gpu.vcs import VelocityCorrectionGPU
    c = hex_case(3, 2, 2, 5)
    coll, amap, sys_ = _system(ctx, c)
    f = np.ascontiguousarray(np.sin(np.pi * c.X[0]).reshape(-1))
    co, ph, _ = osolve.solve_viscous(c.basis, 3, c.jac.reshape(c.E, -1), c.df, amap, [f], 0.05, [0.5], tol=1e-12)
    coeffs, phys, res = VelocityCorrectionGPU(sys_, [0.5]).solve_viscous([f], 0.05, tol=1e-11, mode="mixed")
    assert res[0].rel_residual < 1e-11
    assert rel_err(coeffs[0], co[0]) < 1e-9
    assert rel_err(phys[0], ph[0]) < 1e-9


def test_solve_pressure_matches_oracle(ctx):
    from ithaca_gpu.vcs import VelocityCorrectionGPU
    cv = quad_case(6, 5, 7)
    cp = quad_case(6, 5, 6)  # the pressure expansion one order lower, same mesh
    _, amap_v, sys_v = _system(ctx, cv)
    _, amap_p, sys_p = _system(ctx, cp)
    X = cp.X.reshape(2, -1)
    f = np.ascontiguousarray(np.exp(X[0]) * np.sin(3 * X[1]))
    d = np.random.default_rng(8).uniform(-1, 1, amap_p.ndir)
    po, it_o = osolve.solve_pressure(cp.basis, 2, cp.jac.reshape(cp.E, -1), cp.df, amap_p, f, d, tol=1e-12)
    vcs = VelocityCorrectionGPU(sys_v, [0.01, 0.01], pressure=sys_p)
    out, res = vcs.solve_pressure(f, dirichlet=d, tol=1e-12)
    assert rel_err(out, po) < 1e-10
    assert abs(res.iterations - it_o) <= 1, (res.iterations, it_o)


def test_vcs_argument_errors_leave_context_usable(ctx):
    from ithaca_gpu._capi import ERR_ARG, GpuError
    from ithaca_gpu.mesh import AssemblyMap
    from ithaca_gpu.vcs import VelocityCorrectionGPU
    c = quad_case(4, 4, 5)
    coll, amap, sys_ = _system(ctx, c)
    f = np.ascontiguousarray(np.ones(c.E * c.nq))
    with pytest.raises(GpuError) as ei:
        VelocityCorrectionGPU(sys_, [0.0]).solve_viscous([f], 0.1)
    assert ei.value.code == ERR_ARG
    with pytest.raises(GpuError) as ei:
        VelocityCorrectionGPU(sys_, [1.0]).solve_viscous([f], -1.0)
    assert ei.value.code == ERR_ARG
    # a pressure system without Dirichlet dofs is singular: rejected before any work
    free = AssemblyMap(amap.l2g, amap.sign, amap.nglobal, 0)
    _, _, sys_free = _system(ctx, c, free)
    with pytest.raises(GpuError) as ei:
        VelocityCorrectionGPU(sys_, [1.0], pressure=sys_free).solve_pressure(f)
    assert ei.value.code == ERR_ARG
    coeffs, phys, res = VelocityCorrectionGPU(sys_, [1.0]).solve_viscous([f], 0.1, tol=1e-10)
    assert res[0].rel_residual < 1e-10
