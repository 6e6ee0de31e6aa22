"""GPU global system + CG vs the oracle's restatement of the reference recurrence.

FP64 mode must reproduce the reference iteration count (within one iteration: the
reductions are summed in a different order) and the solution to 1e-10 relative;
the mixed mode must reach the requested FP64 relative residual.
"""
import os

import numpy as np
import pytest

from cases import hex_case, quad_case, rel_err
from oracle import ops as oops
from oracle import solve as osolve

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ctx():
    from ithaca_gpu.operators import Context
    c = Context(0)
    yield c
    c.close()


def _system(ctx, c):
    from ithaca_gpu.operators import Collection, GlobalLinSysIterativeFullGPU
    coll = Collection(ctx, c.shape, c.n, c.Q, c.E, c.jac, c.df, deformed=c.deformed)
    amap = c.mesh.assembly(c.n)
    return coll, amap, GlobalLinSysIterativeFullGPU(coll, amap)


def _forcing(c):
    f = np.sin(np.pi * c.X[0]) * np.sin(np.pi * c.X[1])
    if c.dim == 3:
        f = f * np.sin(np.pi * c.X[2])
    return f.reshape(-1)


def test_golden_reference_cg(ctx):
    """The reference CG recurrence on tests/golden/cg_quad.npz (4x4 quads, 5 modes)."""
    from ithaca_gpu.operators import Collection, GlobalLinSysIterativeFullGPU
    from ithaca_gpu.mesh import AssemblyMap
    g = np.load(os.path.join(G, "cg_quad.npz"))
    n, Q = 5, 6
    E = g["l2g"].size // (n * n)
    coll = Collection(ctx, "quad", n, Q, E, g["jac"], g["df"])
    amap = AssemblyMap(g["l2g"], g["sign"], int(g["nglobal"]), int(g["ndir"]))
    sys_ = GlobalLinSysIterativeFullGPU(coll, amap)
    diag = sys_.diagonal(1.0)
    assert rel_err(1.0 / diag, g["dinv"]) < 1e-12
    x, res = sys_.solve(1.0, g["rhs"], tol=1e-12)
    assert abs(res.iterations - int(g["iterations"])) <= 1
    assert rel_err(x[amap.ndir:], g["x"][amap.ndir:]) < 1e-10


@pytest.mark.parametrize("kind", ["quad_p6", "quad_rot_p4", "hex_p4", "quad_regular_p6"])
def test_fp64_cg_matches_oracle(ctx, kind):
    if kind == "quad_p6":
        c = quad_case(6, 5, 7)
    elif kind == "quad_rot_p4":
        c = quad_case(5, 4, 5, rotate=np.random.default_rng(9).integers(0, 4, 20))
    elif kind == "quad_regular_p6":
        c = quad_case(4, 4, 7, jitter=0.0, deformed=False)
    else:
        c = hex_case(3, 2, 2, 5)
    coll, amap, sys_ = _system(ctx, c)
    lam = 1.0
    rhs = -osolve.Map.of(amap).assemble(oops.iproduct(c.basis, c.dim, c.jac.reshape(c.E, -1), _forcing(c)))
    # global operator
    xr = np.random.default_rng(3).uniform(-1, 1, amap.nglobal)
    y = sys_.apply(lam, xr)
    yo = osolve.global_apply(c.basis, c.dim, c.jac.reshape(c.E, -1), c.df, lam, amap, xr, zero_dir=False)
    assert rel_err(y, yo) < 1e-12
    x, res = sys_.solve(lam, rhs, tol=1e-11)
    xo, it_o, _, _ = osolve.solve(c.basis, c.dim, c.jac.reshape(c.E, -1), c.df, lam, amap, rhs, tol=1e-11)
    assert abs(res.iterations - it_o) <= 1, (res.iterations, it_o)
    assert rel_err(x[amap.ndir:], xo[amap.ndir:]) < 1e-9
    assert res.rel_residual < 1e-10


@pytest.mark.parametrize("lam", [0.1, 1.0, 10.0])
def test_mixed_reaches_fp64_residual(ctx, lam):
    c = quad_case(8, 8, 7)
    coll, amap, sys_ = _system(ctx, c)
    rhs = -osolve.Map.of(amap).assemble(oops.iproduct(c.basis, 2, c.jac.reshape(c.E, -1), _forcing(c)))
    x, res = sys_.solve(lam, rhs, tol=1e-10, mode="mixed")
    assert res.rel_residual < 1e-10
    assert res.outer_iterations >= 1
    xo, _, _, _ = osolve.solve(c.basis, 2, c.jac.reshape(c.E, -1), c.df, lam, amap, rhs, tol=1e-13)
    assert rel_err(x[amap.ndir:], xo[amap.ndir:]) < 1e-8


@pytest.mark.parametrize("inner_tol", [1e-1, 1e-2, 1e-4])
def test_mixed_curved_hex_inner_tolerances(ctx, inner_tol):
    """Mixed refinement on a curved hex mesh for loose and tight inner tolerances: the
    FP64 residual is reached and the solution agrees with the FP64 solve."""
    c = hex_case(4, 4, 3, 5)
    coll, amap, sys_ = _system(ctx, c)
    rhs = np.random.default_rng(5).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    x64, r64 = sys_.solve(1.0, rhs, tol=1e-12)
    x, res = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed", inner_tol=inner_tol)
    assert res.rel_residual < 1e-10
    assert rel_err(x[amap.ndir:], x64[amap.ndir:]) < 1e-8


@pytest.mark.parametrize("variant", [4, 21, 31, 41, 42, 43, 44])
def test_mixed_kernel_variants_curved_hex(ctx, variant):
    """Mixed solves with each FP32 hex kernel; the pipelined ones (21-42) also assemble
    the single-entry rows inside the element kernel. All reach the FP64 residual, agree
    with the FP64 solve and need the same number of inner iterations within a few (only
    the summation order of s.w differs)."""
    c = hex_case(4, 3, 3, 6, amp=0.08)
    coll, amap, sys_ = _system(ctx, c)
    rhs = np.random.default_rng(19).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    x64, _ = sys_.solve(1.0, rhs, tol=1e-12)
    coll.set_variant(4)
    _, ref = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed")
    coll.set_variant(variant)
    x, res = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed")
    assert res.rel_residual < 1e-10
    assert rel_err(x[amap.ndir:], x64[amap.ndir:]) < 1e-8
    assert abs(res.iterations - ref.iterations) <= 4, (res.iterations, ref.iterations)


@pytest.mark.parametrize("variant", [43, 44, 46, 47])
def test_mixed_vector_pencils_q8(ctx, variant):
    """The vector-pencil kernels (Q = 8) inside the mixed solver against their scalar-pencil
    counterparts (42, 41): the same inner iterations within one and the same solution where
    the arithmetic is shared (43, 44); within 10% of the inner iterations summed over the
    refinement steps with the tensor-core stages (46) or the even-odd operators (47), whose
    rounding differs (the count over five loosely converged inner solves moves with it)."""
    c = hex_case(3, 3, 2, 7, amp=0.08)
    coll, amap, sys_ = _system(ctx, c)
    rhs = np.random.default_rng(29).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    coll.set_variant(41 if variant == 44 else 42)
    xr, ref = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed")
    coll.set_variant(variant)
    x, res = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed")
    assert res.rel_residual < 1e-10
    slack = max(4, ref.iterations // 10) if variant in (46, 47) else 1
    assert abs(res.iterations - ref.iterations) <= slack, (res.iterations, ref.iterations)
    assert rel_err(x[amap.ndir:], xr[amap.ndir:]) < 1e-9


@pytest.mark.parametrize("variant", [1, 2])
def test_fp64_cg_even_odd_kernel(ctx, variant):
    """FP64 and mixed solves with the FP64 even-odd pencil kernel (P = 6) against the same
    solves with the shared-memory kernel: the same iterations within 1%, the same solution;
    the variant set after a solve reaches the captured iteration graphs."""
    c = hex_case(4, 3, 3, 7, amp=0.08)
    coll, amap, sys_ = _system(ctx, c)
    rhs = np.random.default_rng(31).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    x0, r0 = sys_.solve(1.0, rhs, tol=1e-12)
    coll.set_variant64(variant)
    x1, r1 = sys_.solve(1.0, rhs, tol=1e-12)
    # about 1300 iterations to 1e-12: the count moves by a few with the rounding order
    assert abs(r1.iterations - r0.iterations) <= max(2, r0.iterations // 100), (r1.iterations, r0.iterations)
    assert rel_err(x1[amap.ndir:], x0[amap.ndir:]) < 1e-10
    x2, r2 = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed")
    assert r2.rel_residual < 1e-10
    assert rel_err(x2[amap.ndir:], x0[amap.ndir:]) < 1e-8
    coll.set_variant64(0)


def _merged_map(amap):
    """The map with a few free global dofs merged: three interior vertices into one row
    of 24 local entries (longer than the ELL classes), a face dof into an edge dof (6
    entries). Any map whose every global dof has a local entry assembles an SPD system."""
    from ithaca_gpu.mesh import AssemblyMap
    l2g = amap.l2g.astype(np.int64).copy()
    cnt = np.bincount(l2g, minlength=amap.nglobal)
    free = np.arange(amap.ndir, amap.nglobal)
    v8, k4, k2 = free[cnt[free] == 8], free[cnt[free] == 4], free[cnt[free] == 2]
    l2g[np.isin(l2g, v8[1:3])] = v8[0]
    l2g[l2g == k2[0]] = k4[0]
    ids = np.unique(l2g)
    l2g = np.searchsorted(ids, l2g)
    return AssemblyMap(l2g, amap.sign, ids.size, amap.ndir)


@pytest.mark.parametrize("variant", [4, 41, 42, 43])
def test_mixed_long_rows(ctx, variant):
    """Rows of 1, 2, 4, 6, 8 and 24 local entries: the FP64 solve against the oracle, and
    the mixed solve with the element-ordered (4) and the scattered (41, 42: owned rows
    and assembly-ordered slots) output of the inner apply."""
    from ithaca_gpu.operators import Collection, GlobalLinSysIterativeFullGPU
    c = hex_case(4, 3, 3, 4, amp=0.08)
    amap = _merged_map(c.mesh.assembly(c.n))
    counts = np.bincount(amap.l2g, minlength=amap.nglobal)
    assert counts.max() == 24 and 6 in counts
    coll = Collection(ctx, c.shape, c.n, c.Q, c.E, c.jac, c.df, deformed=c.deformed)
    sys_ = GlobalLinSysIterativeFullGPU(coll, amap)
    rhs = np.random.default_rng(23).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    x64, res64 = sys_.solve(1.0, rhs, tol=1e-12)
    xo, it_o, _, _ = osolve.solve(c.basis, 3, c.jac.reshape(c.E, -1), c.df, 1.0, amap, rhs, tol=1e-12)
    assert abs(res64.iterations - it_o) <= 1, (res64.iterations, it_o)
    assert rel_err(x64[amap.ndir:], xo[amap.ndir:]) < 1e-9
    coll.set_variant(variant)
    x, res = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed")
    assert res.rel_residual < 1e-10
    assert rel_err(x[amap.ndir:], xo[amap.ndir:]) < 1e-8


@pytest.mark.parametrize("inner_tol", [1e-2, 1e-4])
def test_mixed_geo16_curved_hex(ctx, inner_tol):
    """FP32 inner solves on 16-bit (per-element scaled) geometry inside FP64 refinement:
    the FP64 residual is reached and the solution agrees with the FP64 solve."""
    c = hex_case(4, 3, 3, 6, amp=0.08)
    coll, amap, sys_ = _system(ctx, c)
    rhs = np.random.default_rng(9).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    x64, _ = sys_.solve(1.0, rhs, tol=1e-12)
    x, res = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed_geo16", inner_tol=inner_tol)
    assert res.rel_residual < 1e-10
    assert res.outer_iterations >= 2
    assert rel_err(x[amap.ndir:], x64[amap.ndir:]) < 1e-8
    # the FP32-geometry mixed solve afterwards is unaffected (graph re-captured)
    x2, res2 = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed", inner_tol=inner_tol)
    assert res2.rel_residual < 1e-10
    ms, nbytes = sys_.profile_apply(1.0, mode="mixed_geo16", reps=2)
    assert ms > 0 and nbytes > 0


@pytest.mark.parametrize("variant", [43, 47])
def test_mixed_geo16_vector_pencils_q8(ctx, variant):
    """Half-precision geometry under the vector-pencil kernels (Q = 8, two elements per
    group; 27 elements, so the last group holds one): the FP64 residual is reached, the
    solution equals the FP64 solve's, and the inner iterations match the packed-pair
    half-geometry kernel's (within one for 43, whose arithmetic is the same; within 10%
    for the even-odd operators of 47, whose rounding differs)."""
    c = hex_case(3, 3, 3, 7, amp=0.08)
    coll, amap, sys_ = _system(ctx, c)
    rhs = np.random.default_rng(31).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    x64, _ = sys_.solve(1.0, rhs, tol=1e-12)
    coll.set_variant(42)
    xr, ref = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed_geo16")
    coll.set_variant(variant)
    x, res = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed_geo16")
    assert res.rel_residual < 1e-10
    assert rel_err(x[amap.ndir:], x64[amap.ndir:]) < 1e-8
    slack = max(4, ref.iterations // 10) if variant == 47 else 1
    assert abs(res.iterations - ref.iterations) <= slack, (res.iterations, ref.iterations)
    if variant == 43:
        assert rel_err(x[amap.ndir:], xr[amap.ndir:]) < 1e-9
    ms, nbytes = sys_.profile_apply(1.0, mode="mixed_geo16", reps=2)
    assert ms > 0 and nbytes > 0


@pytest.mark.parametrize("variant,mode", [(42, "mixed"), (43, "mixed"), (47, "mixed"), (47, "mixed_geo16"),
                                          (4, "mixed")])
def test_mixed_fused_update_matches_separate(ctx, variant, mode):
    """The inner FP32 iterations with the assembly fused into the vector update (two
    launches per iteration, the scalars computed by every CTA of the update) against the
    separate assembly and update: the same FP64 residual, inner iterations within a few
    (the partial sums are grouped differently) and the same solution. Variant 4 writes no
    scattered output, so its solve falls back to the separate kernels."""
    c = hex_case(3, 3, 3, 7, amp=0.08)
    coll, amap, sys_ = _system(ctx, c)
    rhs = np.random.default_rng(37).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    x64, _ = sys_.solve(1.0, rhs, tol=1e-12)
    coll.set_variant(variant)
    sys_.set_fused_update(0)
    xs, rs = sys_.solve(1.0, rhs, tol=1e-10, mode=mode)
    sys_.set_fused_update(1)
    xf, rf = sys_.solve(1.0, rhs, tol=1e-10, mode=mode)
    assert rs.rel_residual < 1e-10 and rf.rel_residual < 1e-10
    assert abs(rf.iterations - rs.iterations) <= max(3, rs.iterations // 50), (rf.iterations, rs.iterations)
    assert rel_err(xf[amap.ndir:], x64[amap.ndir:]) < 1e-8
    assert rel_err(xf[amap.ndir:], xs[amap.ndir:]) < 1e-8
    # again after the graph of the other form was captured: the same solve as the first fused one
    xf2, rf2 = sys_.solve(1.0, rhs, tol=1e-10, mode=mode)
    assert rf2.iterations == rf.iterations and rel_err(xf2, xf) == 0.0


def test_mixed_fused_update_long_rows_and_max_iter(ctx):
    """Fused iterations on a mesh whose rows reach 24 local entries (the tail class read
    through its slot ranges), and a max_iter that stops the fused recurrence: NOT_CONVERGED,
    then a normal solve on the same system."""
    from ithaca_gpu._capi import ERR_NOT_CONVERGED, GpuError
    c = hex_case(3, 3, 3, 7, amp=0.08)
    amap = _merged_map(c.mesh.assembly(c.n))
    from ithaca_gpu.operators import Collection, GlobalLinSysIterativeFullGPU
    coll = Collection(ctx, c.shape, c.n, c.Q, c.E, c.jac, c.df, deformed=c.deformed)
    sys_ = GlobalLinSysIterativeFullGPU(coll, amap)
    rhs = np.random.default_rng(41).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    coll.set_variant(47)
    sys_.set_fused_update(1)
    xo, it_o, _, _ = osolve.solve(c.basis, 3, c.jac.reshape(c.E, -1), c.df, 1.0, amap, rhs, tol=1e-12)
    x, res = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed")
    assert res.rel_residual < 1e-10
    assert rel_err(x[amap.ndir:], xo[amap.ndir:]) < 1e-8
    with pytest.raises(GpuError) as ei:
        sys_.solve(1.0, rhs, tol=1e-10, mode="mixed", max_iter=7)
    assert ei.value.code == ERR_NOT_CONVERGED
    x2, res2 = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed")
    assert res2.iterations == res.iterations and rel_err(x2, x) == 0.0


def test_mixed_geo16_rejects_quads(ctx):
    from ithaca_gpu._capi import ERR_UNSUPPORTED, GpuError
    c = quad_case(4, 4, 5)
    coll, amap, sys_ = _system(ctx, c)
    rhs = np.random.default_rng(2).uniform(-1, 1, amap.nglobal)
    with pytest.raises(GpuError) as ei:
        sys_.solve(1.0, rhs, tol=1e-10, mode="mixed_geo16")
    assert ei.value.code == ERR_UNSUPPORTED
    x, res = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed")
    assert res.rel_residual < 1e-10


def test_helmsolve_matches_analytic(ctx):
    c = quad_case(8, 8, 7, jitter=0.1, seed=0)
    coll, amap, sys_ = _system(ctx, c)
    out, res = sys_.helmsolve(1.0, _forcing(c), tol=1e-12)
    phys = oops.bwdtrans(c.basis, 2, out).reshape(-1)
    exact = -_forcing(c) / (2 * np.pi ** 2 + 1.0)
    assert np.max(np.abs(phys - exact)) < 1e-10


def test_deterministic_iterations(ctx):
    c = hex_case(2, 2, 2, 4)
    coll, amap, sys_ = _system(ctx, c)
    rhs = np.random.default_rng(0).uniform(-1, 1, amap.nglobal)
    x1, r1 = sys_.solve(1.0, rhs, tol=1e-12)
    x2, r2 = sys_.solve(1.0, rhs, tol=1e-12)
    assert r1.iterations == r2.iterations
    assert np.array_equal(x1, x2)


def test_max_iter_reports_not_converged(ctx):
    from ithaca_gpu._capi import ERR_NOT_CONVERGED, GpuError
    c = quad_case(4, 4, 5)
    coll, amap, sys_ = _system(ctx, c)
    rhs = np.random.default_rng(1).uniform(-1, 1, amap.nglobal)
    with pytest.raises(GpuError) as ei:
        sys_.solve(1.0, rhs, tol=1e-14, max_iter=3)
    assert ei.value.code == ERR_NOT_CONVERGED
    # the context stays usable
    x, res = sys_.solve(1.0, rhs, tol=1e-10)
    assert res.rel_residual < 1e-9


def test_nan_rhs_reports_numeric(ctx):
    from ithaca_gpu._capi import ERR_NUMERIC, GpuError
    c = quad_case(3, 3, 4)
    coll, amap, sys_ = _system(ctx, c)
    rhs = np.ones(amap.nglobal)
    rhs[amap.ndir + 2] = np.nan
    with pytest.raises(GpuError) as ei:
        sys_.solve(1.0, rhs)
    assert ei.value.code == ERR_NUMERIC
