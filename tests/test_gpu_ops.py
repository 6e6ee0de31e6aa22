"""GPU element operators vs the FP64 oracle (quad + hex, deformed + regular, FP64 + FP32).

Tolerances: FP64 kernels 1e-12 relative (max-norm of the difference over max-norm of
the oracle), as the reference's own collection tests demand 1e-10; FP32 kernels 2e-5.
"""
import numpy as np
import pytest

from cases import hex_case, quad_case, rel_err
from oracle import ops as oops

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-5


@pytest.fixture(scope="module")
def ctx():
    from ithaca_gpu.operators import Context
    c = Context(0)
    yield c
    c.close()


def _coll(ctx, c, precision="fp64"):
    from ithaca_gpu.operators import Collection
    return Collection(ctx, c.shape, c.n, c.Q, c.E, c.jac, c.df, deformed=c.deformed, precision=precision)


QUAD_N = list(range(2, 11))
HEX_N = [2, 3, 4, 5, 7, 9, 10]


def _cases():
    out = []
    for n in QUAD_N:
        out.append(("quad", n, True))
    out += [("quad", 5, False), ("quad", 7, False)]
    for n in HEX_N:
        out.append(("hex", n, True))
    out += [("hex", 5, False), ("hex", 7, False)]
    return out


def _make(shape, n, deformed):
    if shape == "quad":
        return quad_case(5, 3, n, jitter=0.1 if deformed else 0.0, seed=3, deformed=deformed)
    return hex_case(3, 2, 2, n, amp=0.05 if deformed else 0.0, deformed=deformed)


@pytest.mark.parametrize("shape,n,deformed", _cases())
def test_helmholtz_fp64(ctx, shape, n, deformed):
    c = _make(shape, n, deformed)
    coll = _coll(ctx, c)
    rng = np.random.default_rng(1)
    u = rng.uniform(-1, 1, c.E * c.nm)
    for lam in (0.0, 1.0, 10.0):
        out = coll.helmholtz(lam, u)
        ref = oops.helmholtz(c.basis, c.dim, c.jac.reshape(c.E, -1), c.df, lam, u)
        assert rel_err(out, ref) < TOL64, (shape, n, lam)


@pytest.mark.parametrize("shape,n,deformed", _cases())
def test_bwd_iprod_deriv_fp64(ctx, shape, n, deformed):
    c = _make(shape, n, deformed)
    coll = _coll(ctx, c)
    rng = np.random.default_rng(2)
    u = rng.uniform(-1, 1, c.E * c.nm)
    phys = coll.bwdtrans(u)
    assert rel_err(phys, oops.bwdtrans(c.basis, c.dim, u)) < TOL64
    f = rng.uniform(-1, 1, c.E * c.nq)
    ip = coll.iproduct(f)
    assert rel_err(ip, oops.iproduct(c.basis, c.dim, c.jac.reshape(c.E, -1), f)) < TOL64
    ds = coll.physderiv(f)
    refs = oops.physderiv(c.basis, c.dim, c.df, f)
    for d, r in zip(ds, refs):
        assert rel_err(d, r) < TOL64


@pytest.mark.parametrize("shape,n,deformed", _cases())
def test_iproduct_deriv_fp64(ctx, shape, n, deformed):
    """IProductWRTDerivBase against the oracle, and of the physical gradient against the
    Laplacian (lambda = 0 Helmholtz) of the same coefficients."""
    c = _make(shape, n, deformed)
    coll = _coll(ctx, c)
    rng = np.random.default_rng(5)
    comps = [rng.uniform(-1, 1, c.E * c.nq) for _ in range(c.dim)]
    out = coll.iproduct_deriv(comps)
    ref = oops.iproduct_deriv(c.basis, c.dim, c.jac.reshape(c.E, -1), c.df, comps)
    assert rel_err(out, ref) < TOL64
    u = rng.uniform(-1, 1, c.E * c.nm)
    lap = coll.iproduct_deriv(coll.physderiv(coll.bwdtrans(u)))
    assert rel_err(lap, coll.helmholtz(0.0, u)) < TOL64


@pytest.mark.parametrize("shape,n", [("quad", 7), ("hex", 6)])
def test_iproduct_deriv_fp32_and_device(ctx, shape, n):
    torch = pytest.importorskip("torch")
    c = _make(shape, n, True)
    coll = _coll(ctx, c, "fp32")
    rng = np.random.default_rng(6)
    comps = [rng.uniform(-1, 1, c.E * c.nq) for _ in range(c.dim)]
    ref = oops.iproduct_deriv(c.basis, c.dim, c.jac.reshape(c.E, -1), c.df, comps)
    dev = [torch.from_numpy(x.astype(np.float32)).cuda() for x in comps]
    out = coll.iproduct_deriv(dev)
    torch.cuda.synchronize()
    assert rel_err(out.cpu().numpy(), ref) < TOL32


@pytest.mark.parametrize("shape,n,deformed", [("quad", 7, True), ("quad", 9, True), ("hex", 5, True),
                                              ("hex", 7, True), ("hex", 9, True)])
def test_helmholtz_fp32(ctx, shape, n, deformed):
    c = _make(shape, n, deformed)
    coll = _coll(ctx, c, "fp32")
    rng = np.random.default_rng(4)
    u = rng.uniform(-1, 1, c.E * c.nm)
    out = coll.helmholtz(1.0, u.astype(np.float32))
    ref = oops.helmholtz(c.basis, c.dim, c.jac.reshape(c.E, -1), c.df, 1.0, u)
    assert rel_err(out, ref) < TOL32


@pytest.mark.parametrize("shape,n", [("quad", 3), ("quad", 7), ("hex", 3), ("hex", 5)])
def test_helmholtz_diag(ctx, shape, n):
    c = _make(shape, n, True)
    coll = _coll(ctx, c)
    d = coll.helmholtz_diag(2.0)
    ref = oops.helmholtz_diag(c.basis, c.dim, c.jac.reshape(c.E, -1), c.df, 2.0)
    assert rel_err(d, ref) < TOL64
    # and it is the diagonal of the operator the apply uses
    E1 = quad_case(1, 1, n) if shape == "quad" else hex_case(1, 1, 1, n)
    coll1 = _coll(ctx, E1)
    eye = np.eye(E1.nm)
    A = np.stack([coll1.helmholtz(2.0, np.ascontiguousarray(eye[i])) for i in range(E1.nm)], axis=1)
    assert rel_err(coll1.helmholtz_diag(2.0), np.diag(A)) < TOL64


def test_geom_factors_gpu(ctx):
    from ithaca_gpu.operators import geom_factors
    from oracle import geom as ogeom
    for c in (quad_case(4, 3, 6), hex_case(2, 2, 2, 5)):
        jac, df = geom_factors(ctx, c.shape, c.Q, c.X)
        rj, rdf = ogeom.geom_factors(c.X, c.basis.D2, c.dim)
        assert rel_err(jac, rj) < TOL64
        assert rel_err(df, rdf) < TOL64


def test_unsupported_order_raises(ctx):
    from ithaca_gpu._capi import GpuError
    from ithaca_gpu.operators import Collection
    c = quad_case(2, 2, 5)
    with pytest.raises(GpuError):
        Collection(ctx, "quad", 5, 7, c.E, c.jac, c.df)  # npoints != nmodes + 1
    with pytest.raises(GpuError):
        Collection(ctx, "quad", 12, 13, c.E, c.jac, c.df)


@pytest.mark.parametrize("n", [2, 3, 4, 5, 6, 7, 8, 9, 10])
@pytest.mark.parametrize("variant", [0, 2, 4, 21, 22, 31, 32, 41, 42, 43, 44, 46, 47])
def test_hex_fp32_kernel_variants(ctx, n, variant):
    """Every FP32 hex Helmholtz kernel variant (shared-memory; register-pencil with a
    TMA-staged geometry slab, one pass with 2 or 4 elements per CTA or persistent and
    pipelined with 1 or 2 elements per group and one or two geometry buffers) against the
    FP64 oracle; E = 7 leaves a partial last group."""
    c = hex_case(7, 1, 1, n)
    coll = _coll(ctx, c, "fp32")
    coll.set_variant(variant)
    rng = np.random.default_rng(40 + n)
    u = rng.uniform(-1, 1, c.E * c.nm)
    out = coll.helmholtz(0.7, u.astype(np.float32))
    ref = oops.helmholtz(c.basis, 3, c.jac.reshape(c.E, -1), c.df, 0.7, u)
    assert rel_err(out, ref) < TOL32


@pytest.mark.parametrize("n", [3, 6, 7, 9])
def test_hex_pencil_variants_bit_identical(ctx, n):
    """The pencil kernels share one summation order: the single-pass, pipelined
    (one or two geometry buffers) and packed-pair variants give identical bits."""
    c = hex_case(5, 2, 2, n)
    coll = _coll(ctx, c, "fp32")
    u = np.random.default_rng(70 + n).uniform(-1, 1, c.E * c.nm).astype(np.float32)
    outs = {}
    for v in (2, 4, 21, 22, 31, 32, 41, 42, 43, 44):
        coll.set_variant(v)
        outs[v] = coll.helmholtz(0.3, u)
    for v, o in outs.items():
        assert np.array_equal(o, outs[2]), v


def test_hex_tensor_core_and_even_odd_stages_fp32_accuracy(ctx):
    """Variant 46 runs the i and j contractions as TF32 MMAs in three-term split precision,
    variant 47 every 1-D operator in even-odd form: each apply stays within a few FP32
    rounding steps of the FP32-FMA kernel (43) and of the FP64 oracle, on a curved mesh with
    a partial last group."""
    c = hex_case(5, 2, 2, 7)
    coll = _coll(ctx, c, "fp32")
    u = np.random.default_rng(77).uniform(-1, 1, c.E * c.nm)
    ref = oops.helmholtz(c.basis, 3, c.jac.reshape(c.E, -1), c.df, 0.9, u)
    outs = {}
    for v in (43, 46, 47):
        coll.set_variant(v)
        outs[v] = coll.helmholtz(0.9, u.astype(np.float32)).astype(np.float64)
    e43 = rel_err(outs[43], ref)
    for v in (46, 47):  # tensor-core stages; even-odd 1-D operators
        assert rel_err(outs[v], ref) < 4 * max(e43, 1e-7), (v, rel_err(outs[v], ref), e43)
        assert rel_err(outs[v], outs[43]) < 5e-6, v


@pytest.mark.parametrize("n", [3, 4, 5, 7, 9])
@pytest.mark.parametrize("variant", [1, 2])
def test_hex_fp64_even_odd_kernel(ctx, n, variant):
    """The FP64 pipelined kernel with even-odd 1-D operators (Q even; Q odd keeps the
    shared-memory kernel) against the FP64 oracle; E = 7 leaves a partial last group."""
    c = hex_case(7, 1, 1, n)
    coll = _coll(ctx, c, "fp64")
    coll.set_variant64(variant)
    u = np.random.default_rng(90 + n).uniform(-1, 1, c.E * c.nm)
    ref = oops.helmholtz(c.basis, 3, c.jac.reshape(c.E, -1), c.df, 0.7, u)
    assert rel_err(coll.helmholtz(0.7, u), ref) < TOL64


def test_autotune_picks_a_working_variant(ctx):
    c = hex_case(4, 4, 2, 7)
    coll = _coll(ctx, c, "fp32")
    chosen, times = coll.autotune(reps=3)
    assert chosen in (0, 2, 4, 21, 22, 31, 32, 41, 42, 43, 44, 46, 47) and all(t > 0 for t in times.values())
    u = np.random.default_rng(3).uniform(-1, 1, c.E * c.nm)
    out = coll.helmholtz(1.0, u.astype(np.float32))
    ref = oops.helmholtz(c.basis, 3, c.jac.reshape(c.E, -1), c.df, 1.0, u)
    assert rel_err(out, ref) < TOL32
