"""Geometric factors (GeomFactors.cpp:168-475 restated) against closed forms.

Both the oracle's restatement and the GPU kernel (csrc/geom.cu) differentiate the
coordinates held at the quadrature points by collocation, as GeomFactors::ComputeDeriv
does. For a trilinear hexahedron that is exact, so J = det(dx/dxi) and
df[k*3+j] = dxi_j/dx_k must match the closed form of the trilinear map to rounding. For
the benchmark's curved map x_a + 0.05 sin(2 pi x_b) sin(2 pi x_c) (cyclic) on 32^3
elements, the collocation derivative converges spectrally to the analytic one: at
Q >= 8 the difference is at the rounding level (1e-11 relative bound; measured
1e-12..5e-12), at Q = 6 it is interpolation-limited (bound 1e-8; measured 3e-9).
"""
import numpy as np
import pytest

from ithaca_gpu.mesh import HexMesh, gll_points
from oracle import basis as obasis
from oracle import geom as ogeom

TRILINEAR_VERTS = np.array([(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1),
                            (-1, -1, 1), (1, -1, 1), (2, 3, 4), (-1, 1, 1)], float)
CURVED_TOL = {6: 1e-8, 8: 1e-11, 10: 1e-11, 12: 1e-11}


def _factors_from_jacobian(Jm):
    """Jm[..., a, i] = dx_a/dxi_i -> (J, df (9, npts)) in the CoalescedGeomData layout."""
    J = np.linalg.det(Jm)
    inv = np.linalg.inv(Jm)  # inv[..., j, k] = dxi_j / dx_k
    df = np.stack([inv[..., j, k] for k in range(3) for j in range(3)])
    return J.reshape(-1), df.reshape(9, -1)


def trilinear_case(Q):
    z = gll_points(Q)
    a, b = 0.5 * (1 - z), 0.5 * (1 + z)
    da, db = -0.5 * np.ones(Q), 0.5 * np.ones(Q)
    shape = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    f = lambda s: (a, b)[s]
    g = lambda s: (da, db)[s]
    X = np.zeros((3, Q, Q, Q))
    Jm = np.zeros((Q, Q, Q, 3, 3))
    for v, (sx, sy, sz) in enumerate(shape):
        W = np.einsum("k,j,i->kji", f(sz), f(sy), f(sx))
        dW = [np.einsum("k,j,i->kji", f(sz), f(sy), g(sx)), np.einsum("k,j,i->kji", f(sz), g(sy), f(sx)),
              np.einsum("k,j,i->kji", g(sz), f(sy), f(sx))]
        for c in range(3):
            X[c] += W * TRILINEAR_VERTS[v, c]
            for i in range(3):
                Jm[..., c, i] += dW[i] * TRILINEAR_VERTS[v, c]
    J, df = _factors_from_jacobian(Jm)
    return X.reshape(3, 1, Q ** 3), J, df


def curved_case(Q, nel=64, seed=3):
    """A seeded sample of the 32^3 benchmark mesh's elements with the analytic factors
    of the cyclic map composed with the affine element map."""
    mesh = HexMesh(32, 32, 32, curve_amp=0.05)
    eids = np.sort(np.random.default_rng(seed).choice(mesh.E, nel, replace=False))
    X = mesh.coords(Q, eids)
    amp, tp = mesh.curve_amp, 2 * np.pi
    t = 0.5 * (1 + gll_points(Q))
    ix, iy, iz = eids % 32, (eids // 32) % 32, eids // 1024
    x = ((ix[:, None] + t[None, :]) / 32)[:, None, None, :]
    y = ((iy[:, None] + t[None, :]) / 32)[:, None, :, None]
    w = ((iz[:, None] + t[None, :]) / 32)[:, :, None, None]
    x, y, w = np.broadcast_arrays(x, y, w)
    dP = np.zeros(x.shape + (3, 3))  # dPhi_a / dX_b
    dP[..., 0, 0] = dP[..., 1, 1] = dP[..., 2, 2] = 1.0
    dP[..., 0, 1] = amp * tp * np.cos(tp * y) * np.sin(tp * w)
    dP[..., 0, 2] = amp * tp * np.sin(tp * y) * np.cos(tp * w)
    dP[..., 1, 2] = amp * tp * np.cos(tp * w) * np.sin(tp * x)
    dP[..., 1, 0] = amp * tp * np.sin(tp * w) * np.cos(tp * x)
    dP[..., 2, 0] = amp * tp * np.cos(tp * x) * np.sin(tp * y)
    dP[..., 2, 1] = amp * tp * np.sin(tp * x) * np.cos(tp * y)
    Jm = dP * (0.5 / 32)  # dX_b/dxi_i = delta_bi / (2 * 32)
    J, df = _factors_from_jacobian(Jm)
    return X, J, df


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("Q", [2, 5, 8])
def test_oracle_trilinear_hex_is_exact(Q):
    X, J, df = trilinear_case(Q)
    jac, dfo = ogeom.geom_factors(X, obasis.Basis1D(Q - 1, Q).D2, 3)
    assert _rel(jac.reshape(-1), J) < 1e-13 and _rel(dfo, df) < 1e-13


@pytest.mark.parametrize("Q", sorted(CURVED_TOL))
def test_oracle_curved_map_matches_analytic(Q):
    X, J, df = curved_case(Q)
    jac, dfo = ogeom.geom_factors(X, obasis.Basis1D(Q - 1, Q).D2, 3)
    assert _rel(jac.reshape(-1), J) < CURVED_TOL[Q]
    assert _rel(dfo, df) < CURVED_TOL[Q]


@pytest.mark.gpu
@pytest.mark.parametrize("Q", [2, 5, 8])
def test_gpu_trilinear_hex_is_exact(Q):
    from ithaca_gpu.operators import Context, geom_factors
    ctx = Context(0)
    X, J, df = trilinear_case(Q)
    jac, dfg = geom_factors(ctx, "hex", Q, np.repeat(X, 3, axis=1))
    assert _rel(jac[:Q ** 3], J) < 1e-13 and _rel(dfg.reshape(9, 3, -1)[:, 0], df) < 1e-13
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("Q", sorted(CURVED_TOL))
def test_gpu_curved_map_matches_analytic(Q):
    from ithaca_gpu.operators import Context, geom_factors
    ctx = Context(0)
    X, J, df = curved_case(Q)
    jac, dfg = geom_factors(ctx, "hex", Q, X)
    assert _rel(jac, J) < CURVED_TOL[Q] and _rel(dfg, df) < CURVED_TOL[Q]
    ctx.close()
