"""Seeded test cases shared by the CPU and GPU tests (small sizes the oracle runs in seconds)."""
import numpy as np

from ithaca_gpu.mesh import HexMesh, PrismMesh, PyrMesh, QuadMesh, TetMesh, TriMesh
from oracle import basis as obasis
from oracle import geom as ogeom
from oracle import prism as oprism
from oracle import pyr as opyr
from oracle import tet as otet
from oracle import tri as otri


class Case:
    pass


def quad_case(nx, ny, n, jitter=0.1, seed=0, rotate=None, deformed=True):
    c = Case()
    c.dim, c.shape, c.n, c.Q = 2, "quad", n, n + 1
    c.mesh = QuadMesh(nx, ny, jitter=jitter, seed=seed, rotate=rotate)
    c.E = c.mesh.E
    c.X = c.mesh.coords(c.Q)
    c.basis = obasis.Basis1D(n, c.Q)
    jac, df = ogeom.geom_factors(c.X, c.basis.D2, 2)
    c.deformed = deformed
    if deformed:
        c.jac, c.df = jac.reshape(-1).copy(), df.copy()
    else:  # straight-sided parallelograms: per-element constants (GeomFactors eRegular)
        nq = c.Q ** 2
        c.jac = jac[:, 0].copy()
        c.df = df.reshape(4, c.E, nq)[:, :, 0].copy()
    c.nm, c.nq = n * n, c.Q * c.Q
    return c


def hex_case(nx, ny, nz, n, amp=0.05, deformed=True):
    c = Case()
    c.dim, c.shape, c.n, c.Q = 3, "hex", n, n + 1
    c.mesh = HexMesh(nx, ny, nz, curve_amp=amp)
    c.E = c.mesh.E
    c.X = c.mesh.coords(c.Q)
    c.basis = obasis.Basis1D(n, c.Q)
    jac, df = ogeom.geom_factors(c.X, c.basis.D2, 3)
    c.deformed = deformed
    if deformed:
        c.jac, c.df = jac.reshape(-1).copy(), df.copy()
    else:
        nq = c.Q ** 3
        c.jac = jac[:, 0].copy()
        c.df = df.reshape(9, c.E, nq)[:, :, 0].copy()
    c.nm, c.nq = n ** 3, c.Q ** 3
    return c


def tri_case(nx, ny, n, jitter=0.15, seed=3, curve=0.05, deformed=True):
    """TriMesh of 2 nx ny triangles (local vertex orders rotated), n modes; deformed: curved
    and per-point geometry from the oracle's GeomFactors, else straight and per element."""
    c = Case()
    c.dim, c.shape, c.n, c.Q = 2, "tri", n, n + 1
    E = 2 * nx * ny
    c.mesh = TriMesh(nx, ny, jitter=jitter, seed=seed, rotate=np.arange(E) % 3,
                     curve_amp=curve if deformed else 0.0)
    c.E = E
    c.X = c.mesh.coords(n)
    c.basis = otri.TriBasis(n)
    c.deformed = deformed
    if deformed:
        jac, df = otri.geom_factors(c.basis, c.X)
        c.jac, c.df = jac.reshape(-1).copy(), df.copy()
    else:
        c.jac, c.df = otri.straight_tri_geometry(c.mesh.V[c.mesh.EV])
    c.nm, c.nq = c.basis.nc, c.basis.nq
    return c


def tet_case(nx, ny, nz, n, jitter=0.2, seed=3, curve=0.03, deformed=True):
    """TetMesh of 6 nx ny nz tetrahedra, n modes; deformed: curved with per-point geometry
    from the oracle's GeomFactors, else straight and per element."""
    c = Case()
    c.dim, c.shape, c.n, c.Q = 3, "tet", n, n + 1
    c.mesh = TetMesh(nx, ny, nz, jitter=jitter, seed=seed, curve_amp=curve if deformed else 0.0)
    c.E = c.mesh.E
    c.X = c.mesh.coords(n)
    c.basis = otet.TetBasis(n)
    c.deformed = deformed
    if deformed:
        jac, df = otet.geom_factors(c.basis, c.X)
        c.jac, c.df = jac.reshape(-1).copy(), df.copy()
    else:
        c.jac, c.df = otet.straight_tet_geometry(c.mesh.V[c.mesh.EV])
    c.nm, c.nq = c.basis.nc, c.basis.nq
    return c


def prism_case(nx, ny, nz, n, jitter=0.2, seed=3, curve=0.05, deformed=True):
    """PrismMesh of 2 nx ny nz prisms, n modes; deformed: curved and jittered with per-point
    geometry, else straight and unjittered with per-element geometry."""
    c = Case()
    c.dim, c.shape, c.n, c.Q = 3, "prism", n, n + 1
    c.mesh = PrismMesh(nx, ny, nz, jitter=jitter if deformed else 0.0, seed=seed,
                       curve_amp=curve if deformed else 0.0)
    c.E = c.mesh.E
    c.X = c.mesh.coords(n)
    c.basis = oprism.PrismBasis(n)
    c.deformed = deformed
    jac, df = oprism.geom_factors(c.basis, c.X)
    if deformed:
        c.jac, c.df = jac.reshape(-1).copy(), df.copy()
    else:
        c.jac, c.df = jac[:, 0].copy(), df.reshape(9, c.E, -1)[:, :, 0].copy()
    c.nm, c.nq = c.basis.nc, c.basis.nq
    return c


def pyr_case(nx, ny, nz, n, jitter=0.2, seed=3, curve=0.05, deformed=True):
    """PyrMesh of 6 nx ny nz pyramids, n modes; deformed: curved and jittered with per-point
    geometry, else straight with per-element geometry (the straight pyramid maps of this mesh
    are affine)."""
    c = Case()
    c.dim, c.shape, c.n, c.Q = 3, "pyr", n, n + 1
    c.mesh = PyrMesh(nx, ny, nz, jitter=jitter if deformed else 0.0, seed=seed,
                     curve_amp=curve if deformed else 0.0)
    c.E = c.mesh.E
    c.X = c.mesh.coords(n)
    c.basis = opyr.PyrBasis(n)
    c.deformed = deformed
    jac, df = opyr.geom_factors(c.basis, c.X)
    if deformed:
        c.jac, c.df = jac.reshape(-1).copy(), df.copy()
    else:
        c.jac, c.df = jac[:, 0].copy(), df.reshape(9, c.E, -1)[:, :, 0].copy()
    c.nm, c.nq = c.basis.nc, c.basis.nq
    return c


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def hex_dirichlet(mesh, amap, basis, X, fn):
    """Dirichlet global coefficients (amap.ndir values) of fn on the boundary of a
    structured HexMesh: the boundary-constrained projection (oracle.bc) of fn on every
    boundary face, mapped to the element's modes on that face."""
    from oracle import bc
    n, Q, E = basis.n, basis.Q, mesh.E
    nx, ny, nz = mesh.nx, mesh.ny, mesh.nz
    L = amap.l2g.reshape(E, n, n, n)    # [e, r, q, p]
    Xp = X.reshape(3, E, Q, Q, Q)       # [c, e, k, j, i]
    xd = np.full(amap.ndir, np.nan)
    for e in range(E):
        ix, iy, iz = e % nx, (e // nx) % ny, e // (nx * ny)
        faces = []
        for axis, idx, cnt in (("i", ix, nx), ("j", iy, ny), ("k", iz, nz)):
            if idx == 0:
                faces.append((axis, 0, 0))
            if idx == cnt - 1:
                faces.append((axis, Q - 1, 1))
        for axis, pt, mode in faces:
            if axis == "k":      # face (a = i, b = j); modes (p = a, q = b, r = mode)
                P, G = Xp[:, e, pt, :, :], L[e, mode, :, :]
            elif axis == "j":    # face (a = i, b = k); modes (p = a, q = mode, r = b)
                P, G = Xp[:, e, :, pt, :], L[e, :, mode, :]
            else:                # face (a = j, b = k); modes (p = mode, q = a, r = b)
                P, G = Xp[:, e, :, :, pt], L[e, :, :, mode]
            C = bc.quad_fwd_bnd(basis, fn(P[0], P[1], P[2]).reshape(-1)).reshape(n, n)
            assert np.all(G < amap.ndir)
            xd[G.reshape(-1)] = C.reshape(-1)
    assert not np.isnan(xd).any()
    return xd
