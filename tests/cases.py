"""Seeded test cases shared by the CPU and GPU tests (small sizes the oracle runs in seconds)."""
import numpy as np

from ithaca_gpu.mesh import HexMesh, QuadMesh
from oracle import basis as obasis
from oracle import geom as ogeom


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


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
