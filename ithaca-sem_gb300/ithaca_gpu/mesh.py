"""Synthetic structured meshes, quadrature-point coordinates and the C0 assembly map.

The reference reads meshes from session XML (SpatialDomains/MeshGraph) and numbers
C0 degrees of freedom in AssemblyMapCG; the benchmark workloads here are synthetic,
so this module generates them directly:

* ``QuadMesh``  -- nx x ny quadrilaterals of the unit square, interior vertices
  jittered by U(-a h, a h) per coordinate from a seed; elements may be rotated
  (their local vertex order cyclically shifted) to exercise edge-orientation signs.
  Element e = j*nx + i has vertices v0..v3 counter-clockwise (QuadGeom convention)
  and the bilinear map of SpatialDomains/QuadGeom.cpp:261-330.
* ``HexMesh``   -- nx x ny x nz hexahedra of the unit cube, optionally curved by
  x_a + amp * sin(2 pi x_b) sin(2 pi x_c) applied cyclically (a, b, c) =
  (0, 1, 2), (1, 2, 0), (2, 0, 1) to the straight positions.

Numbering follows the ModifiedA C0 rules of AssemblyMapCG (vertex modes p in {0, 1},
edge/face/interior modes p >= 2; an edge mode p flips sign, (-1)^p, where the local
edge direction opposes the global one, MultiRegions/AssemblyMap/AssemblyMapCG.cpp),
with the Dirichlet (boundary) dofs numbered first. ``l2g_signed`` packs sign and id
into one int32 as the kernels read it: g for +1, ~g for -1.
"""
import numpy as np


def gll_points(Q):
    """GLL points on [-1, 1] (same values as the library's basis tables)."""
    N = Q - 1
    z = -np.cos(np.pi * np.arange(Q) / N)
    zi = z[1:-1].copy()
    for _ in range(100):
        p_prev = np.ones_like(zi)
        p = zi.copy()
        for k in range(2, N + 1):
            p_prev, p = p, ((2 * k - 1) * zi * p - (k - 1) * p_prev) / k
        dp = N * (zi * p - p_prev) / (zi * zi - 1.0)
        step = (1.0 - zi * zi) * dp / (-N * (N + 1) * p)
        zi -= step
        if np.max(np.abs(step), initial=0.0) < 1e-16:
            break
    z[1:-1] = zi
    return z


class AssemblyMap:
    """Local-to-global map with signs (AssemblyMapCG analogue)."""

    def __init__(self, l2g, sign, nglobal, ndir):
        self.l2g = np.ascontiguousarray(l2g, dtype=np.int32)
        self.sign = np.ascontiguousarray(sign, dtype=np.float64)
        self.nglobal = int(nglobal)
        self.ndir = int(ndir)

    @property
    def l2g_signed(self):
        return np.where(self.sign > 0, self.l2g, ~self.l2g).astype(np.int32)

    def global_to_local(self, x):
        """AssemblyMapCG::v_GlobalToLocal (:2853-2876): local = sign * global[map]."""
        return self.sign * x[self.l2g]

    def assemble(self, loc):
        """AssemblyMapCG::v_Assemble (:2885-2910): global = sum sign * local."""
        out = np.zeros(self.nglobal)
        np.add.at(out, self.l2g, self.sign * loc)
        return out


def _renumber_dirichlet_first(ids, is_dir_entity):
    """ids: global ids (any order); is_dir_entity: bool per id. Returns (newid map, ndir)."""
    n = is_dir_entity.size
    order = np.concatenate([np.flatnonzero(is_dir_entity), np.flatnonzero(~is_dir_entity)])
    newid = np.empty(n, dtype=np.int64)
    newid[order] = np.arange(n)
    return newid, int(is_dir_entity.sum())


class QuadMesh:
    def __init__(self, nx, ny, jitter=0.0, seed=0, rotate=None, extent=(1.0, 1.0)):
        self.nx, self.ny = nx, ny
        self.E = nx * ny
        hx, hy = extent[0] / nx, extent[1] / ny
        gx, gy = np.meshgrid(np.arange(nx + 1) * hx, np.arange(ny + 1) * hy, indexing="xy")
        V = np.stack([gx.ravel(), gy.ravel()], axis=1)  # vertex id = j*(nx+1) + i
        if jitter > 0:
            rng = np.random.default_rng(seed)
            d = rng.uniform(-jitter, jitter, size=V.shape) * np.array([hx, hy])
            ii = np.tile(np.arange(nx + 1), ny + 1)
            jj = np.repeat(np.arange(ny + 1), nx + 1)
            interior = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny)
            V[interior] += d[interior]
        self.V = V
        ie = np.tile(np.arange(nx), ny)
        je = np.repeat(np.arange(ny), nx)
        vid = lambda i, j: j * (nx + 1) + i
        corners = np.stack([vid(ie, je), vid(ie + 1, je), vid(ie + 1, je + 1), vid(ie, je + 1)], axis=1)
        self.rot = np.zeros(self.E, dtype=np.int64) if rotate is None else np.asarray(rotate, dtype=np.int64)
        k = (np.arange(4)[None, :] + self.rot[:, None]) % 4
        self.EV = np.take_along_axis(corners, k, axis=1)  # element vertices v0..v3 (CCW)

    def coords(self, Q):
        """Coordinates at the Q x Q GLL points, shape (2, E, Q*Q), point j*Q + i."""
        z = gll_points(Q)
        a = 0.5 * (1 - z)
        b = 0.5 * (1 + z)
        # weights for v0..v3 at (xi0_i, xi1_j): v0 a_i a_j, v1 b_i a_j, v2 b_i b_j, v3 a_i b_j
        W = np.stack([np.outer(a, a), np.outer(a, b), np.outer(b, b), np.outer(b, a)], axis=0)  # [v, j, i]
        X = np.einsum("vji,evc->ceji", W, self.V[self.EV])
        return X.reshape(2, self.E, Q * Q).copy()

    def assembly(self, n):
        """C0 numbering for n ModifiedA modes per direction; all boundary dofs Dirichlet."""
        nx, ny, E = self.nx, self.ny, self.E
        nv = (nx + 1) * (ny + 1)
        nh = nx * (ny + 1)
        ne = nh + (nx + 1) * ny
        ni = max(n - 2, 0)
        vi = np.arange(nv) % (nx + 1)
        vj = np.arange(nv) // (nx + 1)
        vbnd = (vi == 0) | (vi == nx) | (vj == 0) | (vj == ny)

        def edge_id(va, vb):
            lo, hi = np.minimum(va, vb), np.maximum(va, vb)
            horiz = (hi - lo) == 1
            i_lo, j_lo = lo % (nx + 1), lo // (nx + 1)
            return np.where(horiz, j_lo * nx + i_lo, nh + j_lo * (nx + 1) + i_lo), lo

        eid_all = np.arange(ne)
        eb_h = (eid_all < nh) & (((eid_all // nx) == 0) | ((eid_all // nx) == ny))
        ev = eid_all - nh
        eb_v = (eid_all >= nh) & (((ev % (nx + 1)) == 0) | ((ev % (nx + 1)) == nx))
        ebnd = eb_h | eb_v
        # entity global ids before renumbering: vertices, edges (ni each), interiors
        nglob = nv + ne * ni + E * ni * ni
        is_dir = np.zeros(nglob, dtype=bool)
        is_dir[:nv] = vbnd
        is_dir[nv:nv + ne * ni] = np.repeat(ebnd, ni)
        newid, ndir = _renumber_dirichlet_first(np.arange(nglob), is_dir)

        EV = self.EV
        l2g = np.zeros((E, n, n), dtype=np.int64)  # [e, q, p]
        sgn = np.ones((E, n, n))
        # vertices: (p,q) = (0,0)->v0 (1,0)->v1 (1,1)->v2 (0,1)->v3
        for (p, q, v) in ((0, 0, 0), (1, 0, 1), (1, 1, 2), (0, 1, 3)):
            l2g[:, q, p] = EV[:, v]
        if ni > 0:
            modes = np.arange(2, n)
            flip_sign = np.where(modes % 2 == 1, -1.0, 1.0)
            # edges along xi0: q=0 (v0->v1), q=1 (v3->v2); along xi1: p=0 (v0->v3), p=1 (v1->v2)
            for (fixed, val, vs, ve) in (("q", 0, 0, 1), ("q", 1, 3, 2), ("p", 0, 0, 3), ("p", 1, 1, 2)):
                eid, lo = edge_id(EV[:, vs], EV[:, ve])
                forward = EV[:, vs] == lo
                g = nv + eid[:, None] * ni + (modes - 2)[None, :]
                s = np.where(forward[:, None], 1.0, flip_sign[None, :])
                if fixed == "q":
                    l2g[:, val, 2:] = g
                    sgn[:, val, 2:] = s
                else:
                    l2g[:, 2:, val] = g
                    sgn[:, 2:, val] = s
            base = nv + ne * ni + np.arange(E)[:, None, None] * ni * ni
            qq, pp = np.meshgrid(np.arange(ni), np.arange(ni), indexing="ij")
            l2g[:, 2:, 2:] = base + (qq * ni + pp)[None]
        l2g = newid[l2g]
        return AssemblyMap(l2g.reshape(-1), sgn.reshape(-1), nglob, ndir)


class HexMesh:
    def __init__(self, nx, ny, nz, curve_amp=0.0):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.E = nx * ny * nz
        self.curve_amp = curve_amp

    def _map(self, x, y, z):
        a = self.curve_amp
        if a == 0.0:
            return x, y, z
        tp = 2.0 * np.pi
        return (x + a * np.sin(tp * y) * np.sin(tp * z),
                y + a * np.sin(tp * z) * np.sin(tp * x),
                z + a * np.sin(tp * x) * np.sin(tp * y))

    def coords(self, Q, elements=None):
        """Coordinates at the Q^3 GLL points, shape (3, E, Q^3), point (k*Q + j)*Q + i.
        Element e = (kz*ny + jy)*nx + ix. `elements`: only these element ids (in order)."""
        nx, ny, nz = self.nx, self.ny, self.nz
        z = gll_points(Q)
        t = 0.5 * (1 + z)
        eids = np.arange(self.E) if elements is None else np.asarray(elements, dtype=np.int64)
        ix = eids % nx
        iy = (eids // nx) % ny
        iz = eids // (nx * ny)
        X0 = ((ix[:, None] + t[None, :]) / nx)[:, None, None, :]
        X1 = ((iy[:, None] + t[None, :]) / ny)[:, None, :, None]
        X2 = ((iz[:, None] + t[None, :]) / nz)[:, :, None, None]
        X0, X1, X2 = np.broadcast_arrays(X0, X1, X2)
        Y = self._map(X0, X1, X2)
        return np.stack([c.reshape(eids.size, Q ** 3) for c in Y], axis=0)

    def assembly(self, n):
        """Aligned structured hexes: the C0 dof of local mode (p, q, r) is the tensor
        product of 1-D global ids (vertex modes shared, p >= 2 modes owned), so every
        sign is +1; boundary dofs are Dirichlet and numbered first."""
        nx, ny, nz = self.nx, self.ny, self.nz
        m = max(n - 2, 0)

        def one_d(ne):
            ids = np.zeros((ne, n), dtype=np.int64)
            ids[:, 0] = np.arange(ne)
            ids[:, 1] = np.arange(ne) + 1
            if m:
                ids[:, 2:] = ne + 1 + np.arange(ne)[:, None] * m + np.arange(m)[None, :]
            bnd = np.zeros(ne + 1 + ne * m, dtype=bool)
            bnd[0] = bnd[ne] = True
            return ids, bnd, ne + 1 + ne * m

        gx, bx, Nx = one_d(nx)
        gy, by, Ny = one_d(ny)
        gz, bz, Nz = one_d(nz)
        E = self.E
        ix = np.arange(E) % nx
        iy = (np.arange(E) // nx) % ny
        iz = np.arange(E) // (nx * ny)
        G = ((gz[iz][:, :, None, None] * Ny + gy[iy][:, None, :, None]) * Nx + gx[ix][:, None, None, :])
        nglob = Nx * Ny * Nz
        is_dir = (bz[:, None, None] | by[None, :, None] | bx[None, None, :]).reshape(-1)
        newid, ndir = _renumber_dirichlet_first(np.arange(nglob), is_dir)
        l2g = newid[G].reshape(-1)
        return AssemblyMap(l2g, np.ones(l2g.size), nglob, ndir)
