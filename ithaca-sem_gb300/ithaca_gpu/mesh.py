"""Synthetic structured meshes, quadrature-point coordinates and the C0 assembly map.

The reference reads meshes from session XML (SpatialDomains/MeshGraph) and numbers
C0 degrees of freedom in AssemblyMapCG; the benchmark workloads here are synthetic,
so this module generates them directly:

* ``QuadMesh``  -- nx x ny quadrilaterals of the unit square, interior vertices
  jittered by U(-a h, a h) per coordinate from a seed; elements may be rotated
  (their local vertex order cyclically shifted) to exercise edge-orientation signs.
  Element e = j*nx + i has vertices v0..v3 counter-clockwise (QuadGeom convention)
  and the bilinear map of SpatialDomains/QuadGeom.cpp:261-330.
* ``TriMesh``   -- the cells of a (jittered) ``QuadMesh`` split into two triangles each
  along the diagonal from (i+1, j) to (i, j+1); optionally curved by
  (x, y) + amp sin(pi x) sin(pi y) (1, -1/2), which fixes the square's boundary.
  Triangle vertices v0, v1, v2 run counter-clockwise with the affine map
  x = v0 + (v1 - v0)(1 + xi0)/2 + (v2 - v0)(1 + xi1)/2 of SpatialDomains/TriGeom.cpp;
  ``rotate`` shifts a triangle's local vertex order cyclically.
* ``TetMesh``   -- nx x ny x nz cubes of the unit cube, each split into the six Kuhn
  tetrahedra v, v + e_a, v + e_a + e_b, v + e_a + e_b + e_c along the permutations (a, b, c)
  of the axes (a conforming triangulation); interior vertices optionally jittered, the map
  optionally curved by (x, y, z) + amp sin(pi x) sin(pi y) sin(pi z) (1, -1/2, 1/4), which
  fixes the cube's boundary. Local vertices are sorted by global id and, where that
  order is negatively oriented, v0 and v1 are exchanged, so that the collapsed vertex of
  every triangular face is its highest-id vertex in both elements sharing it (the
  orientation rule for collapsed simplex faces); x = v0 + (v1 - v0)(1 + xi0)/2 +
  (v2 - v0)(1 + xi1)/2 + (v3 - v0)(1 + xi2)/2 (SpatialDomains/TetGeom.cpp).
* ``PrismMesh`` -- nx x ny x nz cubes of the unit cube, each split into two prisms
  extruded along y over the triangles (c000, c100, c001) and (c101, c001, c100) of its
  xz-face (StdPrismExp vertex order: v0 v1 v4 at the lower y, v3 v2 v5 above them, the
  singular edge v4-v5 along y); jitter and curvature as TetMesh.
* ``PyrMesh``   -- nx x ny x nz cubes of the unit cube, each split into six pyramids with
  the cube's centre as apex and a face as base (StdPyrExp vertex order, base cycle chosen
  so that the element is positively oriented); jitter and curvature as TetMesh.
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


def radau_points(Q, alpha=1.0):
    """Gauss-Radau-Jacobi points (weight (1 - z)^alpha, z_0 = -1): -1 and the zeros of
    P_{Q-1}^{(alpha,1)}, by Newton with deflation (same values as the library's tables)."""
    m = Q - 1
    roots = []
    for k in range(m):
        r = -np.cos((2.0 * k + 1.0) * np.pi / (2.0 * m))
        if k > 0:
            r = 0.5 * (r + roots[-1])
        for _ in range(200):
            p = _jacobi_ab(m, alpha, 1.0, r)
            dp = 0.5 * (m + alpha + 2.0) * _jacobi_ab(m - 1, alpha + 1.0, 2.0, r)
            step = float(p / (dp - p * sum(1.0 / (r - x) for x in roots)))
            r -= step
            if abs(step) < 1e-16:
                break
        roots.append(r)
    return np.concatenate([[-1.0], roots])


def _jacobi_ab(m, a, b, x):
    x = np.asarray(x, dtype=np.float64)
    p0 = np.ones_like(x)
    if m == 0:
        return p0
    p1 = 0.5 * (a - b + (a + b + 2.0) * x)
    for k in range(2, m + 1):
        apb = a + b
        a1 = 2.0 * k * (k + apb) * (2.0 * k + apb - 2.0)
        a2 = (2.0 * k + apb - 1.0) * (a * a - b * b)
        a3 = (2.0 * k + apb - 2.0) * (2.0 * k + apb - 1.0) * (2.0 * k + apb)
        a4 = 2.0 * (k + a - 1.0) * (k + b - 1.0) * (2.0 * k + apb)
        p0, p1 = p1, ((a2 / a1 + a3 / a1 * x) * p1 - a4 / a1 * p0)
    return p1


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


class TriMesh:
    def __init__(self, nx, ny, jitter=0.0, seed=0, rotate=None, curve_amp=0.0):
        q = QuadMesh(nx, ny, jitter=jitter, seed=seed)
        self.nx, self.ny = nx, ny
        self.V = q.V
        self.E = 2 * nx * ny
        self.curve_amp = curve_amp
        c = q.EV  # cell corners c0..c3 counter-clockwise
        # (c0, c1, c3) and (c2, c3, c1): both counter-clockwise, sharing the diagonal c1-c3
        tris = np.empty((self.E, 3), dtype=np.int64)
        tris[0::2] = c[:, [0, 1, 3]]
        tris[1::2] = c[:, [2, 3, 1]]
        self.rot = np.zeros(self.E, dtype=np.int64) if rotate is None else np.asarray(rotate, dtype=np.int64) % 3
        k = (np.arange(3)[None, :] + self.rot[:, None]) % 3
        self.EV = np.take_along_axis(tris, k, axis=1)

    def _map(self, x, y):
        if self.curve_amp == 0.0:
            return x, y
        b = self.curve_amp * np.sin(np.pi * x) * np.sin(np.pi * y)
        return x + b, y - 0.5 * b

    def coords(self, n):
        """Coordinates at the (n + 1) x n collapsed points (GLL x Gauss-Radau), shape
        (2, E, n (n + 1)), point j*(n + 1) + i."""
        z0, z1 = gll_points(n + 1), radau_points(n)
        e0, e1 = np.meshgrid(z0, z1, indexing="xy")   # [j, i]
        xi0 = 0.5 * (1.0 + e0) * (1.0 - e1) - 1.0
        xi1 = e1
        W = np.stack([-0.5 * (xi0 + xi1), 0.5 * (1.0 + xi0), 0.5 * (1.0 + xi1)])  # [v, j, i]
        X = np.einsum("vji,evc->ceji", W, self.V[self.EV]).reshape(2, self.E, -1)
        x, y = self._map(X[0], X[1])
        return np.stack([x, y]).copy()

    def assembly(self, n):
        """C0 numbering for the triangle expansion with n modes per direction; all boundary
        dofs Dirichlet. Local modes m(p, q) (q fastest): vertices m(0,0) = v0, m(1,0) = v1,
        m(0,1) = v2 (the collapsed top vertex); edge 0 (v0 -> v1) the modes (p >= 2, 0) of
        degree p, edge 1 (v1 -> v2) the modes (1, q >= 1) of degree q + 1, edge 2
        (v0 -> v2) the modes (0, q >= 2) of degree q; the rest interior. An edge mode of
        degree k flips sign, (-1)^k, where the local edge runs from the higher global
        vertex id to the lower (StdTriExp edge maps with AssemblyMapCG orientation signs)."""
        E, EV = self.E, self.EV
        nv = self.V.shape[0]
        ni = max(n - 2, 0)
        nint = max((n - 2) * (n - 3) // 2, 0)
        le = np.stack([EV[:, [0, 1]], EV[:, [1, 2]], EV[:, [0, 2]]], axis=1)  # [e, edge, (start, end)]
        key = np.sort(le, axis=2).reshape(-1, 2)
        uniq, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
        inv = inv.reshape(E, 3)
        ne = uniq.shape[0]
        ebnd = cnt == 1
        vbnd = np.zeros(nv, dtype=bool)
        vbnd[uniq[ebnd].ravel()] = True
        nglob = nv + ne * ni + E * nint
        is_dir = np.zeros(nglob, dtype=bool)
        is_dir[:nv] = vbnd
        is_dir[nv:nv + ne * ni] = np.repeat(ebnd, ni)
        newid, ndir = _renumber_dirichlet_first(np.arange(nglob), is_dir)
        nc = n * (n + 1) // 2
        rows = [(p, q) for p in range(n) for q in range(n - p)]
        l2g = np.zeros((E, nc), dtype=np.int64)
        sgn = np.ones((E, nc))
        forward = le[:, :, 0] < le[:, :, 1]
        icount = 0
        for m, (p, q) in enumerate(rows):
            if (p, q) == (0, 0):
                l2g[:, m] = EV[:, 0]
            elif (p, q) == (1, 0):
                l2g[:, m] = EV[:, 1]
            elif (p, q) == (0, 1):
                l2g[:, m] = EV[:, 2]
            elif q == 0 or p <= 1:
                ed, k = (0, p) if q == 0 else ((1, q + 1) if p == 1 else (2, q))
                l2g[:, m] = nv + inv[:, ed] * ni + (k - 2)
                if k % 2 == 1:
                    sgn[:, m] = np.where(forward[:, ed], 1.0, -1.0)
            else:
                l2g[:, m] = nv + ne * ni + np.arange(E) * nint + icount
                icount += 1
        l2g = newid[l2g]
        return AssemblyMap(l2g.reshape(-1), sgn.reshape(-1), nglob, ndir)


def _modA(p, x):
    if p == 0:
        return 0.5 * (1 - x)
    if p == 1:
        return 0.5 * (1 + x)
    return 0.25 * (1 - x) * (1 + x) * _jacobi_ab(p - 2, 1.0, 1.0, x)


def _modB(p, q, x):
    lo, hi = 0.5 * (1 - x), 0.5 * (1 + x)
    if p == 0:
        return lo if q == 0 else (hi if q == 1 else lo * hi * _jacobi_ab(q - 2, 1.0, 1.0, x))
    if q == 0:
        return lo ** p
    return lo ** p * hi * _jacobi_ab(q - 1, 2.0 * p - 1.0, 1.0, x)


def tet_modal(n, xi0, xi1, xi2):
    """Values of the tetrahedron's modes m(p, q, r) at reference points strictly inside or
    on the faces away from the collapsed edge (xi1 + xi2 < 0, xi2 < 1): (npts, nc), with
    the singular-vertex and singular-edge terms (mode (0,0,1) = (1 + eta2)/2, modes
    (0,1,r) without the eta0 factor)."""
    xi0, xi1, xi2 = (np.asarray(a, dtype=np.float64) for a in (xi0, xi1, xi2))
    e2 = xi2
    e1 = 2 * (1 + xi1) / (1 - xi2) - 1
    e0 = 2 * (1 + xi0) / (-xi1 - xi2) - 1
    cols = []
    for p in range(n):
        for q in range(n - p):
            for r in range(n - p - q):
                if (p, q, r) == (0, 0, 1):
                    cols.append(0.5 * (1 + e2))
                    continue
                a = 1.0 if (p == 0 and q == 1) else _modA(p, e0)
                cols.append(a * _modB(p, q, e1) * _modB(p + q, r, e2))
    return np.stack(np.broadcast_arrays(*cols), axis=-1)


_TET_EDGES = ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))
_TET_FACES = ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3))
_TET_XI = np.array([[-1.0, -1, -1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]])
# prism (StdPrismExp): vertices, edges, faces (quads in cyclic order); the singular edge is 4-5
_PRISM_XI = np.array([[-1.0, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [-1, 1, 1]])
_PRISM_EDGES = ((0, 1), (1, 2), (3, 2), (0, 3), (0, 4), (1, 4), (2, 5), (3, 5), (4, 5))
_PRISM_FACES = ((0, 1, 2, 3), (0, 1, 4), (1, 2, 5, 4), (3, 2, 5), (0, 3, 5, 4))
# pyramid (StdPyrExp): the apex is vertex 4
_PYR_XI = np.array([[-1.0, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1]])
_PYR_EDGES = ((0, 1), (1, 2), (3, 2), (0, 3), (0, 4), (1, 4), (2, 4), (3, 4))
_PYR_FACES = ((0, 1, 2, 3), (0, 1, 4), (1, 2, 4), (3, 2, 4), (0, 3, 4))


def pyr_modal(n, xi0, xi1, xi2):
    """Values of the pyramid's modes m(p, q, r) (r fastest, r < n - max(p, q)) at reference
    points with xi2 < 1: (npts, nc); mode 1, the apex, is (1 + eta2)/2."""
    xi0, xi1, xi2 = (np.asarray(a, dtype=np.float64) for a in (xi0, xi1, xi2))
    e0 = 2 * (1 + xi0) / (1 - xi2) - 1
    e1 = 2 * (1 + xi1) / (1 - xi2) - 1
    lo, hi = 0.5 * (1 - xi2), 0.5 * (1 + xi2)
    cols = []
    for p in range(n):
        for q in range(n):
            for r in range(n - max(p, q)):
                if (p, q, r) == (0, 0, 1):
                    cols.append(hi)
                    continue
                if min(p, q) <= 1:
                    c = _modB(max(p, q), r, xi2)
                else:
                    c = lo ** (p + q - 2) * (1.0 if r == 0 else hi * _jacobi_ab(r - 1, 2.0 * p + 2.0 * q - 3.0, 1.0, xi2))
                cols.append(_modA(p, e0) * _modA(q, e1) * c)
    return np.stack(np.broadcast_arrays(*cols), axis=-1)


def prism_modal(n, xi0, xi1, xi2):
    """Values of the prism's modes m(p, q, r) (r fastest, r < n - p) at reference points
    with xi2 < 1: (npts, nc); the singular-edge modes (0, q, 1) carry no eta0 factor."""
    xi0, xi1, xi2 = (np.asarray(a, dtype=np.float64) for a in (xi0, xi1, xi2))
    e0 = 2 * (1 + xi0) / (1 - xi2) - 1
    cols = []
    for p in range(n):
        for q in range(n):
            for r in range(n - p):
                a = 1.0 if (p == 0 and r == 1) else _modA(p, e0)
                cols.append(a * _modA(q, xi1) * _modB(p, r, xi2))
    return np.stack(np.broadcast_arrays(*cols), axis=-1)


def _face_points(nv):
    """Sample parameters on a face: barycentric (3 rows) for triangles, (s, t) for quads."""
    if nv == 3:
        g = np.array([(a, b) for a in np.linspace(0.1, 0.8, 5) for b in np.linspace(0.1, 0.8, 5) if a + b < 0.95])
        return np.stack([1 - g[:, 0] - g[:, 1], g[:, 0], g[:, 1]])
    s = np.linspace(0.1, 0.9, 5)
    S, T = np.meshgrid(s, s, indexing="ij")
    return np.stack([S.ravel(), T.ravel()])


def _face_xi(ref_xi, fverts, frame, pts):
    """Reference coordinates of the sample points of a face seen in `frame` (local vertex
    indices: the triangle's vertices, or the quad's origin, first-axis and second-axis
    neighbours and opposite vertex)."""
    if len(fverts) == 3:
        return sum(pts[c][..., None] * ref_xi[frame[c]] for c in range(3))
    o, a, b, d = (ref_xi[v] for v in frame)
    s, t = pts[0][..., None], pts[1][..., None]
    return (1 - s) * (1 - t) * o + s * (1 - t) * a + (1 - s) * t * b + s * t * d


def _local_topology(n, modal, ref_xi, edges, faces):
    """Per local mode: ('v', vertex), ('e', edge, degree, sign along the local edge),
    ('f', face) or ('i',), found by evaluating the modes: a mode belongs to the
    lowest-dimensional entity on which it does not vanish (points are pulled 1e-9 towards
    the centroid to stay off the collapsed vertices and edges)."""
    cen = ref_xi.mean(axis=0)

    def vals(xi):
        xi = (1 - 1e-9) * np.asarray(xi, dtype=np.float64) + 1e-9 * cen
        return modal(n, xi[..., 0], xi[..., 1], xi[..., 2])
    s = np.linspace(-0.8, 0.8, n + 3)
    vv = vals(ref_xi)
    ev = [vals(((1 - s) / 2)[:, None] * ref_xi[a] + ((1 + s) / 2)[:, None] * ref_xi[b]) for a, b in edges]
    fv = []
    for f in faces:
        frame = f if len(f) == 3 else (f[0], f[1], f[3], f[2])
        fv.append(vals(_face_xi(ref_xi, f, frame, _face_points(len(f)))))
    tol = 1e-6
    one_d = np.stack([_modA(k, s) for k in range(2, n)]) if n > 2 else np.zeros((0, s.size))
    topo = []
    for m in range(vv.shape[1]):
        on_v = np.flatnonzero(np.abs(vv[:, m]) > tol)
        if on_v.size:
            assert on_v.size == 1, "a vertex mode is non-zero at one vertex"
            topo.append(("v", int(on_v[0])))
            continue
        on_e = [k for k in range(len(edges)) if np.max(np.abs(ev[k][:, m])) > tol]
        if on_e:
            assert len(on_e) == 1, "an edge mode lives on one edge"
            f = ev[on_e[0]][:, m]
            coef = one_d @ f / np.sum(one_d * one_d, axis=1)
            k = int(np.argmax(np.abs(coef)))
            assert np.max(np.abs(f - coef[k] * one_d[k])) < 1e-6 and abs(abs(coef[k]) - 1) < 1e-6
            topo.append(("e", on_e[0], k + 2, float(np.sign(coef[k]))))
            continue
        on_f = [k for k in range(len(faces)) if np.max(np.abs(fv[k][:, m])) > tol]
        if on_f:
            assert len(on_f) == 1, "a face mode lives on one face"
            topo.append(("f", on_f[0]))
            continue
        topo.append(("i",))
    return topo


def _canonical_frame(fverts, gids):
    """Local vertex indices of a face in the global frame: triangles by increasing global
    id; quads from the lowest-id vertex towards its lower-id neighbour first."""
    if len(fverts) == 3:
        return tuple(fverts[i] for i in np.argsort(gids))
    o = int(np.argmin(gids))
    nb1, nb2 = (o + 1) % 4, (o + 3) % 4
    if gids[nb2] < gids[nb1]:
        nb1, nb2 = nb2, nb1
    return (fverts[o], fverts[nb1], fverts[nb2], fverts[(o + 2) % 4])


def _c0_assembly(n, modal, ref_xi, edges, faces, EV, nv):
    """C0 numbering of a conforming mesh of one collapsed element type (vertex ids EV):
    vertices, then edge modes (sign (-1)^k where the local edge runs against the global
    low-to-high direction), face modes matched between the elements of a face by their
    restriction to it in the face's global frame (a permutation with signs), then interior
    modes; every boundary dof Dirichlet, numbered first."""
    E = EV.shape[0]
    topo = _local_topology(n, modal, ref_xi, edges, faces)
    nc = len(topo)
    ni = max(n - 2, 0)
    ekeys = np.stack([np.sort(EV[:, list(e)], axis=1) for e in edges], axis=1).reshape(-1, 2)
    ue, einv = np.unique(ekeys, axis=0, return_inverse=True)
    einv = einv.reshape(E, len(edges))
    fkeys = [tuple(sorted(EV[e, list(f)])) for e in range(E) for f in faces]
    fid, fcount = {}, {}
    for k in fkeys:
        if k not in fid:
            fid[k] = len(fid)
        fcount[k] = fcount.get(k, 0) + 1
    finv = np.array([fid[k] for k in fkeys]).reshape(E, len(faces))
    nF = len(fid)
    fmodes = {f: [m for m, t in enumerate(topo) if t[0] == "f" and t[1] == f] for f in range(len(faces))}
    nfm = {f: len(fmodes[f]) for f in fmodes}
    # per global face: its size in modes (the first element's count) and offset
    fsize = np.zeros(nF, dtype=np.int64)
    for e in range(E):
        for f in range(len(faces)):
            fsize[finv[e, f]] = nfm[f]
    foff = np.concatenate([[0], np.cumsum(fsize)])
    nint = sum(1 for t in topo if t[0] == "i")
    nE = ue.shape[0]
    nglob = nv + nE * ni + int(foff[-1]) + E * nint
    fbnd = np.zeros(nF, dtype=bool)
    for k, c in fcount.items():
        fbnd[fid[k]] = c == 1
    is_dir = np.zeros(nglob, dtype=bool)
    bverts = {v for k, c in fcount.items() if c == 1 for v in k}
    is_dir[list(bverts)] = True
    bedges = set()
    for k, c in fcount.items():
        if c == 1:
            kk = list(k)
            for a in range(len(kk)):
                for b in range(a + 1, len(kk)):
                    bedges.add((kk[a], kk[b]))
    eid = {tuple(x): i for i, x in enumerate(ue.tolist())}
    for be in bedges:
        if be in eid:   # quad diagonals are not edges
            i = eid[be]
            is_dir[nv + i * ni:nv + (i + 1) * ni] = True
    for g in np.flatnonzero(fbnd):
        is_dir[nv + nE * ni + foff[g]:nv + nE * ni + foff[g + 1]] = True
    newid, ndir = _renumber_dirichlet_first(np.arange(nglob), is_dir)
    l2g = np.zeros((E, nc), dtype=np.int64)
    sgn = np.ones((E, nc))
    for m, t in enumerate(topo):
        if t[0] == "v":
            l2g[:, m] = EV[:, t[1]]
        elif t[0] == "e":
            _, ed, k, s_loc = t
            a, b = edges[ed]
            fwd = EV[:, a] < EV[:, b]
            l2g[:, m] = nv + einv[:, ed] * ni + (k - 2)
            sgn[:, m] = s_loc * np.where(fwd, 1.0, (-1.0) ** k)
    cen = ref_xi.mean(axis=0)
    cache, owner = {}, {}

    def face_vals(f, frame):
        key = (f, frame)
        if key not in cache:
            xi = _face_xi(ref_xi, faces[f], frame, _face_points(len(faces[f])))
            xi = (1 - 1e-9) * xi + 1e-9 * cen
            cache[key] = modal(n, xi[..., 0], xi[..., 1], xi[..., 2])[:, fmodes[f]]
        return cache[key]
    match = {}
    for e in range(E):
        for f, fv in enumerate(faces):
            if not fmodes[f]:
                continue
            g = finv[e, f]
            frame = _canonical_frame(fv, EV[e, list(fv)])
            key = (f, frame)
            if g not in owner:
                owner[g] = key
            pair = (owner[g], key)
            if pair not in match:
                A, B = face_vals(*owner[g]), face_vals(*key)
                hits = []
                for b in range(B.shape[1]):
                    hit = None
                    for a in range(A.shape[1]):
                        for sg in (1.0, -1.0):
                            if np.max(np.abs(B[:, b] - sg * A[:, a])) < 1e-8:
                                hit = (a, sg)
                    assert hit is not None, "face modes do not match across a shared face"
                    hits.append(hit)
                match[pair] = hits
            for j, m in enumerate(fmodes[f]):
                a, sg = match[pair][j]
                l2g[e, m] = nv + nE * ni + foff[g] + a
                sgn[e, m] = sg
    base = nv + nE * ni + int(foff[-1])
    ints = [m for m, t in enumerate(topo) if t[0] == "i"]
    for j, m in enumerate(ints):
        l2g[:, m] = base + np.arange(E) * nint + j
    l2g = newid[l2g]
    return AssemblyMap(l2g.reshape(-1), sgn.reshape(-1), nglob, ndir)


class TetMesh:
    def __init__(self, nx, ny, nz, jitter=0.0, seed=0, curve_amp=0.0):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.curve_amp = curve_amp
        gx, gy, gz = np.meshgrid(np.arange(nx + 1) / nx, np.arange(ny + 1) / ny, np.arange(nz + 1) / nz,
                                 indexing="ij")
        # vertex id = (k (ny + 1) + j) (nx + 1) + i
        V = np.stack([gx.transpose(2, 1, 0).ravel(), gy.transpose(2, 1, 0).ravel(), gz.transpose(2, 1, 0).ravel()],
                     axis=1)
        if jitter > 0:
            rng = np.random.default_rng(seed)
            i = np.tile(np.arange(nx + 1), (ny + 1) * (nz + 1))
            j = np.tile(np.repeat(np.arange(ny + 1), nx + 1), nz + 1)
            k = np.repeat(np.arange(nz + 1), (nx + 1) * (ny + 1))
            inner = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
            d = rng.uniform(-jitter, jitter, size=V.shape) / np.array([nx, ny, nz])
            V[inner] += d[inner]
        self.V = V
        step = np.array([1, nx + 1, (nx + 1) * (ny + 1)])
        ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
        base = ((ck * (ny + 1) + cj) * (nx + 1) + ci).transpose(2, 1, 0).ravel()
        tets = []
        for perm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
            v1 = base + step[perm[0]]
            v2 = v1 + step[perm[1]]
            v3 = v2 + step[perm[2]]
            tets.append(np.stack([base, v1, v2, v3], axis=1))
        EV = np.stack(tets, axis=1).reshape(-1, 4)  # already ascending by id along each path
        P = V[EV]
        det = np.einsum("ei,ei->e", P[:, 1] - P[:, 0], np.cross(P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]))
        swap = det < 0
        EV[swap] = EV[swap][:, [1, 0, 2, 3]]
        self.EV = EV
        self.swapped = swap
        self.E = EV.shape[0]

    def _map(self, x, y, z):
        if self.curve_amp == 0.0:
            return x, y, z
        b = self.curve_amp * np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z)
        return x + b, y - 0.5 * b, z + 0.25 * b

    def coords(self, n):
        """Coordinates at the (n + 1) x n x n collapsed points (GLL x Gauss-Radau alpha 1 x
        Gauss-Radau alpha 2), shape (3, E, (n + 1) n^2), point (k n + j) (n + 1) + i."""
        z0, z1, z2 = gll_points(n + 1), radau_points(n), radau_points(n, alpha=2.0)
        e2, e1, e0 = np.meshgrid(z2, z1, z0, indexing="ij")
        xi2 = e2
        xi1 = 0.5 * (1 + e1) * (1 - e2) - 1
        xi0 = 0.25 * (1 + e0) * (1 - e1) * (1 - e2) - 1
        W = np.stack([-0.5 * (1 + xi0 + xi1 + xi2), 0.5 * (1 + xi0), 0.5 * (1 + xi1), 0.5 * (1 + xi2)])
        X = np.einsum("vkji,evc->cekji", W, self.V[self.EV]).reshape(3, self.E, -1)
        return np.stack(self._map(X[0], X[1], X[2])).copy()

    def assembly(self, n):
        """C0 numbering of the tetrahedron expansion with n modes per direction; all
        boundary dofs Dirichlet (``_c0_assembly``: with the sorted local vertex order both
        elements of a face see the same collapsed vertex, so its modes match up to sign)."""
        return _c0_assembly(n, tet_modal, _TET_XI, _TET_EDGES, _TET_FACES, self.EV, self.V.shape[0])


class PrismMesh:
    def __init__(self, nx, ny, nz, jitter=0.0, seed=0, curve_amp=0.0):
        t = TetMesh(nx, ny, nz, jitter=jitter, seed=seed)
        self.V = t.V
        self.curve_amp = curve_amp
        step = np.array([1, nx + 1, (nx + 1) * (ny + 1)])
        ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
        c000 = ((ck * (ny + 1) + cj) * (nx + 1) + ci).transpose(2, 1, 0).ravel()
        c = lambda a, b, d: c000 + a * step[0] + b * step[1] + d * step[2]
        pa = np.stack([c(0, 0, 0), c(1, 0, 0), c(1, 1, 0), c(0, 1, 0), c(0, 0, 1), c(0, 1, 1)], axis=1)
        pb = np.stack([c(1, 0, 1), c(0, 0, 1), c(0, 1, 1), c(1, 1, 1), c(1, 0, 0), c(1, 1, 0)], axis=1)
        self.EV = np.stack([pa, pb], axis=1).reshape(-1, 6)
        self.E = self.EV.shape[0]

    _map = TetMesh._map

    def coords(self, n):
        """Coordinates at the (n + 1) x (n + 1) x n points (GLL x GLL x Gauss-Radau alpha 1),
        shape (3, E, (n + 1)^2 n), point (k (n + 1) + j) (n + 1) + i."""
        z0, z2 = gll_points(n + 1), radau_points(n)
        e2, e1, e0 = np.meshgrid(z2, z0, z0, indexing="ij")
        xi0 = 0.5 * (1 + e0) * (1 - e2) - 1
        xi1, xi2 = e1, e2
        tri = lambda: (-0.5 * (xi0 + xi2), 0.5 * (1 + xi0), 0.5 * (1 + xi2))
        lo, hi = 0.5 * (1 - xi1), 0.5 * (1 + xi1)
        a, b, d = tri()
        # v0 v1 v4 below, v3 v2 v5 above
        W = np.stack([lo * a, lo * b, hi * b, hi * a, lo * d, hi * d])
        X = np.einsum("vkji,evc->cekji", W, self.V[self.EV]).reshape(3, self.E, -1)
        return np.stack(self._map(X[0], X[1], X[2])).copy()

    def assembly(self, n):
        """C0 numbering of the prism expansion with n modes; all boundary dofs Dirichlet."""
        return _c0_assembly(n, prism_modal, _PRISM_XI, _PRISM_EDGES, _PRISM_FACES, self.EV, self.V.shape[0])


class PyrMesh:
    def __init__(self, nx, ny, nz, jitter=0.0, seed=0, curve_amp=0.0):
        t = TetMesh(nx, ny, nz, jitter=jitter, seed=seed)
        nv = t.V.shape[0]
        self.curve_amp = curve_amp
        step = np.array([1, nx + 1, (nx + 1) * (ny + 1)])
        ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
        c000 = ((ck * (ny + 1) + cj) * (nx + 1) + ci).transpose(2, 1, 0).ravel()
        ncell = c000.size
        c = lambda a, b, d: c000 + a * step[0] + b * step[1] + d * step[2]
        corners = {(a, b, d): c(a, b, d) for a in (0, 1) for b in (0, 1) for d in (0, 1)}
        centres = nv + np.arange(ncell)
        cen_xyz = np.mean([t.V[corners[k]] for k in corners], axis=0)
        self.V = np.concatenate([t.V, cen_xyz])
        faces = (((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)), ((0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1)),
                 ((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0)), ((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)),
                 ((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)), ((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0)))
        pyrs = []
        for f in faces:
            base = np.stack([corners[k] for k in f], axis=1)
            pyrs.append(np.concatenate([base, centres[:, None]], axis=1))
        EV = np.stack(pyrs, axis=1).reshape(-1, 5)
        P = self.V[EV]
        det = np.einsum("ei,ei->e", P[:, 1] - P[:, 0], np.cross(P[:, 3] - P[:, 0], P[:, 4] - P[:, 0]))
        flip = det < 0
        EV[flip] = EV[flip][:, [0, 3, 2, 1, 4]]
        self.EV = EV
        self.E = EV.shape[0]

    _map = TetMesh._map

    def coords(self, n):
        """Coordinates at the (n + 1) x (n + 1) x n points (GLL x GLL x Gauss-Radau alpha 2),
        shape (3, E, (n + 1)^2 n): x = (1 - eta2)/2 (bilinear base map) + (1 + eta2)/2 apex."""
        z0, z2 = gll_points(n + 1), radau_points(n, alpha=2.0)
        e2, e1, e0 = np.meshgrid(z2, z0, z0, indexing="ij")
        lo, hi = 0.5 * (1 - e2), 0.5 * (1 + e2)
        a0, b0, a1, b1 = 0.5 * (1 - e0), 0.5 * (1 + e0), 0.5 * (1 - e1), 0.5 * (1 + e1)
        W = np.stack([lo * a0 * a1, lo * b0 * a1, lo * b0 * b1, lo * a0 * b1, hi])
        X = np.einsum("vkji,evc->cekji", W, self.V[self.EV]).reshape(3, self.E, -1)
        return np.stack(self._map(X[0], X[1], X[2])).copy()

    def assembly(self, n):
        """C0 numbering of the pyramid expansion with n modes; all boundary dofs Dirichlet."""
        return _c0_assembly(n, pyr_modal, _PYR_XI, _PYR_EDGES, _PYR_FACES, self.EV, self.V.shape[0])


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
