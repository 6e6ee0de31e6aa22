"""Session and mesh input: the subset of the reference's XML session format that the
Helmholtz path needs, for quadrilateral meshes (with boundary conditions) and triangle
meshes (geometry and expansions, the meshes of 2-D snapshot sets).

Reads what LibUtilities::SessionReader (LibUtilities/BasicUtils/SessionReader.cpp) and
SpatialDomains::MeshGraphXml (SpatialDomains/MeshGraphXml.cpp) read from an uncompressed
session file:
  GEOMETRY      VERTEX <V ID>x y z</V>, EDGE <E ID>v0 v1</E>, ELEMENT <Q ID>e0 e1 e2 e3</Q>
                and <T ID>e0 e1 e2</T>, COMPOSITE <C ID>Q[0-15]</C> / T[..] / E[0,13,22,31], DOMAIN
  EXPANSIONS    <E COMPOSITE NUMMODES TYPE FIELDS> (TYPE MODIFIED: ModifiedA on Q = n + 1 GLL points)
  CONDITIONS    PARAMETERS <P>name = value</P>, SOLVERINFO <I PROPERTY VALUE>, VARIABLES,
                BOUNDARYREGIONS <B ID>C[..]</B>, BOUNDARYCONDITIONS (D, N, R, P per region),
                FUNCTION <E VAR VALUE> expressions
Expressions use the reference's syntax (LibUtilities/Interpreter): + - * / ^, the usual
functions (sin, cos, exp, sqrt, ...), the constant PI and the session's parameters, in the
variables x, y, z, t. They are parsed to a Python syntax tree and evaluated over numpy
arrays; only those names and operators are accepted.

``QuadSessionMesh`` turns the element/edge lists into the library's layouts: vertex
cycles (counter-clockwise, from each quad's edge list), quadrature-point coordinates of
the bilinear map (QuadGeom.cpp:261-330) and the C0 assembly map for n ModifiedA modes,
with Dirichlet dofs numbered first and periodic edges identified (the periodic regions'
edges are matched by translation, as MeshGraph/AssemblyMapCG match periodic entities),
plus the boundary-constrained projection of Dirichlet data onto the boundary edges
(StdSegExp::FwdTrans_BndConstrained, StdRegions/StdSegExp.cpp:319-390).
"""
import ast
import math
import re
import xml.etree.ElementTree as ET

import numpy as np

from .mesh import AssemblyMap, gll_points, radau_points

_FUNCS = {"sin": np.sin, "cos": np.cos, "tan": np.tan, "exp": np.exp, "log": np.log, "log10": np.log10,
          "sqrt": np.sqrt, "abs": np.abs, "fabs": np.abs, "sinh": np.sinh, "cosh": np.cosh, "tanh": np.tanh,
          "asin": np.arcsin, "acos": np.arccos, "atan": np.arctan, "atan2": np.arctan2, "pow": np.power}
_CONSTS = {"PI": math.pi, "pi": math.pi, "E": math.e}
_OPS = (ast.Expression, ast.BinOp, ast.UnaryOp, ast.Call, ast.Name, ast.Constant, ast.Load, ast.Add, ast.Sub,
        ast.Mult, ast.Div, ast.Pow, ast.USub, ast.UAdd)


def compile_expression(text, params):
    """A callable f(x, y, z=0, t=0) for a session expression."""
    src = text.strip().replace("^", "**")
    tree = ast.parse(src, mode="eval")
    names = set(_FUNCS) | set(_CONSTS) | set(params) | {"x", "y", "z", "t"}
    for node in ast.walk(tree):
        if not isinstance(node, _OPS):
            raise ValueError(f"unsupported syntax in expression {text!r}: {type(node).__name__}")
        if isinstance(node, ast.Name) and node.id not in names:
            raise ValueError(f"unknown name {node.id!r} in expression {text!r}")
        if isinstance(node, ast.Call) and not (isinstance(node.func, ast.Name) and node.func.id in _FUNCS):
            raise ValueError(f"unsupported call in expression {text!r}")
    code = compile(tree, "<session expression>", "eval")
    env = dict(_FUNCS)
    env.update(_CONSTS)
    env.update(params)

    def f(x, y, z=0.0, t=0.0):
        x = np.asarray(x, dtype=float)
        val = eval(code, {"__builtins__": {}}, dict(env, x=x, y=np.asarray(y, dtype=float),
                                                     z=np.asarray(z, dtype=float), t=t))
        return np.broadcast_to(np.asarray(val, dtype=float), x.shape).copy()

    return f


def parse_id_list(text):
    """'Q[0-3,5]' -> ('Q', [0, 1, 2, 3, 5]); 'E[0,13]' ; '[2]' -> ('', [2])."""
    m = re.fullmatch(r"\s*([A-Za-z]*)\s*\[([^\]]*)\]\s*", text)
    if not m:
        raise ValueError(f"bad id list {text!r}")
    ids = []
    for part in m.group(2).split(","):
        part = part.strip()
        if not part:
            continue
        if "-" in part:
            a, b = part.split("-")
            ids.extend(range(int(a), int(b) + 1))
        else:
            ids.append(int(part))
    return m.group(1), ids


class Session:
    def __init__(self, root):
        geo = root.find("GEOMETRY")
        if geo is None:
            raise ValueError("no GEOMETRY section")
        self.dim = int(geo.get("DIM"))
        self.space = int(geo.get("SPACE", self.dim))
        for sec in ("VERTEX", "EDGE", "ELEMENT"):
            node = geo.find(sec)
            if node is not None and node.get("COMPRESSED"):
                raise ValueError("compressed geometry sections are not supported")
        self.vertices = {int(v.get("ID")): np.array([float(s) for s in v.text.split()]) for v in geo.find("VERTEX")}
        self.edges = {int(e.get("ID")): tuple(int(s) for s in e.text.split()) for e in geo.find("EDGE")}
        self.elements = {}
        for el in geo.find("ELEMENT"):
            self.elements[int(el.get("ID"))] = (el.tag, [int(s) for s in el.text.split()])
        self.composites = {int(c.get("ID")): parse_id_list(c.text) for c in geo.find("COMPOSITE")}
        dom = geo.find("DOMAIN")
        self.domain = parse_id_list(dom.text)[1] if dom is not None else sorted(self.composites)[:1]
        self.expansions = []
        exp = root.find("EXPANSIONS")
        for e in (exp if exp is not None else []):
            self.expansions.append(dict(composites=parse_id_list(e.get("COMPOSITE"))[1],
                                        nummodes=int(e.get("NUMMODES")), type=e.get("TYPE", "MODIFIED"),
                                        fields=[s.strip() for s in e.get("FIELDS", "u").split(",")]))
        cond = root.find("CONDITIONS")
        self.parameters, self.solverinfo, self.variables = {}, {}, []
        self.boundary_regions, self.boundary_conditions, self.functions = {}, {}, {}
        if cond is not None:
            for p in cond.findall("PARAMETERS/P"):
                name, val = p.text.split("=", 1)
                self.parameters[name.strip()] = float(compile_expression(val, self.parameters)(0.0, 0.0))
            for i in cond.findall("SOLVERINFO/I"):
                self.solverinfo[i.get("PROPERTY")] = i.get("VALUE")
            self.variables = [v.text.strip() for v in cond.findall("VARIABLES/V")]
            for b in cond.findall("BOUNDARYREGIONS/B"):
                self.boundary_regions[int(b.get("ID"))] = parse_id_list(b.text)[1]
            for reg in cond.findall("BOUNDARYCONDITIONS/REGION"):
                bcs = {}
                for bc in reg:
                    bcs[bc.get("VAR")] = (bc.tag, bc.get("VALUE"))
                self.boundary_conditions[int(reg.get("REF"))] = bcs
            for fn in cond.findall("FUNCTION"):
                self.functions[fn.get("NAME")] = {e.get("VAR"): e.get("VALUE") for e in fn.findall("E")}

    def to_dict(self):
        """The parsed content as plain data (the reverse of from_dict)."""
        return dict(dim=self.dim, space=self.space,
                    vertices={str(k): list(map(float, v)) for k, v in self.vertices.items()},
                    edges={str(k): list(v) for k, v in self.edges.items()},
                    elements={str(k): [t, list(v)] for k, (t, v) in self.elements.items()},
                    composites={str(k): [t, list(v)] for k, (t, v) in self.composites.items()},
                    domain=list(self.domain), expansions=self.expansions, parameters=self.parameters,
                    solverinfo=self.solverinfo, variables=self.variables,
                    boundary_regions={str(k): v for k, v in self.boundary_regions.items()},
                    boundary_conditions={str(k): {var: list(bc) for var, bc in v.items()}
                                         for k, v in self.boundary_conditions.items()},
                    functions=self.functions)

    @classmethod
    def from_dict(cls, d):
        s = cls.__new__(cls)
        s.dim, s.space = d["dim"], d["space"]
        s.vertices = {int(k): np.array(v) for k, v in d["vertices"].items()}
        s.edges = {int(k): tuple(v) for k, v in d["edges"].items()}
        s.elements = {int(k): (t, list(v)) for k, (t, v) in d["elements"].items()}
        s.composites = {int(k): (t, list(v)) for k, (t, v) in d["composites"].items()}
        s.domain = list(d["domain"])
        s.expansions, s.parameters = d["expansions"], dict(d["parameters"])
        s.solverinfo, s.variables = dict(d["solverinfo"]), list(d["variables"])
        s.boundary_regions = {int(k): list(v) for k, v in d["boundary_regions"].items()}
        s.boundary_conditions = {int(k): {var: tuple(bc) for var, bc in v.items()}
                                 for k, v in d["boundary_conditions"].items()}
        s.functions = d["functions"]
        return s

    def function(self, name, var="u"):
        return compile_expression(self.functions[name][var], self.parameters)

    def nummodes(self):
        ns = {e["nummodes"] for e in self.expansions}
        if len(ns) != 1:
            raise ValueError("one uniform expansion order is supported")
        if self.expansions[0]["type"] != "MODIFIED":
            raise ValueError("TYPE=MODIFIED expansions are supported")
        return ns.pop()

    def composite_edges(self, cid):
        kind, ids = self.composites[cid]
        if kind != "E":
            raise ValueError(f"composite {cid} is not an edge composite")
        return ids


def read_session(path):
    return Session(ET.parse(path).getroot())


class _Classes:
    """Union-find over ids (periodic identification)."""

    def __init__(self, n):
        self.p = list(range(n))

    def find(self, a):
        while self.p[a] != a:
            self.p[a] = self.p[self.p[a]]
            a = self.p[a]
        return a

    def union(self, a, b):
        a, b = self.find(a), self.find(b)
        if a != b:
            self.p[max(a, b)] = min(a, b)


class QuadSessionMesh:
    """A quadrilateral mesh from a session: coordinates, assembly with Dirichlet and
    periodic boundaries, Dirichlet data."""

    def __init__(self, session, var="u"):
        s = session
        if s.dim != 2:
            raise ValueError("QuadSessionMesh takes a 2-D session")
        elems = []
        for cid in s.domain:
            kind, ids = s.composites[cid]
            if kind != "Q":
                raise ValueError("only quadrilateral elements are supported")
            elems.extend(ids)
        self.session = s
        self.elem_ids = sorted(elems)
        self.vid = sorted(s.vertices)
        vindex = {v: i for i, v in enumerate(self.vid)}
        self.V = np.stack([s.vertices[v][:2] for v in self.vid])
        self.eid = sorted(s.edges)
        self.eindex = {e: i for i, e in enumerate(self.eid)}
        self.EDGES = np.array([[vindex[a] for a in s.edges[e]] for e in self.eid])
        self.edge_of_pair = {frozenset(p): i for i, p in enumerate(map(tuple, self.EDGES))}
        EV = []
        for q in self.elem_ids:
            tag, ed = s.elements[q]
            if tag != "Q":
                raise ValueError("only quadrilateral elements are supported")
            E4 = [set(self.EDGES[self.eindex[e]]) for e in ed]
            cyc = [(E4[0] & E4[3]).pop(), (E4[0] & E4[1]).pop(), (E4[1] & E4[2]).pop(), (E4[2] & E4[3]).pop()]
            P = self.V[cyc]
            area = 0.5 * sum(P[i, 0] * P[(i + 1) % 4, 1] - P[(i + 1) % 4, 0] * P[i, 1] for i in range(4))
            if area < 0:  # keep every element counter-clockwise (positive Jacobian)
                cyc = [cyc[0], cyc[3], cyc[2], cyc[1]]
            EV.append(cyc)
        self.EV = np.array(EV)
        self.E = len(self.EV)
        self.var = var
        self._classify(var)

    def _classify(self, var):
        """Dirichlet edges and periodic edge pairs from the boundary conditions."""
        s = self.session
        self.dirichlet_edges, self.periodic_pairs = set(), []
        done = set()
        for reg, bcs in s.boundary_conditions.items():
            kind, value = bcs.get(var, ("", ""))
            edges = [self.eindex[e] for cid in s.boundary_regions[reg] for e in s.composite_edges(cid)]
            if kind == "D":
                self.dirichlet_edges.update(edges)
            elif kind == "P":
                other = parse_id_list(value)[1][0]
                if (other, reg) in done:
                    continue
                done.add((reg, other))
                partner = [self.eindex[e] for cid in s.boundary_regions[other] for e in s.composite_edges(cid)]
                self.periodic_pairs.extend(self._match_translation(edges, partner))
            elif kind in ("N", "R"):
                raise ValueError("Neumann and Robin conditions are not supported by this reader")

    def _match_translation(self, A, B):
        """Pairs (a, b, same_direction) of edges of A and B mapped onto each other by one
        translation (the periodic regions' offset)."""
        ca = np.mean([self.V[self.EDGES[a]].mean(0) for a in A], axis=0)
        cb = np.mean([self.V[self.EDGES[b]].mean(0) for b in B], axis=0)
        shift = cb - ca
        pairs = []
        for a in A:
            pa = self.V[self.EDGES[a]] + shift
            best = None
            for b in B:
                pb = self.V[self.EDGES[b]]
                if np.allclose(pa, pb, atol=1e-9):
                    best = (a, b, True)
                elif np.allclose(pa, pb[::-1], atol=1e-9):
                    best = (a, b, False)
            if best is None:
                raise ValueError("periodic edges do not match by translation")
            pairs.append(best)
        return pairs

    def coords(self, Q):
        """Coordinates at the Q x Q GLL points, (2, E, Q*Q), point j*Q + i."""
        z = gll_points(Q)
        a, b = 0.5 * (1 - z), 0.5 * (1 + z)
        W = np.stack([np.outer(a, a), np.outer(a, b), np.outer(b, b), np.outer(b, a)], axis=0)
        X = np.einsum("vji,evc->ceji", W, self.V[self.EV])
        return X.reshape(2, self.E, Q * Q).copy()

    def assembly(self, n):
        """C0 numbering for n ModifiedA modes: vertex and edge dofs shared (periodic
        partners identified), an edge mode p >= 2 signed (-1)^p where the local direction
        opposes the edge class's direction, interior modes private; Dirichlet dofs first."""
        nv, ne = len(self.V), len(self.EDGES)
        vc = _Classes(nv)
        ec = _Classes(ne)
        for a, b, same in self.periodic_pairs:
            va, vb = self.EDGES[a], self.EDGES[b] if same else self.EDGES[b][::-1]
            vc.union(va[0], vb[0])
            vc.union(va[1], vb[1])
            ec.union(a, b)
        vdir = np.zeros(nv, dtype=bool)
        edir = np.zeros(ne, dtype=bool)
        for e in self.dirichlet_edges:
            edir[e] = True
            vdir[self.EDGES[e]] = True
        vrep = np.array([vc.find(v) for v in range(nv)])
        erep = np.array([ec.find(e) for e in range(ne)])
        for v in range(nv):  # a class is Dirichlet when any member is
            vdir[vrep[v]] |= vdir[v]
        for e in range(ne):
            edir[erep[e]] |= edir[e]
        vclasses = np.unique(vrep)
        eclasses = np.unique(erep)
        ni = max(n - 2, 0)
        # entity numbering before renumbering: vertex classes, edge classes (ni each), interiors
        vnum = {c: i for i, c in enumerate(vclasses)}
        enum = {c: i for i, c in enumerate(eclasses)}
        nV, nE = len(vclasses), len(eclasses)
        nglob = nV + nE * ni + self.E * ni * ni
        is_dir = np.zeros(nglob, dtype=bool)
        for c in vclasses:
            is_dir[vnum[c]] = vdir[c]
        for c in eclasses:
            is_dir[nV + enum[c] * ni: nV + (enum[c] + 1) * ni] = edir[c]
        order = np.concatenate([np.flatnonzero(is_dir), np.flatnonzero(~is_dir)])
        newid = np.empty(nglob, dtype=np.int64)
        newid[order] = np.arange(nglob)
        ndir = int(is_dir.sum())
        l2g = np.zeros((self.E, n, n), dtype=np.int64)
        sgn = np.ones((self.E, n, n))
        for (p, q, v) in ((0, 0, 0), (1, 0, 1), (1, 1, 2), (0, 1, 3)):
            l2g[:, q, p] = [vnum[vrep[x]] for x in self.EV[:, v]]
        if ni > 0:
            modes = np.arange(2, n)
            flip = np.where(modes % 2 == 1, -1.0, 1.0)
            for e in range(self.E):
                ev = self.EV[e]
                for (fixed, val, vs, ve) in (("q", 0, 0, 1), ("q", 1, 3, 2), ("p", 0, 0, 3), ("p", 1, 1, 2)):
                    a, b = ev[vs], ev[ve]
                    edge = self.edge_of_pair[frozenset((a, b))]
                    c = erep[edge]
                    # the class's direction: from its lower to its higher vertex class
                    forward = vrep[a] < vrep[b]
                    g = nV + enum[c] * ni + (modes - 2)
                    sg = np.ones(ni) if forward else flip
                    if fixed == "q":
                        l2g[e, val, 2:] = g
                        sgn[e, val, 2:] = sg
                    else:
                        l2g[e, 2:, val] = g
                        sgn[e, 2:, val] = sg
            base = nV + nE * ni + np.arange(self.E)[:, None, None] * ni * ni
            qq, pp = np.meshgrid(np.arange(ni), np.arange(ni), indexing="ij")
            l2g[:, 2:, 2:] = base + (qq * ni + pp)[None]
        self._vnum, self._enum, self._vrep, self._erep, self._newid, self._nV = vnum, enum, vrep, erep, newid, nV
        return AssemblyMap(newid[l2g].reshape(-1), sgn.reshape(-1), nglob, ndir)

    def dirichlet_coefficients(self, n, fn, amap=None):
        """Global coefficients of the Dirichlet dofs (ndir values) for the boundary
        function fn(x, y): on each Dirichlet edge, the boundary-constrained projection of
        fn (vertex modes take fn at the vertices; the edge modes the L2 projection of the
        rest, with n + 1 GLL points as the edge's quadrature). Call after assembly(n)."""
        amap = amap or self.assembly(n)
        Q = n + 1
        z = gll_points(Q)
        from .operators import basis_modA
        _, w, _, B, _ = basis_modA(n, Q)
        B = B.reshape(n, Q)
        out = np.full(amap.ndir, np.nan)
        ni = n - 2
        for edge in sorted(self.dirichlet_edges):
            a, b = self.EDGES[edge]
            xa, xb = self.V[a], self.V[b]
            pts = np.outer(0.5 * (1 - z), xa) + np.outer(0.5 * (1 + z), xb)
            fv = fn(pts[:, 0], pts[:, 1])
            ga = self._newid[self._vnum[self._vrep[a]]]
            gb = self._newid[self._vnum[self._vrep[b]]]
            out[ga], out[gb] = fv[0], fv[-1]
            if ni > 0:
                resid = fv - fv[0] * B[0] - fv[-1] * B[1]
                Bi = B[2:]
                M = (Bi * w) @ Bi.T
                rhs = (Bi * w) @ resid
                coef = np.linalg.solve(M, rhs)
                forward = self._vrep[a] < self._vrep[b]
                if not forward:  # the class runs from b to a: z -> -z flips odd modes
                    coef = coef * np.where(np.arange(2, n) % 2 == 1, -1.0, 1.0)
                c = self._erep[edge]
                g = self._newid[self._nV + self._enum[c] * ni + np.arange(ni)]
                out[g] = coef
        if np.any(np.isnan(out)):
            raise ValueError("some Dirichlet dofs lie on no Dirichlet edge")
        return out


class TriSessionMesh:
    """A straight-sided triangle mesh from a session, each element in the reference's own
    frame: vertex j is the vertex of edge j that edge j + 1 does not share (TriGeom.cpp:55-80,
    the edge cycle's start of edge j), so v0 = e0 ^ e2, v1 = e0 ^ e1, v2 = e1 ^ e2. Field
    files store each triangle's coefficients in that frame, so it is kept as it is; a
    clockwise triangle (negative Jacobian) is rejected, as the reference rejects it. Elements
    are numbered by sorted global id (``elem_ids``)."""

    def __init__(self, session):
        s = session
        if s.dim != 2:
            raise ValueError("TriSessionMesh takes a 2-D session")
        elems = []
        for cid in s.domain:
            kind, ids = s.composites[cid]
            if kind != "T":
                raise ValueError("only triangular elements are supported")
            elems.extend(ids)
        self.session = s
        self.elem_ids = sorted(elems)
        self.vid = sorted(s.vertices)
        vindex = {v: i for i, v in enumerate(self.vid)}
        self.V = np.stack([s.vertices[v][:2] for v in self.vid])
        EV = []
        for t in self.elem_ids:
            tag, ed = s.elements[t]
            if tag != "T":
                raise ValueError("only triangular elements are supported")
            e3 = [set(s.edges[e]) for e in ed]
            cyc = [(e3[0] & e3[2]).pop(), (e3[0] & e3[1]).pop(), (e3[1] & e3[2]).pop()]
            P = self.V[[vindex[v] for v in cyc]]
            area = 0.5 * ((P[1, 0] - P[0, 0]) * (P[2, 1] - P[0, 1]) - (P[2, 0] - P[0, 0]) * (P[1, 1] - P[0, 1]))
            if area <= 0:
                raise ValueError(f"triangle {t} is clockwise or degenerate in its edge order")
            EV.append([vindex[v] for v in cyc])
        self.EV = np.array(EV)
        self.E = len(self.EV)

    def coords(self, n):
        """Coordinates at the (n + 1) x n collapsed points of n-mode triangles (GLL x
        Gauss-Radau), shape (2, E, n (n + 1)), point j (n + 1) + i."""
        z0, z1 = gll_points(n + 1), radau_points(n)
        e0, e1 = np.meshgrid(z0, z1, indexing="xy")
        xi0 = 0.5 * (1.0 + e0) * (1.0 - e1) - 1.0
        W = np.stack([-0.5 * (xi0 + e1), 0.5 * (1.0 + xi0), 0.5 * (1.0 + e1)])
        return np.einsum("vji,evc->ceji", W, self.V[self.EV]).reshape(2, self.E, -1).copy()
