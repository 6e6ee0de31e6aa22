"""Nektar++ field files (.fld, XML) read and written in the reference's format.

LibUtilities/BasicUtils/FieldIOXml.cpp stores a field as one ``<NEKTAR>`` document holding a
``<Metadata>`` block and one ``<ELEMENTS>`` tag per group of same-shape, same-order
elements. Its attributes are FIELDS (comma list), SHAPE, BASIS (comma list per direction),
NUMMODESPERDIR ("UNIORDER:n0,n1[,n2]" for the group or "MIXORDER:" with one tuple per
element), ID (ranges "a-b" and single ids, comma separated), COMPRESSED="B64Z-LittleEndian"
and BITSIZE="64". The text is the base64 encoding (no '=' padding; the binary is padded with
zero bytes to a multiple of 3, CompressData.cpp:110-132) of the zlib stream of the
little-endian doubles; the doubles are the coefficients of field 0 for every element of the
group in ID order, then field 1, ... (FieldIOXml.cpp:1108-1170, the check
``size == datasize * nfields``).

This module is what lets ITHACA's snapshot sets (the solvers' .fld outputs) feed the GPU
POD: ``read_fld`` returns the groups with their coefficient arrays, ``snapshot_matrix``
stacks chosen fields of a list of files into the columns of a snapshot matrix.
"""
import base64
import os
import warnings
import xml.etree.ElementTree as ET
import zlib
from dataclasses import dataclass, field

import numpy as np

COMPRESS = "B64Z-LittleEndian"


def modes(shape, nm):
    """The (p[, q[, r]]) index of each coefficient of one element, in storage order: the
    StdRegions orderings of the eModified expansions (p fastest for the tensor shapes;
    triangle q fastest with q < n1 - p; tetrahedron r fastest with q < n1 - p,
    r < n2 - p - q; prism r < n2 - p; pyramid r < n2 - max(p, q))."""
    nm = [int(x) for x in nm]
    if shape == "Segment":
        return [(p,) for p in range(nm[0])]
    if shape == "Quadrilateral":
        return [(p, q) for q in range(nm[1]) for p in range(nm[0])]
    if shape == "Hexahedron":
        return [(p, q, r) for r in range(nm[2]) for q in range(nm[1]) for p in range(nm[0])]
    if shape == "Triangle":
        return [(p, q) for p in range(nm[0]) for q in range(nm[1] - p)]
    if shape == "Tetrahedron":
        return [(p, q, r) for p in range(nm[0]) for q in range(nm[1] - p) for r in range(nm[2] - p - q)]
    if shape == "Prism":
        return [(p, q, r) for p in range(nm[0]) for q in range(nm[1]) for r in range(nm[2] - p)]
    if shape == "Pyramid":
        return [(p, q, r) for p in range(nm[0]) for q in range(nm[1]) for r in range(nm[2] - max(p, q))]
    raise ValueError(f"unsupported shape: {shape}")


def ncoeffs(shape, nm):
    """Coefficients of one element (LibUtilities::GetNumberOfCoefficients)."""
    return len(modes(shape, nm))


def parse_ids(s):
    """'0-3,7,9-10' -> [0, 1, 2, 3, 7, 9, 10] (ParseUtils::GenerateSeqVector)."""
    out = []
    for part in s.replace(" ", "").split(","):
        if not part:
            continue
        if "-" in part:
            a, b = part.split("-")
            out.extend(range(int(a), int(b) + 1))
        else:
            out.append(int(part))
    return out


def format_ids(ids):
    """The inverse of parse_ids, ranges for consecutive runs."""
    ids = list(ids)
    parts, i = [], 0
    while i < len(ids):
        j = i
        while j + 1 < len(ids) and ids[j + 1] == ids[j] + 1:
            j += 1
        parts.append(str(ids[i]) if i == j else f"{ids[i]}-{ids[j]}")
        i = j + 1
    return ",".join(parts)


def decode(text):
    raw = base64.b64decode("".join(text.split()))
    d = zlib.decompressobj()
    data = d.decompress(raw)
    return np.frombuffer(data, dtype="<f8").astype(np.float64)


def encode(values):
    raw = zlib.compress(np.ascontiguousarray(values, dtype="<f8").tobytes())
    raw += b"\0" * ((-len(raw)) % 3)
    return base64.b64encode(raw).decode("ascii")


@dataclass
class FieldGroup:
    """One ELEMENTS tag: fields, shape, basis, modes per direction, element ids and the data
    as (nfields, sum of element coefficients)."""
    fields: list
    shape: str
    basis: list
    nummodes: list            # per direction (uniform) or per element list of tuples
    ids: list
    data: np.ndarray
    uniform: bool = True
    extra: dict = field(default_factory=dict)

    def element_sizes(self):
        if self.uniform:
            return [ncoeffs(self.shape, self.nummodes)] * len(self.ids)
        return [ncoeffs(self.shape, nm) for nm in self.nummodes]

    def field(self, name):
        return self.data[self.fields.index(name)]


def read_fld(path):
    """(groups, metadata) of a .fld file (one or several NEKTAR documents), or of a .fld
    directory written in parallel: its Info.xml lists the partition files in Partition (or the
    older MultipleFldFiles) tags (FieldIOXml.cpp:419-500), read here in that order."""
    if os.path.isdir(path):
        info = ET.parse(os.path.join(path, "Info.xml")).getroot()
        tags = info.findall("Partition") or info.findall("MultipleFldFiles")
        if not tags:
            raise ValueError(f"{path}/Info.xml has no Partition or MultipleFldFiles tag")
        groups, meta = [], {}
        for t in tags:
            g, m = read_fld(os.path.join(path, t.attrib["FileName"]))
            groups.extend(g)
            meta.update(m)
        return groups, meta
    root = ET.parse(path).getroot()
    docs = [root] if root.tag == "NEKTAR" else root.findall("NEKTAR")
    groups, meta = [], {}
    for doc in docs:
        md = doc.find("Metadata")
        if md is not None:
            for child in md.iter():
                if child is not md and child.text and child.text.strip():
                    meta[child.tag] = child.text.strip()
        for el in doc.findall("ELEMENTS"):
            a = el.attrib
            comp = a.get("COMPRESSED")
            if comp is not None and comp.upper() != COMPRESS.upper():
                # FieldIOXml.cpp:1147-1156 only warns and decodes base64 + zlib regardless.
                warnings.warn(f"compressed format {comp} is not {COMPRESS}")
            if a.get("BITSIZE", "64") != "64":
                raise ValueError("only 64-bit data is supported")
            fields = a["FIELDS"].split(",")
            basis = a["BASIS"].split(",")
            ids = parse_ids(a["ID"])
            kind, _, rest = a["NUMMODESPERDIR"].partition(":")
            nums = [int(x) for x in rest.split(",") if x]
            dim = len(basis)
            if kind == "UNIORDER":
                nm, uniform = nums[:dim], True
            elif kind == "MIXORDER":
                nm = [tuple(nums[i * dim:(i + 1) * dim]) for i in range(len(ids))]
                uniform = False
            else:
                raise ValueError(f"unknown NUMMODESPERDIR {kind}")
            flat = decode(el.text or "")
            g = FieldGroup(fields, a["SHAPE"], basis, nm, ids, None, uniform,
                           {k: v for k, v in a.items() if k not in ("FIELDS", "SHAPE", "BASIS", "ID",
                                                                    "NUMMODESPERDIR", "COMPRESSED", "BITSIZE")})
            per_field = sum(g.element_sizes())
            if flat.size != per_field * len(fields):
                raise ValueError(f"data length {flat.size} does not match the header ({per_field} x {len(fields)})")
            g.data = flat.reshape(len(fields), per_field)
            groups.append(g)
    return groups, meta


def write_fld(path, groups, metadata=None):
    root = ET.Element("NEKTAR")
    md = ET.SubElement(root, "Metadata")
    for k, v in (metadata or {}).items():
        ET.SubElement(md, k).text = str(v)
    for g in groups:
        if g.uniform:
            nmstr = "UNIORDER:" + ",".join(str(x) for x in g.nummodes)
        else:
            nmstr = "MIXORDER:" + ",".join(str(x) for nm in g.nummodes for x in nm)
        attrs = {"FIELDS": ",".join(g.fields), "SHAPE": g.shape, "BASIS": ",".join(g.basis),
                 "NUMMODESPERDIR": nmstr, "ID": format_ids(g.ids), "COMPRESSED": COMPRESS, "BITSIZE": "64"}
        attrs.update(g.extra)
        el = ET.SubElement(root, "ELEMENTS", attrs)
        el.text = encode(np.asarray(g.data, dtype=np.float64).reshape(-1))
    ET.ElementTree(root).write(path, encoding="utf-8", xml_declaration=True)


def snapshot_matrix(paths, fields):
    """Columns = the chosen fields of each file, concatenated over its groups in order."""
    cols = []
    layout = None
    for p in paths:
        groups, _ = read_fld(p)
        key = [(g.shape, tuple(g.ids), tuple(map(tuple, [g.nummodes])) if g.uniform else None) for g in groups]
        if layout is None:
            layout = key
        elif key != layout:
            raise ValueError(f"{p}: the element layout differs from the first snapshot")
        cols.append(np.concatenate([g.field(f) for f in fields for g in groups]))
    return np.stack(cols, axis=1)


def _map_modes(shape, nm_from, nm_to):
    """(source index, target index) of the modes both orders share: the reference copies
    those and zeroes the rest when a file's order differs from the expansion's
    (TriExp.cpp:1091-1130 and the other shapes' v_ExtractDataToCoeffs)."""
    src = {m: i for i, m in enumerate(modes(shape, nm_from))}
    pairs = [(src[m], j) for j, m in enumerate(modes(shape, nm_to)) if m in src]
    return np.array(pairs, dtype=np.int64).reshape(-1, 2)


def extract_to_coeffs(groups, name, elem_ids, shape, nm):
    """ExpList::ExtractDataToCoeffs (MultiRegions/ExpList.cpp:3450-3530) for one field and
    one same-shape, same-order expansion: an (E, ncoeffs) array whose row k holds the
    coefficients of the element with global id elem_ids[k]. Elements of the file that are
    not in elem_ids are skipped; an element of elem_ids that no group holds raises."""
    row = {int(g): k for k, g in enumerate(elem_ids)}
    nc = ncoeffs(shape, nm)
    out = np.zeros((len(elem_ids), nc))
    seen = np.zeros(len(elem_ids), dtype=bool)
    for g in groups:
        if name not in g.fields:
            continue
        if g.shape != shape:
            if any(i in row for i in g.ids):
                raise ValueError(f"element shape {g.shape} in the file, {shape} expected")
            continue
        data = g.field(name)
        offset = 0
        sizes = g.element_sizes()
        for k, eid in enumerate(g.ids):
            enm = g.nummodes if g.uniform else g.nummodes[k]
            if eid in row:
                r = row[eid]
                if list(enm) == list(nm):
                    out[r] = data[offset:offset + nc]
                else:
                    mp = _map_modes(shape, enm, nm)
                    out[r, mp[:, 1]] = data[offset + mp[:, 0]]
                seen[r] = True
            offset += sizes[k]
    if not seen.all():
        missing = [int(elem_ids[k]) for k in np.flatnonzero(~seen)[:5]]
        raise ValueError(f"field {name}: no data for elements {missing} ...")
    return out


def load_snapshots(coll, paths, fields, elem_ids):
    """ITHACA's load_snapshots (CoupledLinearNS_ROM.cpp:1208-1260): each file evaluated as
    SessionFunction::EvaluateFld does (SolverUtils/Core/SessionFunction.cpp:325-368: Import,
    ExtractDataToCoeffs, BwdTrans) for every name in ``fields``, on the GPU collection
    ``coll`` whose elements carry the global ids ``elem_ids``. Returns a CUDA tensor
    (nsnapshots, nfields * E * nq): row k is snapshot k with its fields one after the other,
    i.e. the column-major snapshot matrix with one snapshot per column. The coefficients go
    to the device in one copy; the BwdTrans runs there, one launch per field and snapshot."""
    import torch

    shape = {"tri": "Triangle", "quad": "Quadrilateral", "hex": "Hexahedron", "tet": "Tetrahedron",
             "prism": "Prism", "pyr": "Pyramid"}[coll.shape]
    nm = {"Triangle": [coll.n, coll.n], "Quadrilateral": [coll.n] * 2}.get(shape, [coll.n] * 3)
    nf, E, ns = len(fields), coll.E, len(paths)
    if coll.dtype != np.float64:
        raise ValueError("snapshots are evaluated by an FP64 collection")
    if len(elem_ids) != E:
        raise ValueError("elem_ids must name the collection's elements")
    host = np.empty((ns, nf, E, coll.nm))
    for k, path in enumerate(paths):
        groups, _ = read_fld(path)
        for f, name in enumerate(fields):
            host[k, f] = extract_to_coeffs(groups, name, elem_ids, shape, nm)
    dev = torch.from_numpy(host.reshape(ns * nf, E * coll.nm)).to(f"cuda:{coll.ctx.device}")
    phys = torch.empty((ns, nf * E * coll.nq), dtype=torch.float64, device=dev.device)
    for k in range(ns):
        for f in range(nf):
            coll.bwdtrans(dev[k * nf + f], phys[k, f * E * coll.nq:(f + 1) * E * coll.nq])
    return phys
