"""Writes the snapshot-set fixtures from the reference's own 2-D ROM test case
(solvers/IncNavierStokesSolver/Tests_ROM/single_geometric_parameter): the session
ICOSAHOM2018_compare_RB_sparsePoly.xml (36 triangles, NUMMODES 11, fields u, v) and its
snapshot files xml_channel_narrowROM_{0..39}.fld, which the session's TestSnap1..40
functions name and ITHACA's load_snapshots evaluates.

  oseen_session.json      the parsed session (Session.to_dict)
  oseen_fld/snap{k}.fld   ten of the snapshots (k = 0, 4, ..., 36), fields u and v, rewritten
                          by ithaca_gpu.fieldio.write_fld; the data elements are byte-identical
                          to the reference's (the codec reproduces its base64 + zlib text,
                          checked below for all forty files)
  oseen_pod.npz
    sel           the snapshot numbers of the ten files
    phys_ref      the reference's compiled BwdTransTriKernel (oracle/_ref) on u and v of the
                  first two files: (2, 2, 36 * 132)
    phys_norm     2-norms of the reference BwdTrans of u and v for all ten files (10, 2)
    sigma         singular values of the 10-column snapshot matrix [u; v] at the quadrature
                  points, by the reference's Eigen 3.3.7 BDCSVD (CoupledLinearNS_ROM.cpp:3925)
    sketch        U^T R for the leading NSK singular vectors, R = 2 rng.random((N, 8)) - 1
                  (seed 41): a check of the leading POD subspace
    rb_size       RBsize of the ten singular values at the session's POD_tolerance
                  (CoupledLinearNS_ROM.cpp:3935-3944)
Run where the reference tree is present (after make -C oracle/ref):
    python tests/golden/make_fld_fixtures.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300")]

from ithaca_gpu import fieldio  # noqa: E402
from ithaca_gpu.session import TriSessionMesh, read_session  # noqa: E402

REF = os.environ.get("ITHACA_REFERENCE", "/root/reference")
CASE = os.path.join(REF, "solvers", "IncNavierStokesSolver", "Tests_ROM", "single_geometric_parameter")
SESSION = "ICOSAHOM2018_compare_RB_sparsePoly.xml"
SEL = list(range(0, 40, 4))
NSK = 6
FIELDS = ["u", "v"]


def snapshot_path(k):
    return os.path.join(CASE, f"xml_channel_narrowROM_{k}.fld")


def rb_size(sigma, tol):
    """RBsize of CoupledLinearNS_ROM.cpp:3935-3944: one more than the last index whose
    cumulative singular-value fraction is below the tolerance."""
    c = np.cumsum(sigma) / sigma.sum()
    r = 1
    for i in range(sigma.size):
        if c[i] < tol:
            r = i + 2
    return r


def main():
    import xml.etree.ElementTree as ET

    from oracle import eigenbind, refbind
    from oracle import tri as otri

    s = read_session(os.path.join(CASE, SESSION))
    mesh = TriSessionMesh(s)
    n = s.nummodes()
    with open(os.path.join(HERE, "oseen_session.json"), "w") as f:
        json.dump(s.to_dict(), f)

    # the codec against the reference's own files: decode, re-encode, same text
    for k in range(40):
        root = ET.parse(snapshot_path(k)).getroot()
        for el in root.iter("ELEMENTS"):
            assert fieldio.encode(fieldio.decode(el.text)) == "".join(el.text.split()), k

    out_dir = os.path.join(HERE, "oseen_fld")
    os.makedirs(out_dir, exist_ok=True)
    tb = otri.TriBasis(n)
    cols, norms, phys_ref = [], [], []
    for j, k in enumerate(SEL):
        groups, meta = fieldio.read_fld(snapshot_path(k))
        kept = []
        for g in groups:
            idx = [g.fields.index(f) for f in FIELDS]
            kept.append(fieldio.FieldGroup(FIELDS, g.shape, g.basis, g.nummodes, g.ids, g.data[idx],
                                           g.uniform, g.extra))
        fieldio.write_fld(os.path.join(out_dir, f"snap{k}.fld"), kept, meta)
        col, nrm = [], []
        for name in FIELDS:
            c = fieldio.extract_to_coeffs(groups, name, mesh.elem_ids, "Triangle", [n, n])
            ref = refbind.tri_bwdtrans(n, mesh.E, c.reshape(-1))
            orc = otri.bwdtrans(tb, c.reshape(-1)).reshape(-1)
            assert np.abs(orc - ref).max() <= 1e-13 * np.abs(ref).max(), name
            col.append(ref)
            nrm.append(np.linalg.norm(ref))
            if j < 2:
                phys_ref.append(ref)
        cols.append(np.concatenate(col))
        norms.append(nrm)
    S = np.stack(cols, axis=1)
    sigma, U = eigenbind.bdcsvd(S, NSK)
    R = 2 * np.random.default_rng(41).random((S.shape[0], 8)) - 1
    np.savez_compressed(os.path.join(HERE, "oseen_pod.npz"), sel=np.array(SEL),
                        phys_ref=np.array(phys_ref).reshape(2, 2, -1), phys_norm=np.array(norms),
                        sigma=sigma, sketch=U.T @ R,
                        rb_size=rb_size(sigma, s.parameters["POD_tolerance"]))
    print("oseen fixtures written; sigma / sigma_1 =", sigma / sigma[0])


if __name__ == "__main__":
    main()
