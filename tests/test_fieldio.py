"""Field files (.fld) and snapshot sets: the reader / writer against the reference's own files,
ExtractDataToCoeffs with order changes, and ITHACA's snapshot loading evaluated on the GPU
and fed to the GPU POD, pinned to the reference's compiled BwdTrans and its Eigen BDCSVD.

The snapshot fixtures (tests/golden/oseen_*) come from the reference's 2-D ROM test case
(36 triangles, 11 modes, fields u and v) by tests/golden/make_fld_fixtures.py.
"""
import glob
import json
import os
import xml.etree.ElementTree as ET
from collections import defaultdict

import numpy as np
import pytest

from cases import rel_err

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
SNAP_DIR = os.path.join(GOLD, "oseen_fld")
P = np.load(os.path.join(GOLD, "oseen_pod.npz"))
SNAPS = [os.path.join(SNAP_DIR, f"snap{k}.fld") for k in P["sel"]]
N_MODES = 11
REF_CASE = os.path.join(os.environ.get("ITHACA_REFERENCE", "/root/reference"), "solvers",
                        "IncNavierStokesSolver", "Tests_ROM")
TOL_PHYS = 1e-12       # GPU BwdTrans of the snapshots vs the reference kernel, relative
TOL_SIGMA = 1e-10      # |sigma - sigma_BDCSVD| / sigma_1, all ten values
TOL_SUBSPACE = 1e-9    # Procrustes residual of the leading-subspace sketch


def session_mesh():
    from ithaca_gpu.session import Session, TriSessionMesh
    with open(os.path.join(GOLD, "oseen_session.json")) as f:
        s = Session.from_dict(json.load(f))
    return s, TriSessionMesh(s)


def subspace_residual(V, R, sketch):
    Gs = V.T @ R
    Pm, _, Qt = np.linalg.svd(sketch @ Gs.T)
    return np.linalg.norm(sketch - (Pm @ Qt) @ Gs) / np.linalg.norm(sketch)


# ---------------------------------------------------------------------------- CPU
def test_codec_round_trip(tmp_path):
    from ithaca_gpu import fieldio as fio
    rng = np.random.default_rng(5)
    tri_ids = [0, 1, 2, 3, 7, 9, 10]
    g1 = fio.FieldGroup(["u", "v"], "Triangle", ["Modified_A", "Modified_B"], [4, 4], tri_ids,
                        rng.standard_normal((2, 7 * 10)))
    nm = [(2, 2), (3, 3), (4, 2)]
    g2 = fio.FieldGroup(["u", "v"], "Quadrilateral", ["Modified_A", "Modified_A"], nm, [11, 12, 15],
                        rng.standard_normal((2, 4 + 9 + 8)), uniform=False)
    path = str(tmp_path / "f.fld")
    fio.write_fld(path, [g1, g2], {"Time": 0.5})
    groups, meta = fio.read_fld(path)
    assert meta["Time"] == "0.5"
    assert [g.shape for g in groups] == ["Triangle", "Quadrilateral"]
    assert groups[0].ids == tri_ids and groups[0].nummodes == [4, 4] and groups[0].uniform
    assert groups[1].nummodes == nm and not groups[1].uniform
    assert ET.parse(path).getroot().find("ELEMENTS").get("ID") == "0-3,7,9-10"
    for a, b in zip(groups, (g1, g2)):
        assert np.array_equal(a.data, b.data)


@pytest.mark.parametrize("nvals", [1, 2, 3, 5, 64, 1000])
def test_codec_padding(nvals):
    """Binary padded with zero bytes to a multiple of 3, so no '=' (CompressData.cpp:110-132)."""
    from ithaca_gpu import fieldio as fio
    x = np.random.default_rng(nvals).standard_normal(nvals)
    t = fio.encode(x)
    assert "=" not in t and len(t) % 4 == 0
    assert np.array_equal(fio.decode(t), x)


def test_ncoeffs_match_reference_counts():
    from ithaca_gpu import fieldio as fio
    assert fio.ncoeffs("Triangle", [11, 11]) == 66
    assert fio.ncoeffs("Quadrilateral", [3, 5]) == 15
    assert fio.ncoeffs("Hexahedron", [2, 3, 4]) == 24
    assert fio.ncoeffs("Tetrahedron", [4, 4, 4]) == 20
    assert fio.ncoeffs("Prism", [4, 4, 4]) == 40
    assert fio.ncoeffs("Pyramid", [4, 4, 4]) == 30


def test_extract_to_coeffs_order_change():
    """Modes both orders share are copied, the rest zero (TriExp.cpp:1091-1130)."""
    from ithaca_gpu import fieldio as fio
    rng = np.random.default_rng(7)
    src_modes = fio.modes("Triangle", [5, 5])
    data = rng.standard_normal((1, 3 * len(src_modes)))
    g = fio.FieldGroup(["u"], "Triangle", ["Modified_A", "Modified_B"], [5, 5], [4, 2, 9], data)
    same = fio.extract_to_coeffs([g], "u", [9, 4], "Triangle", [5, 5])
    assert np.array_equal(same[0], data[0, 30:45]) and np.array_equal(same[1], data[0, 0:15])
    for n in (3, 7):
        out = fio.extract_to_coeffs([g], "u", [2], "Triangle", [n, n])
        for j, m in enumerate(fio.modes("Triangle", [n, n])):
            want = data[0, 15 + src_modes.index(m)] if m in src_modes else 0.0
            assert out[0, j] == want
    with pytest.raises(ValueError):
        fio.extract_to_coeffs([g], "u", [1], "Triangle", [5, 5])


def test_snapshot_files_read():
    from ithaca_gpu import fieldio as fio
    for path in SNAPS:
        groups, meta = fio.read_fld(path)
        assert len(groups) == 1
        g = groups[0]
        assert g.fields == ["u", "v"] and g.shape == "Triangle" and g.nummodes == [11, 11]
        assert g.ids == list(range(36)) and g.data.shape == (2, 36 * 66)
        assert meta["NektarVersion"] and meta["SessionName0"]


def test_session_triangles():
    s, mesh = session_mesh()
    assert s.nummodes() == N_MODES and mesh.E == 36 and mesh.elem_ids == list(range(36))
    V = mesh.V[mesh.EV]
    area = 0.5 * ((V[:, 1, 0] - V[:, 0, 0]) * (V[:, 2, 1] - V[:, 0, 1])
                  - (V[:, 2, 0] - V[:, 0, 0]) * (V[:, 1, 1] - V[:, 0, 1]))
    assert np.all(area > 0)
    X = mesh.coords(N_MODES)
    assert X.shape == (2, 36, 132)


def test_snapshots_continuous_across_edges():
    """The loaded fields are C0 across every shared edge when evaluated from both sides:
    element frames, vertex order and coefficient placement all agree with the files'."""
    from ithaca_gpu import fieldio as fio
    from oracle import tri as otri
    s, mesh = session_mesh()
    edges = defaultdict(list)
    for e, vs in enumerate(mesh.EV):
        for a, b in ((0, 1), (1, 2), (2, 0)):
            edges[frozenset((vs[a], vs[b]))].append(e)
    t = np.linspace(0.05, 0.95, 7)

    def local(e, X):
        v0, v1, v2 = mesh.V[mesh.EV[e]]
        A = np.stack([0.5 * (v1 - v0), 0.5 * (v2 - v0)], axis=1)
        xi = np.linalg.solve(A, (X - 0.5 * (v1 + v2)).T).T
        return 2 * (1 + xi[:, 0]) / (1 - xi[:, 1]) - 1, xi[:, 1]

    for path in SNAPS[:3]:
        groups, _ = fio.read_fld(path)
        for name in ("u", "v"):
            c = fio.extract_to_coeffs(groups, name, mesh.elem_ids, "Triangle", [N_MODES, N_MODES])
            jump, scale = 0.0, 0.0
            for key, els in edges.items():
                if len(els) != 2:
                    continue
                a, b = sorted(key)
                X = np.outer(1 - t, mesh.V[a]) + np.outer(t, mesh.V[b])
                vals = [otri.modal_values(N_MODES, *local(e, X)) @ c[e] for e in els]
                jump = max(jump, np.abs(vals[0] - vals[1]).max())
                scale = max(scale, np.abs(vals[0]).max())
            assert jump < 1e-12 * scale, (path, name, jump)


def test_oracle_bwdtrans_matches_reference_fixture():
    from ithaca_gpu import fieldio as fio
    from oracle import tri as otri
    _, mesh = session_mesh()
    tb = otri.TriBasis(N_MODES)
    for j in range(2):
        groups, _ = fio.read_fld(SNAPS[j])
        for f, name in enumerate(("u", "v")):
            c = fio.extract_to_coeffs(groups, name, mesh.elem_ids, "Triangle", [N_MODES, N_MODES])
            assert rel_err(otri.bwdtrans(tb, c.reshape(-1)).reshape(-1), P["phys_ref"][j, f]) < 1e-13


def test_rb_size_rule():
    """The library's RBsize rule on the BDCSVD singular values gives the fixture's."""
    from ithaca_gpu import pod
    assert pod.rb_size(P["sigma"], 0.999999) == int(P["rb_size"])


@pytest.mark.skipif(not os.path.isdir(REF_CASE), reason="reference tree not present")
def test_codec_reproduces_reference_files():
    """Every field file of the reference's ROM tests decodes, and re-encodes to the same text."""
    from ithaca_gpu import fieldio as fio
    files = sorted(glob.glob(os.path.join(REF_CASE, "**", "*.fld"), recursive=True))
    assert len(files) > 100
    for path in files[::7]:
        groups, _ = fio.read_fld(path)
        root = ET.parse(path).getroot()
        els = list(root.iter("ELEMENTS"))
        assert len(els) == len(groups)
        for el, g in zip(els, groups):
            assert fio.encode(g.data.reshape(-1)) == "".join(el.text.split()), path


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_CASE, "..", "..", "..", "utilities")),
                    reason="reference tree not present")
def test_partitioned_directory():
    """A .fld directory (Info.xml + one file per partition, FieldIOXml.cpp:419-500)."""
    from ithaca_gpu import fieldio as fio
    d = os.path.join(REF_CASE, "..", "..", "..", "utilities", "FieldConvert", "Tests", "chan_interpfield_nparts.fld")
    groups, _ = fio.read_fld(d)
    ids = sorted(i for g in groups for i in g.ids)
    assert ids == list(range(25))


# ---------------------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def loaded():
    import torch
    from ithaca_gpu import fieldio as fio
    from ithaca_gpu.operators import Collection, Context, geom_factors
    ctx = Context(0)
    _, mesh = session_mesh()
    X = mesh.coords(N_MODES)
    jac, df = geom_factors(ctx, "tri", N_MODES + 1, X)
    coll = Collection(ctx, "tri", N_MODES, N_MODES + 1, mesh.E, jac, df, deformed=True)
    phys = fio.load_snapshots(coll, SNAPS, ["u", "v"], mesh.elem_ids)
    torch.cuda.synchronize()
    yield dict(ctx=ctx, coll=coll, phys=phys, mesh=mesh)
    coll.close()
    ctx.close()


@pytest.mark.gpu
def test_gpu_load_snapshots_matches_reference(loaded):
    phys = loaded["phys"].cpu().numpy()
    nq = 36 * 132
    assert phys.shape == (len(SNAPS), 2 * nq)
    for j in range(2):
        for f in range(2):
            assert rel_err(phys[j, f * nq:(f + 1) * nq], P["phys_ref"][j, f]) < TOL_PHYS
    norms = np.linalg.norm(phys.reshape(len(SNAPS), 2, nq), axis=2)
    assert np.max(np.abs(norms - P["phys_norm"]) / P["phys_norm"]) < TOL_PHYS


@pytest.mark.gpu
def test_gpu_pod_of_snapshots_matches_bdcsvd(loaded):
    from ithaca_gpu import pod
    phys = loaded["phys"]
    ns = phys.shape[0]
    V, sigma, r = pod.offline_device(loaded["ctx"], phys, ns)
    assert r == ns
    s1 = P["sigma"][0]
    assert np.max(np.abs(sigma - P["sigma"])) / s1 < TOL_SIGMA
    Vh = V.cpu().numpy().T   # (N, r)
    R = 2 * np.random.default_rng(41).random((Vh.shape[0], 8)) - 1
    nsk = P["sketch"].shape[0]
    assert subspace_residual(Vh[:, :nsk], R, P["sketch"]) < TOL_SUBSPACE
    assert np.abs(Vh.T @ Vh - np.eye(r)).max() < 1e-12
    S = phys.cpu().numpy().T
    assert np.linalg.norm(S - Vh @ (Vh.T @ S)) / np.linalg.norm(S) < 1e-12
    assert pod.rb_size(sigma, 0.999999) == int(P["rb_size"])
