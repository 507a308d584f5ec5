"""Nastran die meshes (wf_read_nastran) and contact decks with two rigid bodies.

The reader and the die orientation are pinned bit-for-bit to the reference's
own NastranReader and TriMesh_d(NastranReader&, flipnormals, orientNormals,
orient_pt) where the reference harness is built (node coordinates and the
triangle connectivity after flipping and orienting), and checked everywhere
against an independent restatement of the field rules: fixed 8-column GRID
and CTRIA3 cards, Fortran D exponents, exponents without a letter ("1.5-3"),
node ids that are neither contiguous nor in order. The files are written by
this test. A deck with a File body and a Plane body is read on the CPU and,
on the GPU, run against the oracle set up from the same deck.
"""
import json
import os

import numpy as np
import pytest

import weldformfem_gb300 as wf
from oracle import orabind as O
from oracle import refbind as R
from tests import helpers as H

NEEDS_REF = pytest.mark.skipif(not R.available(), reason="reference harness not built")


def fmt_real(v, style):
    """One 8-column real field in one of the spellings Nastran files use."""
    if style == "fixed":
        s = f"{v:8.5f}"
    elif style == "implicit":          # 1.2345-3: the exponent letter left out
        m, e = f"{v:.{3 if v < 0 else 4}e}".split("e")
        s = f"{m}{int(e):+d}"
    elif style == "fortran":           # 2.000D-2
        m, e = f"{v:.{2 if v < 0 else 3}E}".split("E")
        s = f"{m}D{int(e):+d}"
    else:                              # explicit lower-case e
        s = f"{v:.2e}".replace("e-0", "e-").replace("e+0", "e+")
    assert len(s) <= 8, (v, style, s)
    return s.rjust(8)


def field_value(s):
    """The restated rule: D reads as E; no exponent letter -> E before the
    first sign past the first column."""
    s = s.replace("D", "E").replace("d", "E")
    if "E" not in s and "e" not in s:
        for k in range(1, len(s)):
            if s[k] in "+-":
                s = s[:k] + "E" + s[k:]
                break
    return float(s)


def write_nas(path, n_side=5, z=0.01, span=(-0.003, 0.006), seed=3):
    """A square plane die of n_side x n_side nodes at height z, node ids
    scattered and listed out of order, mixed real spellings."""
    rng = np.random.default_rng(seed)
    lin = np.round(np.linspace(span[0], span[1], n_side), 9)
    pts = np.array([(x, y, z) for y in lin for x in lin])
    ids = 7 + 3 * rng.permutation(len(pts))          # not contiguous, not ordered
    styles = ["fixed", "implicit", "fortran", "lower"]
    lines = ["NASTRAN bulk data written by a test", "BEGIN BULK", "$ Nodes"]
    text_vals = []
    for n, p in enumerate(pts):
        fs = [fmt_real(float(p[k]), styles[(n + k) % 4]) for k in range(3)]
        text_vals.append([field_value(f) for f in fs])
        lines.append(f"{'GRID':<8}{ids[n]:>8}{0:>8}" + "".join(fs))
    lines.append("$ Elements")
    eid = 1
    for j in range(n_side - 1):
        for i in range(n_side - 1):
            a, b = j * n_side + i, j * n_side + i + 1
            c, d = (j + 1) * n_side + i, (j + 1) * n_side + i + 1
            for t in ((a, b, d), (a, d, c)):
                lines.append(f"{'CTRIA3':<8}{eid:>8}{3:>8}" + "".join(f"{ids[v]:>8}" for v in t))
                eid += 1
    lines += ["PSHELL         3       1,0.1", "ENDDATA"]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    tris = []
    for j in range(n_side - 1):
        for i in range(n_side - 1):
            a, b = j * n_side + i, j * n_side + i + 1
            c, d = (j + 1) * n_side + i, (j + 1) * n_side + i + 1
            tris += [(a, b, d), (a, d, c)]
    return np.array(text_vals), np.array(tris, np.int32)


def normals(xyz, tri):
    n = np.cross(xyz[tri[:, 1]] - xyz[tri[:, 0]], xyz[tri[:, 2]] - xyz[tri[:, 0]])
    return n / np.linalg.norm(n, axis=1)[:, None]


ORIENT = [(False, None), (True, None), (False, (0.001, 0.001, -0.02)),
          (True, (0.001, 0.001, -0.02)), (False, (0.0, 0.002, 0.05)), (True, (0.0, 0.002, 0.05))]


# ---- CPU -------------------------------------------------------------------------
def test_reader_fields_and_connectivity(tmp_path):
    p = str(tmp_path / "die.nas")
    vals, tris = write_nas(p)
    xyz, tri = wf.read_nastran(p)
    np.testing.assert_array_equal(xyz, vals)
    np.testing.assert_array_equal(tri, tris)
    # spot checks of the spellings themselves
    assert field_value("1.2345-3") == 1.2345e-3 and field_value("-2.00D-2") == -0.02
    assert field_value("+.01") == 0.01 and field_value("-0.02000") == -0.02


@pytest.mark.parametrize("flip,pt", ORIENT)
def test_flip_and_orientation(tmp_path, flip, pt):
    p = str(tmp_path / "die.nas")
    vals, tris = write_nas(p)
    xyz, tri = wf.read_nastran(p, flip, pt)
    nz = normals(xyz, tri)[:, 2]
    if pt is None:
        assert np.all(nz > 0) if not flip else np.all(nz < 0)
    else:
        # normals face the orientation point, with or without flipnormals
        assert np.all(nz < 0) if pt[2] < 0.01 else np.all(nz > 0)


@NEEDS_REF
@pytest.mark.parametrize("flip,pt", ORIENT)
def test_reader_matches_reference(tmp_path, flip, pt):
    p = str(tmp_path / "die.nas")
    write_nas(p, n_side=7, seed=11)
    xyz, tri = wf.read_nastran(p, flip, pt)
    rx, rt = R.nastran_trimesh(p, flip, pt)
    np.testing.assert_array_equal(xyz, rx)
    np.testing.assert_array_equal(tri, rt)


def test_reader_errors(tmp_path):
    p = tmp_path / "bad.nas"
    p.write_text("GRID           1       0 0.00000 0.00000 0.00000\n"
                 "GRID           2       0 1.00000 0.00000 0.00000\n"
                 "GRID           3       0 0.00000 1.00000 0.00000\n"
                 "CTRIA3         1       3       1       2       9\n")
    with pytest.raises(wf.WfError, match="unknown node 9"):
        wf.read_nastran(str(p))
    p.write_text("GRID           1       0 0.00000\n")
    with pytest.raises(wf.WfError):
        wf.read_nastran(str(p))
    p.write_text("GRID           1       0 0.00000 0.00000 0.00000\n"
                 "CBAR           1       1       1       2\n")
    with pytest.raises(wf.WfError) as e:
        wf.read_nastran(str(p))
    assert e.value.status == wf.WF_ERR_UNSUPPORTED
    with pytest.raises(wf.WfError):
        wf.read_nastran(str(tmp_path / "missing.nas"))


STEEL = {"type": "Bilinear", "const": [2.0e9], "density0": 7850.0, "youngsModulus": 200e9,
         "poissonsRatio": 0.3, "yieldStress0": 300e6}


def two_body_deck(tmp_path, top="File", third=False, tet=False, thermal=False):
    """A 4 x 4 x 5 mm block (hexahedra, or tetrahedra) with x/y symmetry,
    pressed by a die (File: a Nastran plane, flipnormals, oriented toward the
    part; or Plane) moving down and a fixed Plane body under it."""
    write_nas(str(tmp_path / "top.nas"), n_side=6, z=0.005 - 1e-6, span=(-0.0005, 0.0045))
    top_body = ({"type": "File", "fileName": "top.nas", "zoneId": 10, "flipnormals": True}
                if top == "File" else
                {"type": "Plane", "zoneId": 10, "start": [-0.0005, -0.0005, 0.005 - 1e-6],
                 "dim": [0.0045, 0.0045, 0.0], "partSide": 5, "flipnormals": True})
    bodies = [top_body, {"type": "Plane", "zoneId": 1, "start": [-0.0005, -0.0005, 1e-6],
                         "dim": [0.0045, 0.0045, 0.0], "partSide": 4}]
    if third:
        bodies.append({"type": "Plane", "zoneId": 5, "start": [0, 0, 1], "dim": [1, 1, 0]})
    deck = {
        "Configuration": {"simTime": 2.0e-5, "outTime": 1.0e-5, "cflFactor": 0.3,
                          "xSymm": True, "ySymm": True},
        "Materials": [dict(STEEL)],
        "DomainBlocks": [{"type": "Box", "dim": [0.004, 0.004, 0.005], "start": [0, 0, 0],
                          "elemLength": 0.001, "elemType": "TriTet" if tet else "Hexa"}],
        "RigidBodies": bodies,
        "Contact": [{"fricCoeffStatic": 0.2, "fricCoeffDynamic": 0.15, "penaltyFactor": 0.5}],
        "BoundaryConditions": [{"zoneId": 10, "valueType": 0, "value": [0.0, 0.0, -3.0]},
                               {"zoneId": 1, "valueType": 0, "value": [0.0, 0.0, 0.0]},
                               {"zoneId": 5, "valueType": 0, "value": [1.0, 0.0, 0.0]}],
    }
    if thermal:
        # the reference's thermal contact decks: hot die, plastic heat
        deck["Configuration"]["thermal"] = True
        deck["InitialConditions"] = [{"Temp": 30.0}]
        deck["Materials"][0].update(thermalCond=50.0, thermalHeatCap=460.0, thermalExp=1.2e-5)
        deck["Contact"][0].update(heatConductance=True, heatCondCoeff=2.0e6, dieTemp=500.0)
    p = tmp_path / "two_body.json"
    p.write_text(json.dumps(deck, indent=1))
    return str(p)


def test_two_body_deck(tmp_path):
    k = wf.Deck(two_body_deck(tmp_path, third=True))
    i = k.info
    # the reference driver reads RigidBodies[0] and [1] only
    assert i["contact"] == 1 and i["rigid_bodies"] == 2
    x0, t0, v0 = k.body(0)
    x1, t1, v1 = k.body(1)
    assert i["die_vel"] == (0.0, 0.0, -3.0) and tuple(v0) == (0.0, 0.0, -3.0)
    assert tuple(v1) == (0.0, 0.0, 0.0)
    np.testing.assert_array_equal(k.die()[0], x0)
    # File body: oriented toward the part's centroid (below the die): normals -z
    part_centroid = k.mesh()[0].mean(axis=0)
    ex, et = wf.read_nastran(str(tmp_path / "top.nas"), True, part_centroid)
    np.testing.assert_array_equal(x0, ex)
    np.testing.assert_array_equal(t0, et)
    assert np.all(normals(x0, t0)[:, 2] < 0) and np.all(normals(x1, t1)[:, 2] > 0)
    assert x1.shape == (25, 3) and t1.shape == (32, 3)
    with pytest.raises(wf.WfError):
        k.body(2)


def test_two_body_deck_drives_the_oracle(tmp_path):
    k = wf.Deck(two_body_deck(tmp_path))
    o = O.OracleDomain()
    k.setup(o)
    o.init()
    o.solve()
    cf = o.node_vec("contforce")
    x = k.mesh()[0]
    assert cf[x[:, 2] > 0.0049, 2].min() < 0          # pushed down by the die
    assert cf[x[:, 2] < 1e-9, 2].max() > 0            # held up by the plate
    assert o.reaction().max() > 0


def test_thermal_deck(tmp_path):
    i = wf.Deck(two_body_deck(tmp_path, thermal=True)).info
    assert i["thermal"] == 1 and i["T0"] == 30.0
    assert (i["thermal_k"], i["thermal_cp"], i["thermal_exp"]) == (50.0, 460.0, 1.2e-5)
    assert (i["heat_cond"], i["die_temp"]) == (2.0e6, 500.0)
    assert wf.Deck(two_body_deck(tmp_path)).info["thermal"] == 0


@NEEDS_REF
@pytest.mark.parametrize("thermal", [False, True])
def test_two_plane_bodies_match_reference(tmp_path, thermal):
    """Two Plane bodies from a deck, oracle against the reference harness
    (tetrahedra: the reference's 3-D surface search is compiled for 4-node
    elements)."""
    k = wf.Deck(two_body_deck(tmp_path, top="Plane", tet=True, thermal=thermal))
    res = []
    for dom in (O.OracleDomain(), R.RefDomain()):
        k.setup(dom)
        if isinstance(dom, R.RefDomain):
            # the reference's Bilinear radial return leaves sigma_y fixed and
            # reads an unset tangent; the harness restates linear hardening
            dom.set_linear_hardening(True)
        dom.init()
        dom.step(150)
        res.append((dom.node_vec("u"), dom.reaction(), dom.trimesh_nodes(),
                    dom.node_scalar("T") if thermal else None))
    for a, b in zip(*res):
        np.testing.assert_array_equal(a, b)
    if thermal:
        assert res[0][3].max() > 30.0


# ---- GPU -------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("top,tet,thermal", [("File", False, False), ("Plane", True, False),
                                             ("File", True, True)])
def test_two_body_deck_on_gpu_matches_oracle(tmp_path, top, tet, thermal):
    k = wf.Deck(two_body_deck(tmp_path, top=top, tet=tet, thermal=thermal))
    d = wf.Domain(wf.WF_FP64)
    k.apply(d)
    d.init()
    n = d.solve()
    o = O.OracleDomain()
    k.setup(o)
    o.init()
    assert o.solve() == n
    assert o.reaction().max() > 0
    assert H.rel_err(d.node_vec("u"), o.node_vec("u")) <= 1e-9
    assert H.rel_err(d.node_vec("contforce"), o.node_vec("contforce")) <= 1e-9
    assert H.rel_err(d.reaction(), o.reaction()) <= 1e-9
    np.testing.assert_allclose(d.trimesh_nodes(), o.trimesh_nodes(), rtol=1e-12, atol=0)
    if thermal:
        assert H.rel_err(d.node_scalar("T"), o.node_scalar("T")) <= 1e-9
