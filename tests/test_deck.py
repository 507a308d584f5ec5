"""JSON deck and LS-DYNA keyword front-end (wf_deck_read / wf_deck_apply).

CPU: the deck object is checked against independent restatements of the
reference driver's rules (src/explicit/main.C): box numbering, the order of
the AddBCVelNode calls (velocity zones, then symmetry planes), the time step
cflFactor * min length / sqrt(K / rho) with the reference's 3-D length rule,
the material mapping, and the .k reader on fixed-column and comma-separated
cards. GPU: a deck run on the GPU agrees with the oracle set up from the same
deck (FP64, 1e-9), and the command-line driver writes its VTK series.
"""
import json
import os
import subprocess

import numpy as np
import pytest

import weldformfem_gb300 as wf
from oracle import orabind as O
from tests import helpers as H
from weldformfem_gb300 import build as B
from weldformfem_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI_SRC = os.path.join(ROOT, "weldformfem_gb300", "examples", "wf_deck_solve.cpp")
CLI_EXE = os.path.join(ROOT, "weldformfem_gb300", "_lib", "wf_deck_solve")
REF_INPUT = os.path.join(H.REFERENCE_ROOT, "examples", "input")

STEEL = {"type": "Bilinear", "const": [2.0e9], "density0": 7850.0, "youngsModulus": 200e9,
         "poissonsRatio": 0.3, "yieldStress0": 300e6}


def box_deck(tmp_path, **over):
    deck = {
        "Configuration": {"simTime": 4.0e-6, "outTime": 2.0e-6, "cflFactor": 0.3,
                          "xSymm": True, "ySymm": True, "zSymm": True, "hourglass3D": 0.1},
        "Materials": [dict(STEEL)],
        "DomainBlocks": [{"type": "Box", "dim": [0.004, 0.004, 0.005], "start": [0.0, 0.0, 0.0],
                          "elemLength": 0.001}],
        "BoundaryConditions": [{"start": [-1.0, -1.0, 0.0045], "end": [1.0, 1.0, 1.0],
                                "value": [0.0, 0.0, -2.0]}],
    }
    for k, v in over.items():
        deck[k] = v
    p = tmp_path / "deck.json"
    p.write_text(json.dumps(deck, indent=1))
    return str(p), deck


def write_k(path, x, elnod, comma=False, offset=1):
    """Keyword file: node ids offset..., elements with degenerate tets padded to 8."""
    lines = ["$# test mesh", "*KEYWORD", "*NODE"]
    for n, p in enumerate(x):
        if comma:
            lines.append(f"{n + offset},{float(p[0])!r},{float(p[1])!r},{float(p[2])!r},0,0")
        else:
            lines.append(f"{n + offset:8d}{p[0]:16.9f}{p[1]:16.9f}{p[2]:16.9f}{0:8d}{0:8d}")
    lines += ["*PART", "part", "         1         0         0", "*ELEMENT_SOLID",
              "$#   eid     pid      n1      n2      n3      n4      n5      n6      n7      n8"]
    for e, row in enumerate(elnod):
        ids = [int(v) + offset for v in row]
        if len(ids) == 4:
            ids += [ids[3]] * 4
        if comma:
            lines.append(",".join(str(v) for v in [e + 1, 1] + ids))
        else:
            lines.append("".join(f"{v:8d}" for v in [e + 1, 1] + ids))
    lines.append("*END")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def parsed_coords(x, comma):
    """The coordinates a reader recovers from write_k's text."""
    if comma:
        return np.array(x, dtype=np.float64)
    return np.array([[float(f"{v:16.9f}") for v in p] for p in x])


def ref_min_length(x, el):
    pr = [(1, 0), (2, 0), (3, 0), (2, 1), (3, 1), (3, 2)]
    return min(np.linalg.norm(x[el[:, a]] - x[el[:, b]], axis=1).min() for a, b in pr)


def expected_bcs(x, zones, sym, symtol=1e-4):
    node, dim, val = [], [], []
    for st, en, v in zones:
        inside = np.all((x >= np.array(st)) & (x <= np.array(en)), axis=1)
        for a in np.nonzero(inside)[0]:
            for d in range(3):
                node.append(a)
                dim.append(d)
                val.append(v[d])
    for a in range(x.shape[0]):
        for d in range(3):
            if sym[d] and x[a, d] < symtol:
                node.append(a)
                dim.append(d)
                val.append(0.0)
    return np.array(node), np.array(dim), np.array(val)


# ---- CPU -------------------------------------------------------------------------
def test_box_deck_mesh_bcs_dt(tmp_path):
    p, deck = box_deck(tmp_path)
    k = wf.Deck(p)
    x, el = k.mesh()
    o = O.OracleDomain()
    o.add_box((0.004, 0.004, 0.005), 0.0005)
    np.testing.assert_array_equal(x, o.node_vec("x"))
    np.testing.assert_array_equal(el, o.conn()[0])
    bc = deck["BoundaryConditions"][0]
    node, dim, val = expected_bcs(x, [(bc["start"], bc["end"], bc["value"])], (True, True, True))
    kn, kd, kv = k.bcs()
    np.testing.assert_array_equal(kn, node)
    np.testing.assert_array_equal(kd, dim)
    np.testing.assert_array_equal(kv, val)
    i = k.info
    assert i["zone_nodes"] == 25 and i["n_zones"] == 1 and i["n_bc"] == node.size
    K = 200e9 / (3 * (1 - 2 * 0.3))
    assert i["min_length"] == ref_min_length(x, el)
    assert i["dt"] == 0.3 * i["min_length"] / np.sqrt(K / 7850.0)
    assert i["end_time"] == 4.0e-6 and i["out_time"] == 2.0e-6 and i["hourglass"] == 0.1
    m = i["material"]
    assert m["model"] == 0 and m["H"] == 200e9 * 2e9 / (200e9 - 2e9) and m["sy0"] == 300e6


def test_hollomon_stab_and_zone_ids(tmp_path):
    mat = dict(STEEL, type="Hollomon", const=[600e6, 0.2])
    p, _ = box_deck(tmp_path, Materials=[mat],
                    Stabilization={"alpha_free": 0.3, "J_min": 0.1, "log_factor": 0.8},
                    DomainZones=[{"id": 7, "start": [-1, -1, 0.0045], "end": [1, 1, 1]}],
                    BoundaryConditions=[{"zoneId": 7, "valueType": 0, "value": [0, 0, -1.0]}])
    k = wf.Deck(p)
    i = k.info
    assert i["material"]["model"] == 1 and i["material"]["hol_K"] == 600e6
    assert i["material"]["hol_m"] == 0.2
    assert i["has_stab"] == 1 and i["stab"][0] == 0.3 and i["stab"][9] == 0.1
    assert i["stab"][6] == 0.8 and i["stab"][7] == 0.0
    assert i["zone_nodes"] == 25


@pytest.mark.parametrize("comma", [False, True], ids=["fixed", "comma"])
@pytest.mark.parametrize("tet", [False, True], ids=["hex", "tet"])
def test_lsdyna_reader(tmp_path, comma, tet):
    c = W.config(1 if tet else 0, scale=(2, 3, 2))
    c.perturb = 0.1
    x, el = c.coords(), c.elnod()
    write_k(tmp_path / "m.k", x, el, comma=comma, offset=101)
    p, _ = box_deck(tmp_path, DomainBlocks=[{"type": "File", "fileName": "m.k"}])
    k = wf.Deck(p)
    kx, kel = k.mesh()
    assert k.info["npe"] == (4 if tet else 8)
    np.testing.assert_array_equal(kel, el)
    np.testing.assert_array_equal(kx, parsed_coords(x, comma))


def test_deck_errors(tmp_path):
    cases = [
        (dict(Configuration={"thermal": True}), 1),    # no thermalHeatCap
        (dict(Configuration={"domType": "AxiSymm"}), 5),
        (dict(RigidBodies=[{"type": "File", "fileName": "missing.nas"}]), 1),
        (dict(RigidBodies=[{"type": "Line", "dim": [1.0, 0.0, 0.0]}]), 5),
        (dict(RigidBodies=[{"type": "Plane"}, {"type": "Sphere"}]), 5),
        (dict(RigidBodies=[{"zoneId": 1}, {"type": "Plane"}]), 1),
        (dict(Materials=[dict(STEEL, type="NortonHoff")]), 5),
        (dict(Materials=[dict(STEEL, type="GMT")]), 1),      # strRange missing: e_min = 0
        (dict(DomainBlocks=[{"type": "File", "fileName": "missing.k"}]), 1),
        (dict(BoundaryConditions=[{"zoneId": 3, "value": [0, 0, 1.0]}]), 1),
    ]
    for over, status in cases:
        p, _ = box_deck(tmp_path, **over)
        with pytest.raises(wf.WfError) as e:
            wf.Deck(p)
        assert e.value.status == status, over
    bad = tmp_path / "bad.json"
    bad.write_text('{\n "Configuration": {"simTime": 1e-5,, }\n}')
    with pytest.raises(wf.WfError) as e:
        wf.Deck(str(bad))
    assert e.value.status == 1 and "line 2" in str(e.value)
    (tmp_path / "u.k").write_text("*NODE\n1,0,0,0\n*ELEMENT_SOLID\n1,1,1,2,3,4,4,4,4,4\n")
    p, _ = box_deck(tmp_path, DomainBlocks=[{"type": "File", "fileName": "u.k"}])
    with pytest.raises(wf.WfError) as e:
        wf.Deck(p)
    assert "unknown node 2" in str(e.value)


@pytest.mark.skipif(not os.path.isdir(REF_INPUT), reason="reference examples not present")
def test_reference_example_meshes():
    for name, npe in (("cyl_hex.k", 8), ("tetra_cyl.k", 4), ("test_1el/1_el.k", 4)):
        path = os.path.join(REF_INPUT, name)
        text = open(path).read().splitlines()
        sec, counts = None, {"NODE": 0, "ELEMENT_SOLID": 0}
        for ln in text:
            if ln.startswith("*"):
                sec = ln[1:].split()[0].upper()
            elif ln.strip() and not ln.startswith("$") and sec in counts:
                counts[sec] += 1
        deck = {"Materials": [STEEL], "DomainBlocks": [{"type": "File", "fileName": path}]}
        dp = os.path.join(os.environ.get("TMPDIR", "/tmp"), "wf_ref_mesh_deck.json")
        with open(dp, "w") as f:
            json.dump(deck, f)
        k = wf.Deck(dp)
        assert k.info["npe"] == npe
        assert k.info["nn"] == counts["NODE"] and k.info["ne"] == counts["ELEMENT_SOLID"]


CONTACT = dict(
    Configuration={"simTime": 2.0e-5, "outTime": 1.0e-5, "cflFactor": 0.3, "zSymm": True},
    RigidBodies=[{"type": "Plane", "zoneId": 10, "start": [-0.0005, -0.0005, 0.005 - 1e-6],
                  "dim": [0.0045, 0.0045, 0.0], "partSide": 3, "flipnormals": True}],
    Contact=[{"fricCoeffStatic": 0.2, "fricCoeffDynamic": 0.15, "penaltyFactor": 0.5}],
    BoundaryConditions=[{"zoneId": 10, "valueType": 0, "value": [0.0, 0.0, -3.0]},
                        {"zoneId": 2, "start": [-1, -1, -1], "end": [1, 1, 1e-4],
                         "value": [0.0, 0.0, 0.0]}])


def test_contact_deck(tmp_path):
    p, _ = box_deck(tmp_path, **CONTACT)
    k = wf.Deck(p)
    i = k.info
    assert i["contact"] == 1 and i["die_nodes"] == 16 and i["die_tris"] == 18
    assert i["die_vel"] == (0.0, 0.0, -3.0)
    assert (i["mu_static"], i["mu_dynamic"], i["penalty_factor"]) == (0.2, 0.15, 0.5)
    xyz, tri = k.die()
    ex, et = W.axis_plane_mesh([-0.0005, -0.0005, 0.005 - 1e-6], [0.0045, 0.0045, 0.0], 3, True)
    np.testing.assert_array_equal(xyz, ex)
    np.testing.assert_array_equal(tri, et)
    # contact decks apply no velocity zone to the part: only the zSymm plane
    x, _ = k.mesh()
    node, dim, val = expected_bcs(x, [], (False, False, True))
    np.testing.assert_array_equal(k.bcs()[0], node)
    assert i["zone_nodes"] == 0
    over = dict(CONTACT)
    over["Contact"] = [{}]
    p2, _ = box_deck(tmp_path, **over)
    assert wf.Deck(p2).info["penalty_factor"] == 0.1


def build_cli():
    lib = B.build()
    libdir = os.path.dirname(lib)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                           CLI_SRC, "-L", libdir, "-lwf_gb300", f"-Wl,-rpath,{libdir}",
                           "-o", CLI_EXE])
    return CLI_EXE


def test_cli_compiles():
    assert os.path.exists(build_cli())


def test_deck_drives_the_oracle(tmp_path):
    p, _ = box_deck(tmp_path)
    o = O.OracleDomain()
    wf.Deck(p).setup(o)
    o.init()
    n = o.solve()
    assert n > 10 and np.all(np.isfinite(o.node_vec("u")))


# ---- GPU -------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["box", "k_tet", "k_hex_hollomon", "box_gmt"])
def test_deck_on_gpu_matches_oracle(tmp_path, kind):
    if kind == "box":
        p, _ = box_deck(tmp_path)
    elif kind == "box_gmt":
        # the GMT law with its ranges, and a strain-rate cap below the rates
        gmt = dict(STEEL, type="GMT", const=[-2e-4, 0.2, 1200e6, -1.5e-3, 1e-4, 0.02, -1e-5, -2e-3],
                   strRange=[0.01, 2.0], strdotRange=[1e-2, 1e5], tempRange=[0.0, 1500.0])
        p, deck = box_deck(tmp_path, Materials=[gmt])
        deck["Configuration"]["maxStrRate"] = 50.0
        deck["Configuration"]["simTime"] = 2.0e-5
        deck["BoundaryConditions"][0]["value"] = [0.0, 0.0, -20.0]
        with open(p, "w") as f:
            json.dump(deck, f)
    else:
        tet = kind == "k_tet"
        c = W.config(1 if tet else 0, scale=(3, 3, 4))
        c.perturb = 0.1
        write_k(tmp_path / "m.k", c.coords(), c.elnod(), comma=tet)
        mats = [dict(STEEL, type="Hollomon", const=[600e6, 0.2])] if not tet else [dict(STEEL)]
        p, _ = box_deck(tmp_path, DomainBlocks=[{"type": "File", "fileName": "m.k"}],
                        Materials=mats)
    k = wf.Deck(p)
    d = wf.Domain(wf.WF_FP64)
    k.apply(d)
    d.init()
    n = d.solve()
    o = O.OracleDomain()
    k.setup(o)
    o.init()
    assert o.solve() == n
    assert H.rel_err(d.node_vec("u"), o.node_vec("u")) <= 1e-9
    assert H.rel_err(d.elem_tensor("sigma"), o.elem_tensor("sigma")) <= 1e-9
    # one-call loader: same result
    d2 = wf.Domain(wf.WF_FP64)
    d2.load_deck(p)
    d2.init()
    d2.solve()
    np.testing.assert_array_equal(d2.node_vec("u"), d.node_vec("u"))


@pytest.mark.gpu
def test_contact_deck_on_gpu_matches_oracle(tmp_path):
    p, _ = box_deck(tmp_path, **CONTACT)
    k = wf.Deck(p)
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
    assert H.rel_err(d.reaction(), o.reaction()) <= 1e-9


@pytest.mark.gpu
def test_load_lsdyna_and_vtk(tmp_path):
    c = W.config(0, scale=(2, 2, 3))
    write_k(tmp_path / "m.k", c.coords(), c.elnod())
    d = wf.Domain(wf.WF_FP64)
    d.load_lsdyna(str(tmp_path / "m.k"))
    np.testing.assert_array_equal(d.conn()[0], c.elnod())
    W.apply_options(d, c)
    d.init()
    d.run(5)
    out = tmp_path / "s.vtk"
    d.write_vtk(str(out))
    text = out.read_text().splitlines()
    assert text[0].startswith("# vtk DataFile") and f"POINTS {c.n_node} double" in text
    assert f"CELLS {c.n_elem} {9 * c.n_elem}" in text and "VECTORS DISP double" in text
    i = text.index("VECTORS DISP double")
    disp = np.array([[float(v) for v in ln.split()] for ln in text[i + 1:i + 1 + c.n_node]])
    np.testing.assert_allclose(disp, d.node_vec("u"), rtol=1e-8, atol=1e-18)


@pytest.mark.gpu
def test_cli_runs_deck(tmp_path):
    exe = build_cli()
    p, _ = box_deck(tmp_path)
    r = subprocess.run([exe, p, "--energy"], capture_output=True, text=True, check=True)
    summary = json.loads(r.stdout.strip().splitlines()[-1])
    k = wf.Deck(p)
    o = O.OracleDomain()
    k.setup(o)
    o.init()
    assert summary["steps"] == o.solve()
    res = json.loads((tmp_path / "deck_res.json").read_text())
    assert len(res["vtk_files"]) == summary["vtk_files"] >= 3
    assert all(os.path.exists(f["file"]) for f in res["vtk_files"])
    rows = (tmp_path / "deck_energy.csv").read_text().splitlines()
    assert rows[0] == "t,Eint,Ekin" and len(rows) == summary["steps"] + 1
    ek, ei = o.energies()
    last = [float(v) for v in rows[-1].split(",")]
    assert abs(last[1] - ei[-1]) <= 1e-6 * abs(ei[-1]) and abs(last[2] - ek[-1]) <= 1e-6 * abs(ek[-1])
