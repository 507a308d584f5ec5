"""Shared test helpers: running one case on several backends and comparing."""
from __future__ import annotations

import json
import os

import numpy as np

from weldformfem_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
HOLLOMON = dict(model=1, E=200e9, nu=0.3, rho=7850.0, sy0=300e6, hol_K=600e6, hol_m=0.2)
STAB = [0.3, 0.7, 0.2, 0.08, 0.15, 0.15, 0.8, 0.2, 0.05, 0.0]
# The reference checkout read by the CPU parity tests that need it: the
# WF_REFERENCE_ROOT environment variable, else a "reference" directory beside
# the repository (absent on machines without it; those tests skip).
REFERENCE_ROOT = os.environ.get("WF_REFERENCE_ROOT") or os.path.normpath(
    os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), os.pardir,
                 "reference"))


def golden_cases():
    """The cases of tests/golden/gen_golden.py, rebuilt without the reference."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("gen_golden", os.path.join(GOLDEN, "gen_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.cases()


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def kats():
    with open(os.path.join(GOLDEN, "validation_kats.json")) as f:
        return json.load(f)


def setup(dom, case, extra=None):
    """Applies a case to a backend; returns dt. `extra` as in gen_golden."""
    extra = extra or {}
    dt = W.apply(dom, case)
    if "stab" in extra:
        dom.set_stab(np.array(extra["stab"], float))
    if "av" in extra:
        dom.set_artif_visc(*extra["av"])
    if "jc" in extra:
        dom.set_johnson_cook(0, *extra["jc"])
    if "gmt" in extra:
        g = extra["gmt"]
        dom.set_gmt(0, g["c"], g["range"], g["T"])
    if "plheat" in extra:
        dom.set_plastic_heat_fraction(extra["plheat"])
    if "max_edot" in extra:
        dom.set_max_strain_rate(extra["max_edot"])
    if "die" in extra:
        die = extra["die"]
        xyz, tri = W.axis_plane_mesh(die["start"], die["end"], die["dens"], die["flip"])
        dom.set_contact_trimesh(xyz, tri, die["vel"], die["mu_s"], die["mu_d"], die["pf"])
        dom.set_end_time(die["end_t"])
    if "thermal" in extra:
        t = extra["thermal"]
        dom.set_thermal(True, t["T0"])
        dom.set_material_thermal(0, t["k"], t["cp"], t.get("exp", 0.0))
        if "hc" in t:
            dom.set_contact_heat(t["hc"], t["T_die"])
    if "die2" in extra:
        b = extra["die2"]
        xyz, tri = W.axis_plane_mesh(b["start"], b["end"], b["dens"], b["flip"])
        dom.add_contact_trimesh(xyz, tri, b["vel"])
    return dt


def rel_err(a, b):
    """max |a - b| / max |b| (0 when both vanish)."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    scale = np.max(np.abs(b)) if b.size else 0.0
    diff = np.max(np.abs(a - b)) if b.size else 0.0
    if scale == 0.0:
        return float(diff)
    return float(diff / scale)


STATE_FIELDS = [("node_vec", "x"), ("node_vec", "u"), ("node_vec", "v"), ("node_vec", "a"),
                ("node_vec", "fi"), ("node_scalar", "mass"), ("elem_scalar", "vol"),
                ("elem_scalar", "p"), ("elem_scalar", "pl_strain"), ("elem_tensor", "sigma"),
                ("elem_tensor", "tau"), ("elem_tensor", "eps")]


def compare_state(a, b, fields=STATE_FIELDS):
    """Relative errors of a against b over the standard state fields."""
    out = {}
    for kind, name in fields:
        out[name] = rel_err(getattr(a, kind)(name), getattr(b, kind)(name))
    return out


def parse_vtk(path):
    """Point and cell data blocks of a legacy ASCII VTK file: {(section, name):
    array}, section "point" or "cell", vectors as [n, 3], tensors as [n, 3, 3],
    scalars as [n]; also ("points", "POINTS") and ("cells", "CELLS")."""
    toks = open(path).read().split()
    out = {}
    i, section, count = 0, None, 0
    while i < len(toks):
        t = toks[i]
        if t == "POINTS":
            n = int(toks[i + 1])
            out[("points", "POINTS")] = np.array(toks[i + 3:i + 3 + 3 * n], float).reshape(n, 3)
            i += 3 + 3 * n
        elif t == "CELLS":
            n, items = int(toks[i + 1]), int(toks[i + 2])
            out[("cells", "CELLS")] = np.array(toks[i + 3:i + 3 + items], np.int64)
            i += 3 + items
        elif t == "CELL_TYPES":
            n = int(toks[i + 1])
            i += 2 + n
        elif t in ("POINT_DATA", "CELL_DATA"):
            section, count = ("point" if t == "POINT_DATA" else "cell"), int(toks[i + 1])
            i += 2
        elif t == "VECTORS":
            name = toks[i + 1]
            out[(section, name)] = np.array(toks[i + 3:i + 3 + 3 * count], float).reshape(-1, 3)
            i += 3 + 3 * count
        elif t == "TENSORS":
            name = toks[i + 1]
            out[(section, name)] = np.array(toks[i + 3:i + 3 + 9 * count],
                                            float).reshape(-1, 3, 3)
            i += 3 + 9 * count
        elif t == "SCALARS":
            name = toks[i + 1]
            j = i + 3 if toks[i + 3] == "LOOKUP_TABLE" else i + 4   # component count optional
            assert toks[j] == "LOOKUP_TABLE", toks[i:j + 2]
            out[(section, name)] = np.array(toks[j + 2:j + 2 + count], float)
            i = j + 2 + count
        else:
            i += 1
    return out
