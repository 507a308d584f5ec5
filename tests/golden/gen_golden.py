"""Generates the golden fixtures under tests/golden/ from the reference itself.

Runs the reference WeldFormFEM CPU code, compiled from its own sources into
oracle/_ref/libwfref.so (oracle/build_ref.sh), on small cases and stores the
results as .npz files; also extracts the known-answer values of the
reference's validation/ files into validation_kats.json. The fixtures travel
with the repository so that tests can pin the oracle where the reference
checkout is absent.

Usage: python tests/golden/gen_golden.py /path/to/reference [--vtk-only] [--only NAME ...]

--only regenerates the named step fixtures alone and keeps the other entries
of cases.json (and their .npz files) as they are.

The VTK fixtures (vtk_*.npz) hold the data blocks that the reference's own
VTKWriter prints for the state after a run (--vtk-only writes only those).
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refbind as R  # noqa: E402
from weldformfem_gb300 import workloads as W  # noqa: E402

HOLLOMON = dict(model=1, E=200e9, nu=0.3, rho=7850.0, sy0=300e6, hol_K=600e6, hol_m=0.2)
STAB = [0.3, 0.7, 0.2, 0.08, 0.15, 0.15, 0.8, 0.2, 0.05, 0.0]
# Johnson-Cook B, n, C, eps0_dot, m, T_melt, T_transition, T
JC = [400e6, 0.35, 0.02, 1.0, 1.0, 1500.0, 20.0, 300.0]
# GMT constants n1, n2, C1, C2, m1, m2, I1, I2, the e / edot / T ranges and the
# temperature: about 300 MPa at eps_p = 0.01 and a strain rate of 100 /s
GMT = dict(c=[-2e-4, 0.2, 1200e6, -1.5e-3, 1e-4, 0.02, -1e-5, -2e-3],
           range=[0.01, 2.0, 1e-2, 1e5, 0.0, 1500.0], T=300.0)
# a 2x2-cell plane of triangles just below the top face of the 3x3x4-cell
# tetrahedral block (top at z = 2 mm), normal -z, moving down at 5 m/s
DIE = dict(start=[-0.001, -0.001, 0.002 - 1e-5], end=[0.004, 0.004, 0.0], dens=2, flip=True,
           vel=[0.0, 0.0, -5.0], mu_s=0.1, mu_d=0.08, pf=0.1, end_t=2e-6)


# a second, fixed-velocity body: a plane 1e-5 above the bottom face (z = 0),
# normal +z, moving up at 2 m/s; the part keeps only its x/y symmetry planes
DIE_BOTTOM = dict(start=[-0.001, -0.001, 1e-5], end=[0.004, 0.004, 0.0], dens=3, flip=False,
                  vel=[0.0, 0.0, 2.0])


# thermal coupling: T0, conductivity, heat capacity, expansion coefficient and
# (with a die) the die's heat transfer coefficient and temperature
THERMAL_DIE = dict(T0=20.0, k=50.0, cp=460.0, exp=1.2e-5, hc=2.0e6, T_die=600.0)
THERMAL = dict(T0=25.0, k=45.0, cp=480.0, exp=1.0e-5)


def cases():
    """(name, Case, steps, mode, extra) with mode 'step' (harness loop) or 'verbatim'."""
    out = []
    c = W.config(0, scale=(4, 4, 4))
    out.append(("hex4_hg_linear", c, 300, "step", dict(linear=True)))
    c = W.config(1, scale=(3, 3, 4))
    out.append(("tet3x3x4_linear", c, 300, "step", dict(linear=True)))
    c = W.config(0, scale=(3, 3, 3))
    c.hg = 0.0
    c.materials = [dict(HOLLOMON)]
    out.append(("hex3_hollomon_verbatim", c, 400, "verbatim", {}))
    c = W.config(0, scale=(2, 2, 3))
    c.hg = 0.0
    c.tritetra = True
    c.materials = [dict(HOLLOMON)]
    out.append(("tet2x2x3_hollomon_verbatim", c, 400, "verbatim", {}))
    c = W.config(1, scale=(2, 3, 3))
    c.press_alg = 1
    c.materials = [dict(HOLLOMON)]
    # pressure algorithm 1 accumulates the element pressure across steps and
    # diverges within a few dozen steps (as in the reference): pin 12 steps
    out.append(("tet_anp_alg1", c, 12, "step", {}))
    c = W.config(0, scale=(3, 3, 4))
    c.perturb = 0.1
    c.seed = W.SEED_BASE + 7
    c.materials = [dict(HOLLOMON)]
    out.append(("hex_stab_av", c, 200, "step", dict(stab=STAB, av=(0.2, 0.1))))
    c = W.config(4, scale=(4, 4, 4))
    mats = []
    for i in range(8):
        m = dict(W.STEEL)
        m["E"] *= 0.9 + 0.03 * i
        m["sy0"] *= 0.8 + 0.05 * i
        m["H"] *= 0.7 + 0.1 * i
        mats.append(m)
    c.materials = mats
    out.append(("hex_octants_linear", c, 300, "step", dict(linear=True)))
    # rigid triangle-mesh die on perturbed tetrahedra (the reference's own
    # CalcContactForces; its 3-D surface search is the tetrahedron's)
    c = W.config(1, scale=(3, 3, 4))
    c.perturb = 0.1
    c.bc = "bottom_z"
    out.append(("tet_die_trimesh", c, 300, "step", dict(linear=True, die=DIE)))
    # two rigid bodies (TriMesh_d::AddMesh): only the contacts with body 0
    # (the top die) feed the reaction
    c = W.config(1, scale=(3, 3, 4))
    c.perturb = 0.1
    c.seed = W.SEED_BASE + 13
    c.bc = "sym_xy"
    out.append(("tet_two_dies", c, 300, "step", dict(linear=True, die=DIE, die2=DIE_BOTTOM)))
    # thermal coupling (ThermalCalcs, calcThermalExpansion, plastic heat, die
    # heat transfer) with the die, and with Hollomon through the reference's
    # own CalcStressStrain
    c = W.config(1, scale=(3, 3, 4))
    c.perturb = 0.1
    c.bc = "bottom_z"
    out.append(("tet_die_thermal", c, 300, "step",
                dict(linear=True, die=DIE, thermal=THERMAL_DIE)))
    c = W.config(1, scale=(2, 3, 3))
    c.perturb = 0.1
    c.seed = W.SEED_BASE + 17
    c.top_vz = -20.0
    c.materials = [dict(HOLLOMON)]
    out.append(("tet_hollomon_thermal", c, 300, "step", dict(thermal=THERMAL)))
    # Johnson-Cook through Material_::Init_JohnsonCook and the reference's own
    # CalcStressStrain (hexahedra: the reference reads the temperature T[e] of a
    # node-sized array by element index)
    c = W.config(0, scale=(3, 3, 4))
    c.perturb = 0.1
    c.seed = W.SEED_BASE + 9
    c.top_vz = -5.0
    c.materials = [dict(model=2, E=200e9, nu=0.3, rho=7850.0, sy0=250e6)]
    out.append(("hex_johnson_cook", c, 400, "step", dict(jc=JC)))
    # GMT through the reference's own CalcGMTYieldStress / CalcGMTTangentModulus
    # (the harness sets the Material_ fields those functions read)
    c = W.config(0, scale=(3, 3, 4))
    c.perturb = 0.1
    c.seed = W.SEED_BASE + 19
    c.top_vz = -5.0
    c.materials = [dict(model=3, E=200e9, nu=0.3, rho=7850.0, sy0=250e6)]
    out.append(("hex_gmt", c, 400, "step", dict(gmt=GMT)))
    # the strain-rate cap of the rate-dependent tangent (m_max_edot) below the
    # element rates, and the plastic heat fraction (m_plheatfraction) other
    # than 0.9, each through the reference's own CalcStressStrain
    c = W.config(0, scale=(3, 3, 4))
    c.perturb = 0.1
    c.seed = W.SEED_BASE + 9
    c.top_vz = -5.0
    c.materials = [dict(model=2, E=200e9, nu=0.3, rho=7850.0, sy0=250e6)]
    out.append(("hex_jc_rate_cap", c, 400, "step", dict(jc=JC, max_edot=50.0)))
    c = W.config(1, scale=(2, 3, 3))
    c.perturb = 0.1
    c.seed = W.SEED_BASE + 17
    c.top_vz = -20.0
    c.materials = [dict(HOLLOMON)]
    out.append(("tet_hollomon_heat_frac", c, 300, "step", dict(thermal=THERMAL, plheat=0.6)))
    return out


def setup_ref(d, case, extra):
    """Applies a case and its extra options to a reference domain; returns dt."""
    dt = W.apply(d, case)
    if extra.get("linear"):
        d.set_linear_hardening(True)
    if "stab" in extra:
        d.set_stab(np.array(extra["stab"], float))
    if "av" in extra:
        d.set_artif_visc(*extra["av"])
    if "jc" in extra:
        d.set_johnson_cook(0, *extra["jc"])
    if "gmt" in extra:
        g = extra["gmt"]
        d.set_gmt(0, g["c"], g["range"], g["T"])
    if "plheat" in extra:
        d.set_plastic_heat_fraction(extra["plheat"])
    if "max_edot" in extra:
        d.set_max_strain_rate(extra["max_edot"])
    if "die" in extra:
        die = extra["die"]
        xyz, tri = W.axis_plane_mesh(die["start"], die["end"], die["dens"], die["flip"])
        d.set_contact_trimesh(xyz, tri, die["vel"], die["mu_s"], die["mu_d"], die["pf"])
        d.set_end_time(die["end_t"])
    if "die2" in extra:
        b = extra["die2"]
        xyz, tri = W.axis_plane_mesh(b["start"], b["end"], b["dens"], b["flip"])
        d.add_contact_trimesh(xyz, tri, b["vel"])
    if "thermal" in extra:
        t = extra["thermal"]
        d.set_thermal(True, t["T0"])
        d.set_material_thermal(0, t["k"], t["cp"], t.get("exp", 0.0))
        if "hc" in t:
            d.set_contact_heat(t["hc"], t["T_die"])
    return dt


def run_case(name, case, steps, mode, extra):
    d = R.RefDomain()
    dt = setup_ref(d, case, extra)
    if mode == "verbatim":
        d.set_end_time(steps * dt)
        with tempfile.TemporaryDirectory() as td:
            d.solve_verbatim(td)
    else:
        d.init()
        d.step(steps)
    elnod, nodel, loc, off, cnt = d.conn()
    res = dict(
        dt=np.float64(dt), steps=np.int64(steps),
        elnod=elnod, nodel=nodel, nodel_loc=loc, nodel_offset=off, nodel_count=cnt,
        x=d.node_vec("x"), u=d.node_vec("u"), v=d.node_vec("v"), a=d.node_vec("a"),
        fi=d.node_vec("fi"), mass=d.node_scalar("mass"),
        vol=d.elem_scalar("vol"), p=d.elem_scalar("p"), pl_strain=d.elem_scalar("pl_strain"),
        sigma=d.elem_tensor("sigma"), tau=d.elem_tensor("tau"), eps=d.elem_tensor("eps"),
        p_node=d.node_scalar("p_node"),
    )
    if mode == "step":
        res["reaction"] = d.reaction()
        res["ekin"], res["eint"] = d.energies()
    if "thermal" in extra:
        res["T"] = d.node_scalar("T")
    if "die" in extra:
        res["contforce"] = d.contforce()
        res["die_nodes"] = d.trimesh_nodes()
        res["ext"], res["node_area"], res["nodlen"] = d.surface()
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **res)
    meta = dict(name=name, mode=mode, steps=steps, extra={k: list(v) if isinstance(v, tuple) else v
                                                           for k, v in extra.items()})
    return meta


def vtk_cases():
    """Cases whose state the reference's own VTKWriter writes (VTKWriter.C:238-664)."""
    c = W.config(0, scale=(4, 4, 4))
    out = [("vtk_hex4", c, 300, dict(linear=True))]
    c = W.config(1, scale=(3, 3, 4))
    c.perturb = 0.1
    c.bc = "bottom_z"
    out.append(("vtk_tet_die", c, 300, dict(linear=True, die=DIE)))
    return out


def run_vtk_case(name, case, steps, extra):
    """Runs the case on the reference (stepwise loop), writes the VTK file with
    the reference's VTKWriter and stores its data blocks as {section/name:
    values} in tests/golden/<name>.npz (the text file is parsed here, so the
    fixture holds exactly the numbers the reference printed)."""
    from tests import helpers as H

    d = R.RefDomain()
    setup_ref(d, case, extra)
    d.init()
    d.step(steps)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "ref.vtk")
        d.write_vtk(path)
        blocks = H.parse_vtk(path)
    res = {f"{sec}/{nm}": v for (sec, nm), v in blocks.items()}
    res["steps"] = np.int64(steps)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **res)
    return dict(name=name, steps=steps, extra={k: list(v) if isinstance(v, tuple) else v
                                               for k, v in extra.items()})


def parse_validation(ref_root):
    """Known-answer values of validation/1elem_3d_red_int_f_0.06.txt and
    validation/1step_red_int_cube3D_hf_c_0.06.txt (one 0.1 m hexahedron)."""
    txt = open(os.path.join(ref_root, "validation", "1elem_3d_red_int_f_0.06.txt")).read()

    def block(after, title, rows=8):
        i = txt.index(after)
        j = txt.index(title, i)
        lines = txt[j:].splitlines()[1:1 + rows]
        return [[float(v) for v in ln.split()] for ln in lines]

    kats = {
        "source": "validation/1elem_3d_red_int_f_0.06.txt, "
                  "validation/1step_red_int_cube3D_hf_c_0.06.txt",
        "hg006_disp": block("C++", "DISPLACEMENTS"),
        "hg006_vel": block("C++", "VELOCITIES"),
        "nohg_disp": block("NO HG", "DISPLACEMENTS"),
        "nohg_vel": block("NO HG", "VELOCITIES"),
    }
    t1 = open(os.path.join(ref_root, "validation", "1step_red_int_cube3D_hf_c_0.06.txt")).read()
    i = t1.index("INITIAL DERIVATIVE MATRIX")
    rows = t1[i:].splitlines()[1:4]
    kats["dHdxy_detJ"] = [[float(v) for v in r.split()] for r in rows]
    m = re.search(r"dt\s*=\s*([0-9.eE+-]+)", txt + t1)
    kats["dt"] = 0.8e-5 if m is None else float(m.group(1))
    kats["setup"] = dict(L=0.1, r=0.05, E=206e9, nu=0.3, rho=7850.0, dt=0.8e-5, t_end=1.0e-3,
                         hg=0.06)
    return kats


def main():
    if len(sys.argv) < 2:
        print(__doc__)
        sys.exit(2)
    ref_root = sys.argv[1]
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), ref_root])
    if "--only" in sys.argv:
        names = sys.argv[sys.argv.index("--only") + 1:]
        with open(os.path.join(HERE, "cases.json")) as f:
            old = {m["name"]: m for m in json.load(f)}
        metas = [run_case(*c) if c[0] in names else old[c[0]] for c in cases()]
        with open(os.path.join(HERE, "cases.json"), "w") as f:
            json.dump(metas, f, indent=1)
        print("wrote", len(names), "fixtures")
        return
    vmetas = [run_vtk_case(*c) for c in vtk_cases()]
    with open(os.path.join(HERE, "vtk_cases.json"), "w") as f:
        json.dump(vmetas, f, indent=1)
    if "--vtk-only" in sys.argv:
        print("wrote", len(vmetas), "VTK fixtures")
        return
    metas = [run_case(*c) for c in cases()]
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(metas, f, indent=1)
    with open(os.path.join(HERE, "validation_kats.json"), "w") as f:
        json.dump(parse_validation(ref_root), f, indent=1)
    print("wrote", len(metas), "fixtures")


if __name__ == "__main__":
    main()
