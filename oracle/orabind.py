"""ctypes binding to the C restatement oracle (oracle/_build/libwforacle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, always as the checker / baseline, never as
the thing measured or shipped. The method names match the product's Python
mirror (weldformfem_gb300.Domain) so one case description drives both.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libwforacle.so")
SRC = os.path.join(HERE, "wf_oracle.c")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_lib = None


class WfoMaterial(C.Structure):
    _fields_ = [("model", C.c_int), ("E", C.c_double), ("nu", C.c_double),
                ("rho", C.c_double), ("sy0", C.c_double), ("H", C.c_double),
                ("hol_K", C.c_double), ("hol_m", C.c_double)]


def build(force: bool = False) -> str:
    """Compiles the oracle with gcc (-ffp-contract=off keeps it bit-faithful)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC)):
        return LIB_PATH
    cmd = ["gcc", "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           SRC, "-o", LIB_PATH + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    i64 = C.c_int64
    sig = {
        "wfo_create": ([], vp),
        "wfo_destroy": ([vp], None),
        "wfo_set_threads": ([vp, C.c_int], None),
        "wfo_add_box_length": ([vp, _dp, _dp, C.c_double, C.c_int], C.c_int),
        "wfo_set_mesh": ([vp, i64, i64, C.c_int, _dp, _ip], C.c_int),
        "wfo_set_nodes": ([vp, _dp], C.c_int),
        "wfo_sizes": ([vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(C.c_int), C.POINTER(i64)], None),
        "wfo_get_connectivity": ([vp, _ip, _ip, _ip, _ip, _ip], None),
        "wfo_set_materials": ([vp, C.c_int, C.POINTER(WfoMaterial)], C.c_int),
        "wfo_set_elem_materials": ([vp, _ip], C.c_int),
        "wfo_set_johnson_cook": ([vp, C.c_int] + [C.c_double] * 8, C.c_int),
        "wfo_set_gmt": ([vp, C.c_int, _dp, _dp, C.c_double], C.c_int),
        "wfo_add_bc_vel_node": ([vp, i64, C.c_int, C.c_double], C.c_int),
        "wfo_allocate_bcs": ([vp], C.c_int),
        "wfo_set_reaction_nodes": ([vp, i64, _ip, C.c_int], C.c_int),
        "wfo_set_dt": ([vp, C.c_double], None),
        "wfo_set_end_time": ([vp, C.c_double], None),
        "wfo_set_hourglass": ([vp, C.c_double], None),
        "wfo_set_press_algorithm": ([vp, C.c_int], None),
        "wfo_set_stab": ([vp, _dp], None),
        "wfo_set_artif_visc": ([vp, C.c_double, C.c_double], None),
        "wfo_set_plastic_heat_fraction": ([vp, C.c_double], None),
        "wfo_set_max_strain_rate": ([vp, C.c_double], None),
        "wfo_set_mass_mode": ([vp, C.c_int], None),
        "wfo_set_contact_plane": ([vp, C.c_double, C.c_double, C.c_double, C.c_double, _ip, i64], None),
        "wfo_init": ([vp], C.c_int),
        "wfo_run": ([vp, i64], C.c_int),
        "wfo_solve": ([vp], i64),
        "wfo_time": ([vp], C.c_double),
        "wfo_get_node_vec": ([vp, C.c_int, _dp], C.c_int),
        "wfo_set_thermal": ([vp, C.c_int, C.c_double], None),
        "wfo_set_material_thermal": ([vp, C.c_int, C.c_double, C.c_double, C.c_double], C.c_int),
        "wfo_set_contact_heat": ([vp, C.c_double, C.c_double], None),
        "wfo_get_node_scalar": ([vp, C.c_int, _dp], C.c_int),
        "wfo_get_elem_scalar": ([vp, C.c_int, _dp], C.c_int),
        "wfo_get_elem_tensor": ([vp, C.c_int, _dp], C.c_int),
        "wfo_get_derivs": ([vp, _dp], None),
        "wfo_get_elem_forces": ([vp, _dp, _dp], None),
        "wfo_get_reaction": ([vp, _dp, i64], i64),
        "wfo_get_energies": ([vp, _dp, _dp, i64], i64),
        "wfo_set_contact_trimesh": ([vp, i64, _dp, i64, _ip, _dp, C.c_double, C.c_double,
                                     C.c_double], None),
        "wfo_add_contact_trimesh": ([vp, i64, _dp, i64, _ip, _dp], C.c_int),
        "wfo_get_trimesh_nodes": ([vp, _dp, i64], i64),
        "wfo_get_surface": ([vp, _u8, _dp, _dp], i64),
        "wfo_step_begin": ([vp], None),
        "wfo_step_end": ([vp], None),
        "wfo_get_elem_forces_range": ([vp, i64, i64, _dp], C.c_int),
        "wfo_set_elem_forces_range": ([vp, i64, i64, _dp], C.c_int),
        "wfo_get_node_state_range": ([vp, i64, i64, _dp], C.c_int),
        "wfo_set_node_state_range": ([vp, i64, i64, _dp], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


NODE_VEC = {"x": 0, "v": 1, "a": 2, "u": 3, "prev_a": 4, "fi": 5, "u_dt": 6, "contforce": 7}
NODE_SCALAR = {"mass": 0, "voln": 1, "p_node": 2, "T": 3}
ELEM_SCALAR = {"vol": 0, "vol0": 1, "detJ": 2, "p": 3, "pl_strain": 4, "sigma_y": 5, "rho": 6}
ELEM_TENSOR = {"sigma": 0, "tau": 1, "eps": 2, "str_rate": 3, "rot_rate": 4}


class OracleDomain:
    """CPU oracle domain; same method names as the product's Python mirror."""

    def __init__(self, threads: int = 0):
        self.h = lib().wfo_create()
        if threads:
            lib().wfo_set_threads(self.h, int(threads))

    def close(self):
        if getattr(self, "h", None):
            lib().wfo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            raise ValueError(f"oracle {what} failed ({rc})")

    # mesh -------------------------------------------------------------
    def add_box(self, L, r, tritetra=False, origin=(0.0, 0.0, 0.0)):
        self._check(lib().wfo_add_box_length(self.h, np.array(origin, float), np.array(L, float),
                                             float(r), int(tritetra)), "AddBoxLength")

    def set_mesh(self, x, elnod):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        elnod = np.ascontiguousarray(elnod, dtype=np.int32)
        ne, npe = elnod.shape
        self._check(lib().wfo_set_mesh(self.h, x.size // 3, ne, npe, x, elnod.reshape(-1)),
                    "set_mesh")

    def sizes(self):
        nn, ne, tot = C.c_int64(), C.c_int64(), C.c_int64()
        npe = C.c_int()
        lib().wfo_sizes(self.h, C.byref(nn), C.byref(ne), C.byref(npe), C.byref(tot))
        return nn.value, ne.value, npe.value, tot.value

    @property
    def nn(self):
        return self.sizes()[0]

    @property
    def ne(self):
        return self.sizes()[1]

    @property
    def npe(self):
        return self.sizes()[2]

    def conn(self):
        nn, ne, npe, tot = self.sizes()
        elnod = np.zeros(ne * npe, np.int32)
        nodel = np.zeros(tot, np.int32)
        loc = np.zeros(tot, np.int32)
        off = np.zeros(nn, np.int32)
        cnt = np.zeros(nn, np.int32)
        lib().wfo_get_connectivity(self.h, elnod, nodel, loc, off, cnt)
        return elnod.reshape(ne, npe), nodel, loc, off, cnt

    def set_nodes(self, x):
        self._check(lib().wfo_set_nodes(self.h, np.ascontiguousarray(x, np.float64).reshape(-1)),
                    "set_nodes")

    # setup ------------------------------------------------------------
    def set_materials(self, mats, elem_ids=None):
        arr = (WfoMaterial * len(mats))()
        for i, m in enumerate(mats):
            arr[i] = WfoMaterial(int(m.get("model", 0)), float(m["E"]), float(m["nu"]),
                                 float(m["rho"]), float(m.get("sy0", 1e10)), float(m.get("H", 0.0)),
                                 float(m.get("hol_K", 1.0)), float(m.get("hol_m", 1.0)))
        self._check(lib().wfo_set_materials(self.h, len(mats), arr), "set_materials")
        if elem_ids is not None:
            self._check(lib().wfo_set_elem_materials(self.h, np.ascontiguousarray(elem_ids, np.int32)),
                        "set_elem_materials")

    def set_johnson_cook(self, mat, B, n, C, eps0, m, Tm, Tt, T=0.0):
        self._check(lib().wfo_set_johnson_cook(self.h, int(mat), float(B), float(n), float(C),
                                               float(eps0), float(m), float(Tm), float(Tt),
                                               float(T)), "set_johnson_cook")

    def set_gmt(self, mat, c, rng, T=0.0):
        """GMT law: c = (n1, n2, C1, C2, m1, m2, I1, I2), rng = (e_min, e_max,
        er_min, er_max, T_min, T_max), T the uniform element temperature."""
        self._check(lib().wfo_set_gmt(self.h, int(mat), np.ascontiguousarray(c, np.float64),
                                      np.ascontiguousarray(rng, np.float64), float(T)),
                    "set_gmt")

    def set_hourglass(self, coef):
        lib().wfo_set_hourglass(self.h, float(coef))

    def set_press_algorithm(self, alg):
        lib().wfo_set_press_algorithm(self.h, int(alg))

    def set_stab(self, s10):
        lib().wfo_set_stab(self.h, np.ascontiguousarray(s10, np.float64))

    def set_artif_visc(self, a, b):
        lib().wfo_set_artif_visc(self.h, float(a), float(b))

    def set_plastic_heat_fraction(self, f):
        lib().wfo_set_plastic_heat_fraction(self.h, float(f))

    def set_max_strain_rate(self, r):
        lib().wfo_set_max_strain_rate(self.h, float(r))

    def set_mass_mode(self, mode):
        lib().wfo_set_mass_mode(self.h, int(mode))

    def add_bcs(self, bcs):
        """bcs: (node, dim, value) triples, or a tuple of three arrays."""
        L = lib()
        if isinstance(bcs, tuple) and len(bcs) == 3 and hasattr(bcs[0], "__len__"):
            triples = zip(*bcs)
        else:
            triples = bcs
        for node, dim, val in triples:
            self._check(L.wfo_add_bc_vel_node(self.h, int(node), int(dim), float(val)), "AddBCVelNode")
        L.wfo_allocate_bcs(self.h)

    def set_reaction_nodes(self, nodes, dim=2):
        nodes = np.ascontiguousarray(nodes, np.int32)
        lib().wfo_set_reaction_nodes(self.h, nodes.size, nodes, int(dim))

    def set_contact_plane(self, z0, vz, kpen, mu, cand_nodes):
        cand = np.ascontiguousarray(cand_nodes, np.int32)
        lib().wfo_set_contact_plane(self.h, float(z0), float(vz), float(kpen), float(mu),
                                    cand, cand.size)

    def set_contact_trimesh(self, xyz, tri, vel, mu_static=0.0, mu_dynamic=0.0,
                            penalty_factor=0.1):
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1)
        tri = np.ascontiguousarray(tri, np.int32).reshape(-1)
        lib().wfo_set_contact_trimesh(self.h, xyz.size // 3, xyz, tri.size // 3, tri,
                                      np.ascontiguousarray(vel, np.float64), float(mu_static),
                                      float(mu_dynamic), float(penalty_factor))

    def add_contact_trimesh(self, xyz, tri, vel):
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1)
        tri = np.ascontiguousarray(tri, np.int32).reshape(-1)
        if lib().wfo_add_contact_trimesh(self.h, xyz.size // 3, xyz, tri.size // 3, tri,
                                         np.ascontiguousarray(vel, np.float64)) != 0:
            raise RuntimeError("add_contact_trimesh needs set_contact_trimesh first")

    def trimesh_nodes(self):
        n = lib().wfo_get_trimesh_nodes(self.h, np.zeros(3), 0)
        out = np.zeros(3 * max(n, 1))
        lib().wfo_get_trimesh_nodes(self.h, out, n)
        return out[:3 * n].reshape(-1, 3)

    def surface(self):
        nn = self.nn
        ext, area, nl = np.zeros(nn, np.uint8), np.zeros(nn), np.zeros(nn)
        lib().wfo_get_surface(self.h, ext, area, nl)
        return ext, area, nl

    def set_dt(self, dt):
        lib().wfo_set_dt(self.h, float(dt))

    def set_end_time(self, t):
        lib().wfo_set_end_time(self.h, float(t))

    # run --------------------------------------------------------------
    def init(self):
        self._check(lib().wfo_init(self.h), "init")

    def step(self, n=1):
        self._check(lib().wfo_run(self.h, int(n)), "run")

    def solve(self):
        return lib().wfo_solve(self.h)

    # step halves and halo data (slab decomposition) -------------------
    def step_begin(self):
        lib().wfo_step_begin(self.h)

    def step_end(self):
        lib().wfo_step_end(self.h)

    def halo_forces(self, e0, e1):
        """Element and hourglass forces of elements [e0, e1), flat."""
        out = np.zeros(2 * (e1 - e0) * self.npe * 3)
        self._check(lib().wfo_get_elem_forces_range(self.h, int(e0), int(e1), out), "elem forces")
        return out

    def set_halo_forces(self, e0, e1, data):
        self._check(lib().wfo_set_elem_forces_range(self.h, int(e0), int(e1),
                                              np.ascontiguousarray(data, np.float64)),
                    "set elem forces")

    def halo_nodes(self, n0, n1):
        """Node state of nodes [n0, n1), flat."""
        out = np.zeros(15 * (n1 - n0))
        self._check(lib().wfo_get_node_state_range(self.h, int(n0), int(n1), out), "node state")
        return out

    def set_halo_nodes(self, n0, n1, data):
        self._check(lib().wfo_set_node_state_range(self.h, int(n0), int(n1),
                                             np.ascontiguousarray(data, np.float64)),
                    "set node state")

    @property
    def time(self):
        return lib().wfo_time(self.h)

    # readback ---------------------------------------------------------
    def node_vec(self, name):
        out = np.zeros(self.nn * 3)
        lib().wfo_get_node_vec(self.h, NODE_VEC[name], out)
        return out.reshape(-1, 3)

    def set_thermal(self, on=True, T0=20.0):
        lib().wfo_set_thermal(self.h, int(bool(on)), float(T0))

    def set_material_thermal(self, mat, k_T, cp_T, exp_T=0.0):
        lib().wfo_set_material_thermal(self.h, int(mat), float(k_T), float(cp_T), float(exp_T))

    def set_contact_heat(self, heat_cond, T_die=20.0):
        lib().wfo_set_contact_heat(self.h, float(heat_cond), float(T_die))

    def node_scalar(self, name):
        out = np.zeros(self.nn)
        lib().wfo_get_node_scalar(self.h, NODE_SCALAR[name], out)
        return out

    def elem_scalar(self, name):
        out = np.zeros(self.ne)
        lib().wfo_get_elem_scalar(self.h, ELEM_SCALAR[name], out)
        return out

    def elem_tensor(self, name):
        out = np.zeros(self.ne * 6)
        lib().wfo_get_elem_tensor(self.h, ELEM_TENSOR[name], out)
        return out.reshape(-1, 6)

    def derivs(self):
        nn, ne, npe, _ = self.sizes()
        out = np.zeros(ne * 3 * npe)
        lib().wfo_get_derivs(self.h, out)
        return out.reshape(ne, 3, npe)

    def elem_forces(self):
        nn, ne, npe, _ = self.sizes()
        f = np.zeros(ne * npe * 3)
        fhg = np.zeros(ne * npe * 3)
        lib().wfo_get_elem_forces(self.h, f, fhg)
        return f.reshape(ne, npe, 3), fhg.reshape(ne, npe, 3)

    def energies(self):
        """(kinetic energy, accumulated internal energy) after each step."""
        n = lib().wfo_get_energies(self.h, np.zeros(1), np.zeros(1), 0)
        k, e = np.zeros(max(n, 1)), np.zeros(max(n, 1))
        lib().wfo_get_energies(self.h, k, e, n)
        return k[:n], e[:n]

    def reaction(self):
        n = lib().wfo_get_reaction(self.h, np.zeros(1), 0)
        out = np.zeros(max(n, 1))
        lib().wfo_get_reaction(self.h, out, n)
        return out[:n]
