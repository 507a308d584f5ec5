"""ctypes binding to oracle/_ref/libwfref.so (the reference CPU code + harness).

TEST INFRASTRUCTURE ONLY: used by tests/ and by the golden-fixture generator
to run the reference WeldFormFEM CPU solver in-process. The product never
imports this module. The library exists only where oracle/build_ref.sh could
compile the reference sources (it needs the reference checkout).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libwfref.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is not None:
        return _lib
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    sig = {
        "wfr_create": ([], vp),
        "wfr_destroy": ([vp], None),
        "wfr_add_box": ([vp] + [C.c_double] * 7 + [C.c_int], None),
        "wfr_set_mesh": ([vp, C.c_int, C.c_int, C.c_int, _dp, _ip], None),
        "wfr_dim": ([vp], C.c_int),
        "wfr_npe": ([vp], C.c_int),
        "wfr_node_count": ([vp], C.c_int),
        "wfr_elem_count": ([vp], C.c_int),
        "wfr_get_conn": ([vp, _ip, _ip, _ip, _ip, _ip], None),
        "wfr_set_node": ([vp, C.c_int, C.c_double, C.c_double, C.c_double], None),
        "wfr_set_materials": ([vp, C.c_int, _dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp], None),
        "wfr_set_elem_materials": ([vp, _ip], None),
        "wfr_set_johnson_cook": ([vp, C.c_int] + [C.c_double] * 8, None),
        "wfr_set_gmt": ([vp, C.c_int, _dp, _dp, C.c_double], None),
        "wfr_set_linear_hardening": ([vp, C.c_int], None),
        "wfr_set_hourglass": ([vp, C.c_double], None),
        "wfr_set_press_algorithm": ([vp, C.c_int], None),
        "wfr_set_stab": ([vp, _dp], None),
        "wfr_set_artif_visc": ([vp, C.c_double, C.c_double], None),
        "wfr_set_plastic_heat_fraction": ([vp, C.c_double], None),
        "wfr_set_max_strain_rate": ([vp, C.c_double], None),
        "wfr_add_bc_vel_node": ([vp, C.c_int, C.c_int, C.c_double], None),
        "wfr_allocate_bcs": ([vp], None),
        "wfr_set_reaction_nodes": ([vp, C.c_int, _ip, C.c_int], None),
        "wfr_set_dt": ([vp, C.c_double], None),
        "wfr_set_end_time": ([vp, C.c_double], None),
        "wfr_set_nproc": ([vp, C.c_int], None),
        "wfr_init": ([vp], None),
        "wfr_step": ([vp, C.c_int], None),
        "wfr_time": ([vp], C.c_double),
        "wfr_solve_verbatim": ([vp], None),
        "wfr_get_node_vec": ([vp, C.c_int, _dp], C.c_int),
        "wfr_set_thermal": ([vp, C.c_int, C.c_double], None),
        "wfr_set_material_thermal": ([vp, C.c_int, C.c_double, C.c_double, C.c_double], None),
        "wfr_set_contact_heat": ([vp, C.c_double, C.c_double], None),
        "wfr_get_node_scalar": ([vp, C.c_int, _dp], C.c_int),
        "wfr_get_elem_scalar": ([vp, C.c_int, _dp], C.c_int),
        "wfr_get_elem_tensor": ([vp, C.c_int, _dp], C.c_int),
        "wfr_get_derivs": ([vp, _dp], None),
        "wfr_get_elem_forces": ([vp, _dp, _dp], None),
        "wfr_get_reaction": ([vp, _dp, C.c_int], C.c_int),
        "wfr_get_energies": ([vp, _dp, _dp, C.c_int], C.c_int),
        "wfr_set_trimesh": ([vp, C.c_int, _dp, C.c_int, _ip, _dp, C.c_double, C.c_double,
                             C.c_double], None),
        "wfr_add_trimesh": ([vp, C.c_int, _dp, C.c_int, _ip, _dp], None),
        "wfr_nastran_trimesh": ([C.c_char_p, C.c_int, C.c_int, _dp, _dp, C.c_int, _ip, C.c_int,
                                 C.POINTER(C.c_int)], C.c_int),
        "wfr_get_trimesh_nodes": ([vp, _dp, C.c_int], C.c_int),
        "wfr_get_surface": ([vp, _u8, _dp, _dp], C.c_int),
        "wfr_get_contforce": ([vp, _dp], C.c_int),
        "wfr_write_vtk": ([vp, C.c_char_p], None),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


class _Silence:
    """Redirects fd 1 (the reference prints a lot through cout/printf)."""

    def __enter__(self):
        import sys

        sys.stdout.flush()
        self.saved = os.dup(1)
        self.null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self.null, 1)
        return self

    def __exit__(self, *exc):
        C.CDLL(None).fflush(None)
        os.dup2(self.saved, 1)
        os.close(self.saved)
        os.close(self.null)


NODE_VEC = {"x": 0, "v": 1, "a": 2, "u": 3, "prev_a": 4, "fi": 5, "u_dt": 6}
NODE_SCALAR = {"mass": 0, "voln": 1, "p_node": 2, "T": 3}
ELEM_SCALAR = {"vol": 0, "vol0": 1, "detJ": 2, "p": 3, "pl_strain": 4, "sigma_y": 5, "rho": 6}
ELEM_TENSOR = {"sigma": 0, "tau": 1, "eps": 2, "str_rate": 3, "rot_rate": 4}


def nastran_trimesh(path, flip_normals=False, orient_point=None):
    """The reference's Nastran die (NastranReader + TriMesh_d constructor):
    (xyz[n, 3], tri[m, 3]); orient_point None disables orientNormals."""
    pt = np.zeros(3) if orient_point is None else np.asarray(orient_point, np.float64)
    nt = C.c_int()
    args = (os.fsencode(path), int(bool(flip_normals)), int(orient_point is not None), pt)
    with _Silence():
        nn = lib().wfr_nastran_trimesh(*args, np.zeros(3), 0, np.zeros(3, np.int32), 0,
                                       C.byref(nt))
        x = np.zeros(3 * max(nn, 1))
        t = np.zeros(3 * max(nt.value, 1), np.int32)
        lib().wfr_nastran_trimesh(*args, x, nn, t, nt.value, C.byref(nt))
    return x[: 3 * nn].reshape(-1, 3), t[: 3 * nt.value].reshape(-1, 3)


class RefDomain:
    """One reference Domain_d (subclass harness) driven through the C API."""

    def __init__(self):
        self.h = lib().wfr_create()

    def close(self):
        if self.h:
            lib().wfr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # mesh -------------------------------------------------------------
    def add_box(self, L, r, tritetra=False, origin=(0.0, 0.0, 0.0)):
        with _Silence():
            lib().wfr_add_box(self.h, *map(float, origin), *map(float, L), float(r), int(tritetra))

    def set_mesh(self, x, elnod):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        elnod = np.ascontiguousarray(elnod, dtype=np.int32)
        ne, npe = elnod.shape
        with _Silence():
            lib().wfr_set_mesh(self.h, x.size // 3, ne, npe, x, elnod.reshape(-1))

    @property
    def nn(self):
        return lib().wfr_node_count(self.h)

    @property
    def ne(self):
        return lib().wfr_elem_count(self.h)

    @property
    def npe(self):
        return lib().wfr_npe(self.h)

    def conn(self):
        ne, npe, nn = self.ne, self.npe, self.nn
        elnod = np.zeros(ne * npe, np.int32)
        nodel = np.zeros(ne * npe, np.int32)
        loc = np.zeros(ne * npe, np.int32)
        off = np.zeros(nn, np.int32)
        cnt = np.zeros(nn, np.int32)
        lib().wfr_get_conn(self.h, elnod, nodel, loc, off, cnt)
        return elnod.reshape(ne, npe), nodel, loc, off, cnt

    def set_nodes(self, x):
        x = np.asarray(x, dtype=np.float64).reshape(-1, 3)
        L = lib()
        for n in range(x.shape[0]):
            L.wfr_set_node(self.h, n, *x[n])

    # setup ------------------------------------------------------------
    def set_materials(self, mats, elem_ids=None):
        """mats: list of dicts with E, nu, rho, sy0, H, model, hol_K, hol_m."""
        k = len(mats)
        arr = lambda key, dflt=0.0: np.array([float(m.get(key, dflt)) for m in mats])
        model = np.array([int(m.get("model", 0)) for m in mats], np.int32)
        with _Silence():
            lib().wfr_set_materials(
                self.h, k, arr("E"), arr("nu"), arr("rho"), arr("sy0", 1e10), arr("H"),
                model, arr("hol_K", 1.0), arr("hol_m", 1.0))
        if elem_ids is not None:
            lib().wfr_set_elem_materials(self.h, np.ascontiguousarray(elem_ids, np.int32))

    def set_johnson_cook(self, mat, B, n, C, eps0, m, Tm, Tt, T=0.0):
        lib().wfr_set_johnson_cook(self.h, int(mat), float(B), float(n), float(C), float(eps0),
                                   float(m), float(Tm), float(Tt), float(T))

    def set_gmt(self, mat, c, rng, T=0.0):
        lib().wfr_set_gmt(self.h, int(mat), np.ascontiguousarray(c, np.float64),
                          np.ascontiguousarray(rng, np.float64), float(T))

    def set_linear_hardening(self, on=True):
        lib().wfr_set_linear_hardening(self.h, int(on))

    def set_hourglass(self, coef):
        lib().wfr_set_hourglass(self.h, float(coef))

    def set_press_algorithm(self, alg):
        lib().wfr_set_press_algorithm(self.h, int(alg))

    def set_stab(self, s10):
        lib().wfr_set_stab(self.h, np.ascontiguousarray(s10, np.float64))

    def set_artif_visc(self, a, b):
        lib().wfr_set_artif_visc(self.h, float(a), float(b))

    def set_plastic_heat_fraction(self, f):
        lib().wfr_set_plastic_heat_fraction(self.h, float(f))

    def set_max_strain_rate(self, r):
        lib().wfr_set_max_strain_rate(self.h, float(r))

    def add_bcs(self, bcs):
        L = lib()
        if isinstance(bcs, tuple) and len(bcs) == 3 and hasattr(bcs[0], "__len__"):
            bcs = list(zip(*bcs))
        for node, dim, val in bcs:
            L.wfr_add_bc_vel_node(self.h, int(node), int(dim), float(val))
        with _Silence():
            L.wfr_allocate_bcs(self.h)

    def set_reaction_nodes(self, nodes, dim=2):
        nodes = np.ascontiguousarray(nodes, np.int32)
        lib().wfr_set_reaction_nodes(self.h, nodes.size, nodes, int(dim))

    def set_contact_trimesh(self, xyz, tri, vel, mu_static=0.0, mu_dynamic=0.0,
                            penalty_factor=0.1):
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1)
        tri = np.ascontiguousarray(tri, np.int32).reshape(-1)
        lib().wfr_set_trimesh(self.h, xyz.size // 3, xyz, tri.size // 3, tri,
                              np.ascontiguousarray(vel, np.float64), float(mu_static),
                              float(mu_dynamic), float(penalty_factor))

    def add_contact_trimesh(self, xyz, tri, vel):
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1)
        tri = np.ascontiguousarray(tri, np.int32).reshape(-1)
        with _Silence():
            lib().wfr_add_trimesh(self.h, xyz.size // 3, xyz, tri.size // 3, tri,
                                  np.ascontiguousarray(vel, np.float64))

    def trimesh_nodes(self):
        n = lib().wfr_get_trimesh_nodes(self.h, np.zeros(3), 0)
        out = np.zeros(3 * max(n, 1))
        lib().wfr_get_trimesh_nodes(self.h, out, n)
        return out[:3 * n].reshape(-1, 3)

    def surface(self):
        nn = self.nn
        ext, area, nl = np.zeros(nn, np.uint8), np.zeros(nn), np.zeros(nn)
        lib().wfr_get_surface(self.h, ext, area, nl)
        return ext, area, nl

    def contforce(self):
        out = np.zeros(3 * self.nn)
        lib().wfr_get_contforce(self.h, out)
        return out.reshape(-1, 3)

    def set_dt(self, dt):
        lib().wfr_set_dt(self.h, float(dt))

    def set_end_time(self, t):
        lib().wfr_set_end_time(self.h, float(t))

    def set_nproc(self, n):
        lib().wfr_set_nproc(self.h, int(n))

    # run --------------------------------------------------------------
    def init(self):
        with _Silence():
            lib().wfr_init(self.h)

    def step(self, n=1):
        with _Silence():
            lib().wfr_step(self.h, int(n))

    def solve_verbatim(self, workdir):
        cwd = os.getcwd()
        os.makedirs(workdir, exist_ok=True)
        os.chdir(workdir)
        try:
            with _Silence():
                lib().wfr_solve_verbatim(self.h)
        finally:
            os.chdir(cwd)

    def write_vtk(self, path):
        """The reference's VTKWriter on the current state (writes `path`)."""
        with _Silence():
            lib().wfr_write_vtk(self.h, os.fsencode(path))

    # readback ---------------------------------------------------------
    def node_vec(self, name):
        out = np.zeros(self.nn * 3)
        lib().wfr_get_node_vec(self.h, NODE_VEC[name], out)
        return out.reshape(-1, 3)

    def set_thermal(self, on=True, T0=20.0):
        lib().wfr_set_thermal(self.h, int(bool(on)), float(T0))

    def set_material_thermal(self, mat, k_T, cp_T, exp_T=0.0):
        lib().wfr_set_material_thermal(self.h, int(mat), float(k_T), float(cp_T), float(exp_T))

    def set_contact_heat(self, heat_cond, T_die=20.0):
        lib().wfr_set_contact_heat(self.h, float(heat_cond), float(T_die))

    def node_scalar(self, name):
        out = np.zeros(self.nn)
        lib().wfr_get_node_scalar(self.h, NODE_SCALAR[name], out)
        return out

    def elem_scalar(self, name):
        out = np.zeros(self.ne)
        lib().wfr_get_elem_scalar(self.h, ELEM_SCALAR[name], out)
        return out

    def elem_tensor(self, name):
        out = np.zeros(self.ne * 6)
        lib().wfr_get_elem_tensor(self.h, ELEM_TENSOR[name], out)
        return out.reshape(-1, 6)

    def derivs(self):
        out = np.zeros(self.ne * 3 * self.npe)
        lib().wfr_get_derivs(self.h, out)
        return out.reshape(self.ne, 3, self.npe)

    def elem_forces(self):
        n = self.ne * self.npe * 3
        f = np.zeros(n)
        fhg = np.zeros(n)
        lib().wfr_get_elem_forces(self.h, f, fhg)
        return f.reshape(self.ne, self.npe, 3), fhg.reshape(self.ne, self.npe, 3)

    def energies(self):
        """(kinetic energy, accumulated internal energy) after each step."""
        n = lib().wfr_get_energies(self.h, np.zeros(1), np.zeros(1), 0)
        k, e = np.zeros(max(n, 1)), np.zeros(max(n, 1))
        lib().wfr_get_energies(self.h, k, e, n)
        return k[:n], e[:n]

    def reaction(self):
        n = lib().wfr_get_reaction(self.h, np.zeros(1), 0)
        out = np.zeros(max(n, 1))
        lib().wfr_get_reaction(self.h, out, n)
        return out[:n]
