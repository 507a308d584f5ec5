"""weldformfem_gb300: GB300-native explicit updated-Lagrangian step.

Python mirror of the C ABI in include/wf.h (the library is
weldformfem_gb300/_lib/libwf_gb300.so, built by weldformfem_gb300/build.py).
`Domain` exposes the reference's Domain_d vocabulary (AddBoxLength, setNode,
AssignMaterial, AddBCVelNode, AllocateBCs, SetDT, SolveChungHulbert, ...)
under Python names. There is no CPU fallback: constructing a Domain without
the CUDA library or without a GPU raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import workloads  # noqa: F401  (re-exported helper)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libwf_gb300.so")

WF_FP64, WF_MIXED = 0, 1
# wf_status codes (include/wf.h)
WF_OK, WF_ERR_ARG, WF_ERR_STATE, WF_ERR_CUDA, WF_ERR_NOMEM = 0, 1, 2, 3, 4
WF_ERR_UNSUPPORTED, WF_ERR_NONFINITE, WF_ERR_TIMEOUT = 5, 6, 7
STATUS = {0: "ok", 1: "invalid argument", 2: "call out of order", 3: "CUDA error",
          4: "out of memory", 5: "unsupported option", 6: "non-finite state",
          7: "device wait timed out"}

NODE_VEC = {"x": 0, "v": 1, "a": 2, "u": 3, "prev_a": 4, "fi": 5, "contforce": 7}
NODE_SCALAR = {"mass": 0, "voln": 1, "p_node": 2, "T": 3}
ELEM_SCALAR = {"vol": 0, "vol0": 1, "detJ": 2, "p": 3, "pl_strain": 4, "sigma_y": 5, "rho": 6}
ELEM_TENSOR = {"sigma": 0, "tau": 1, "eps": 2, "str_rate": 3, "rot_rate": 4}


class WfError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class WfMaterial(C.Structure):
    _fields_ = [("model", C.c_int32), ("E", C.c_double), ("nu", C.c_double),
                ("rho", C.c_double), ("sy0", C.c_double), ("H", C.c_double),
                ("hol_K", C.c_double), ("hol_m", C.c_double)]


class WfStab(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "alpha_free", "alpha_contact", "hg_coeff_free", "hg_coeff_contact", "av_coeff_div",
        "av_coeff_bulk", "log_factor", "pspg_scale", "p_pspg_bulkfac", "J_min")]


class WfDeckInfo(C.Structure):
    _fields_ = [("nn", C.c_int64), ("ne", C.c_int64), ("npe", C.c_int32),
                ("press_alg", C.c_int32), ("n_bc", C.c_int64), ("zone_nodes", C.c_int64),
                ("n_zones", C.c_int32), ("has_stab", C.c_int32), ("dt", C.c_double),
                ("end_time", C.c_double), ("out_time", C.c_double), ("cfl", C.c_double),
                ("min_length", C.c_double), ("sound_speed", C.c_double),
                ("hourglass", C.c_double), ("artif_visc", C.c_double * 2), ("stab", WfStab),
                ("material", WfMaterial), ("contact", C.c_int32), ("die_nodes", C.c_int32),
                ("die_tris", C.c_int32), ("die_vel", C.c_double * 3), ("mu_static", C.c_double),
                ("mu_dynamic", C.c_double), ("penalty_factor", C.c_double),
                ("johnson_cook", C.c_double * 8), ("rigid_bodies", C.c_int32),
                ("thermal", C.c_int32), ("T0", C.c_double), ("thermal_k", C.c_double),
                ("thermal_cp", C.c_double), ("thermal_exp", C.c_double),
                ("heat_cond", C.c_double), ("die_temp", C.c_double),
                ("gmt", C.c_double * 8), ("gmt_range", C.c_double * 6),
                ("plheat_frac", C.c_double), ("max_edot", C.c_double)]


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_lib = None

# name -> (argtypes); every function returns wf_status (int)
_SIGS = {
    "wf_domain_create": [C.POINTER(C.c_void_p)],
    "wf_domain_create_on_device": [C.POINTER(C.c_void_p), C.c_int],
    "wf_domain_destroy": [C.c_void_p],
    "wf_add_box_length": [C.c_void_p, _dp, _dp, C.c_double, C.c_int32, C.c_int32],
    "wf_set_mesh": [C.c_void_p, C.c_int64, C.c_int64, C.c_int32, _dp, _ip],
    "wf_set_node": [C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_double],
    "wf_set_nodes": [C.c_void_p, _dp],
    "wf_get_sizes": [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                     C.POINTER(C.c_int32), C.POINTER(C.c_int64)],
    "wf_get_connectivity": [C.c_void_p, _ip, _ip, _ip, _ip, _ip],
    "wf_set_density": [C.c_void_p, C.c_double],
    "wf_set_materials": [C.c_void_p, C.c_int32, C.POINTER(WfMaterial)],
    "wf_set_elem_materials": [C.c_void_p, _ip],
    "wf_add_bc_vel_node": [C.c_void_p, C.c_int64, C.c_int32, C.c_double],
    "wf_add_bc_vel_zone": [C.c_void_p, _dp, _dp, _dp, C.POINTER(C.c_int64)],
    "wf_add_bc_vel_nodes": [C.c_void_p, C.c_int64, _lp, _ip, _dp],
    "wf_set_specimens": [C.c_void_p, C.c_int32, _lp, _lp, _dp],
    "wf_get_specimen_reaction": [C.c_void_p, C.c_int32, _dp, C.c_int64, C.POINTER(C.c_int64)],
    "wf_allocate_bcs": [C.c_void_p],
    "wf_set_dt": [C.c_void_p, C.c_double],
    "wf_set_end_time": [C.c_void_p, C.c_double],
    "wf_set_precision": [C.c_void_p, C.c_int32],
    "wf_set_hourglass": [C.c_void_p, C.c_double],
    "wf_set_press_algorithm": [C.c_void_p, C.c_int32],
    "wf_set_stab": [C.c_void_p, C.POINTER(WfStab)],
    "wf_set_artif_visc": [C.c_void_p, C.c_double, C.c_double],
    "wf_set_plastic_heat_fraction": [C.c_void_p, C.c_double],
    "wf_set_max_strain_rate": [C.c_void_p, C.c_double],
    "wf_set_mass_mode": [C.c_void_p, C.c_int32],
    "wf_set_reaction_nodes": [C.c_void_p, C.c_int64, _ip, C.c_int32],
    "wf_set_contact_plane": [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double,
                             C.c_int64, _ip],
    "wf_init": [C.c_void_p],
    "wf_run": [C.c_void_p, C.c_int64],
    "wf_solve": [C.c_void_p, C.POINTER(C.c_int64)],
    "wf_get_time": [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)],
    "wf_sync": [C.c_void_p],
    "wf_min_edge_length": [C.c_void_p, C.POINTER(C.c_double)],
    "wf_get_node_field": [C.c_void_p, C.c_int32, _dp],
    "wf_get_node_scalar": [C.c_void_p, C.c_int32, _dp],
    "wf_get_elem_scalar": [C.c_void_p, C.c_int32, _dp],
    "wf_get_elem_tensor": [C.c_void_p, C.c_int32, _dp],
    "wf_get_disp": [C.c_void_p, _dp],
    "wf_get_vel": [C.c_void_p, _dp],
    "wf_get_pl_strain": [C.c_void_p, _dp],
    "wf_get_reaction_history": [C.c_void_p, _dp, C.c_int64, C.POINTER(C.c_int64)],
    "wf_set_node_state": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
    "wf_set_phase_timing": [C.c_void_p, C.c_int32],
    "wf_get_phase_times": [C.c_void_p, _dp, C.POINTER(C.c_int64), C.c_int32],
    "wf_get_launch_count": [C.c_void_p, C.POINTER(C.c_int64)],
    "wf_get_graph_launches": [C.c_void_p, C.POINTER(C.c_int64)],
    "wf_prepare_run": [C.c_void_p, C.c_int64],
    "wf_get_stream": [C.c_void_p, C.POINTER(C.c_void_p)],
    "wf_set_autotune": [C.c_void_p, C.c_int32],
    "wf_get_launch_config": [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                             C.POINTER(C.c_double)],
    "wf_get_transfer_bytes": [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
    "wf_set_launch_config": [C.c_void_p, C.c_int32, C.c_int32, C.c_int32],
    "wf_set_step_mode": [C.c_void_p, C.c_int32],
    "wf_get_step_mode": [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                         C.POINTER(C.c_int32)],
    "wf_set_box_indexing": [C.c_void_p, C.c_int32],
    "wf_set_sweep_rows": [C.c_void_p, C.c_int32],
    "wf_get_halo_node_width": [C.c_void_p, C.POINTER(C.c_int32)],
    "wf_set_flow_tiles": [C.c_void_p, C.c_int32, C.c_int32],
    "wf_get_flow": [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_char_p,
                    C.c_int64],
    "wf_get_sweep": [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                     C.POINTER(C.c_int32), C.c_char_p, C.c_int64],
    "wf_get_box": [C.c_void_p, _ip],
    "wf_get_tiles": [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                     C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_char_p, C.c_int64],
    "wf_adjoint_forward": [C.c_void_p, C.c_int64, C.c_int64],
    "wf_deck_read": [C.c_char_p, C.POINTER(C.c_void_p), C.c_char_p, C.c_int64],
    "wf_deck_free": [C.c_void_p],
    "wf_deck_get_info": [C.c_void_p, C.POINTER(WfDeckInfo)],
    "wf_deck_get_mesh": [C.c_void_p, _dp, _ip],
    "wf_deck_get_bcs": [C.c_void_p, _lp, _ip, _dp],
    "wf_deck_get_die": [C.c_void_p, _dp, _ip],
    "wf_deck_apply": [C.c_void_p, C.c_void_p],
    "wf_load_deck": [C.c_void_p, C.c_char_p, C.POINTER(WfDeckInfo), C.c_char_p, C.c_int64],
    "wf_load_lsdyna": [C.c_void_p, C.c_char_p],
    "wf_write_vtk": [C.c_void_p, C.c_char_p],
    "wf_snapshot": [C.c_void_p, C.POINTER(C.c_int32)],
    "wf_step_begin": [C.c_void_p],
    "wf_step_end": [C.c_void_p],
    "wf_get_halo_forces": [C.c_void_p, C.c_int64, C.c_int64, _dp],
    "wf_set_halo_forces": [C.c_void_p, C.c_int64, C.c_int64, _dp],
    "wf_get_halo_nodes": [C.c_void_p, C.c_int64, C.c_int64, _dp],
    "wf_set_halo_nodes": [C.c_void_p, C.c_int64, C.c_int64, _dp],
    "wf_write_snapshot_vtk": [C.c_void_p, C.c_int32, C.c_char_p],
    "wf_set_contact_trimesh": [C.c_void_p, C.c_int64, _dp, C.c_int64, _ip, _dp, C.c_double,
                               C.c_double, C.c_double],
    "wf_get_trimesh_nodes": [C.c_void_p, _dp, C.c_int64, C.POINTER(C.c_int64)],
    "wf_add_contact_trimesh": [C.c_void_p, C.c_int64, _dp, C.c_int64, _ip, _dp],
    "wf_set_thermal": [C.c_void_p, C.c_int32, C.c_double],
    "wf_set_material_thermal": [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double],
    "wf_set_contact_heat": [C.c_void_p, C.c_double, C.c_double],
    "wf_deck_get_body": [C.c_void_p, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                         C.POINTER(C.c_double), C.c_void_p, C.c_void_p],
    "wf_read_nastran": [C.c_char_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                        C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_char_p,
                        C.c_int64],
    "wf_set_energy_history": [C.c_void_p, C.c_int32],
    "wf_set_johnson_cook": [C.c_void_p, C.c_int32] + [C.c_double] * 8,
    "wf_set_gmt": [C.c_void_p, C.c_int32, _dp, _dp, C.c_double],
    "wf_get_energy_history": [C.c_void_p, _dp, _dp, C.c_int64, C.POINTER(C.c_int64)],
    "wf_adjoint_backward": [C.c_void_p, _dp, C.c_int32, _dp],
    # allocation-free nodal volumes: device pointers in, device pointer out
    "wf_nodal_volumes_noalloc": [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int32,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
}


def lib():
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"CUDA library missing: {LIB_PATH} (run weldformfem_gb300/build.py)")
    L = C.CDLL(LIB_PATH)
    for name, args in _SIGS.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.wf_last_error.argtypes = [C.c_void_p]
    L.wf_last_error.restype = C.c_char_p
    L.wf_status_string.argtypes = [C.c_int]
    L.wf_status_string.restype = C.c_char_p
    L.wf_abi_version.argtypes = []
    L.wf_abi_version.restype = C.c_int32
    _lib = L
    return L


def _bc_arrays(bcs):
    if isinstance(bcs, tuple) and len(bcs) == 3 and hasattr(bcs[0], "__len__") and \
            not isinstance(bcs[0], tuple):
        nodes, dims, vals = bcs
    else:
        arr = list(bcs)
        nodes = [b[0] for b in arr]
        dims = [b[1] for b in arr]
        vals = [b[2] for b in arr]
    return (np.ascontiguousarray(nodes, np.int64), np.ascontiguousarray(dims, np.int32),
            np.ascontiguousarray(vals, np.float64))


class Domain:
    """One GPU domain (MetFEM::Domain_d drop-in) driven through the C ABI."""

    def __init__(self, precision: int = WF_FP64, device: int = 0):
        L = lib()
        h = C.c_void_p()
        st = L.wf_domain_create_on_device(C.byref(h), int(device))
        if st != 0:
            raise WfError(st, "wf_domain_create: no usable CUDA device")
        self.h = h
        self.precision = precision
        self._nmat = 0
        self._call("wf_set_precision", int(precision))

    def _call(self, name, *args):
        st = getattr(lib(), name)(self.h, *args)
        if st != 0:
            raise WfError(st, f"{name}: {lib().wf_last_error(self.h).decode()}")
        return st

    def close(self):
        if getattr(self, "h", None):
            lib().wf_domain_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # mesh -------------------------------------------------------------
    def add_box(self, L, r, tritetra=False, origin=(0.0, 0.0, 0.0)):
        self._call("wf_add_box_length", np.array(origin, float), np.array(L, float), float(r), 1,
                   int(bool(tritetra)))

    def set_mesh(self, x, elnod):
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        elnod = np.ascontiguousarray(elnod, np.int32)
        ne, npe = elnod.shape
        self._call("wf_set_mesh", x.size // 3, ne, npe, x, elnod.reshape(-1))

    def set_nodes(self, x):
        self._call("wf_set_nodes", np.ascontiguousarray(x, np.float64).reshape(-1))

    def sizes(self):
        nn, ne, tot = C.c_int64(), C.c_int64(), C.c_int64()
        npe = C.c_int32()
        self._call("wf_get_sizes", C.byref(nn), C.byref(ne), C.byref(npe), C.byref(tot))
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
        self._call("wf_get_connectivity", elnod, nodel, loc, off, cnt)
        return elnod.reshape(ne, npe), nodel, loc, off, cnt

    # setup ------------------------------------------------------------
    def set_materials(self, mats, elem_ids=None):
        arr = (WfMaterial * len(mats))()
        for i, m in enumerate(mats):
            arr[i] = WfMaterial(int(m.get("model", 0)), float(m["E"]), float(m["nu"]),
                                float(m["rho"]), float(m.get("sy0", 1e10)), float(m.get("H", 0.0)),
                                float(m.get("hol_K", 1.0)), float(m.get("hol_m", 1.0)))
        self._call("wf_set_materials", len(mats), arr)
        self._nmat = len(mats)
        if elem_ids is not None:
            self._call("wf_set_elem_materials", np.ascontiguousarray(elem_ids, np.int32))

    def set_johnson_cook(self, mat, B, n, C, eps0, m, Tm, Tt, T=0.0):
        """Material_::Init_JohnsonCook constants of material `mat` (model 2)."""
        self._call("wf_set_johnson_cook", int(mat), float(B), float(n), float(C), float(eps0),
                   float(m), float(Tm), float(Tt), float(T))

    def set_gmt(self, mat, c, rng, T=0.0):
        """GMT law of material `mat` (model 3): c = (n1, n2, C1, C2, m1, m2, I1,
        I2), rng = (e_min, e_max, er_min, er_max, T_min, T_max), T the
        temperature without thermal coupling."""
        c = np.ascontiguousarray(c, np.float64)
        rng = np.ascontiguousarray(rng, np.float64)
        if c.size != 8 or rng.size != 6:
            raise ValueError("set_gmt takes 8 constants and 6 range bounds")
        self._call("wf_set_gmt", int(mat), c, rng, float(T))

    def set_hourglass(self, coef):
        self._call("wf_set_hourglass", float(coef))

    def set_press_algorithm(self, alg):
        self._call("wf_set_press_algorithm", int(alg))

    def set_stab(self, s10):
        s = WfStab(*[float(v) for v in s10])
        self._call("wf_set_stab", C.byref(s))

    def set_artif_visc(self, a, b):
        self._call("wf_set_artif_visc", float(a), float(b))

    def set_plastic_heat_fraction(self, f):
        """m_plheatfraction: plastic work fraction turned into heat (before init)."""
        self._call("wf_set_plastic_heat_fraction", float(f))

    def set_max_strain_rate(self, r):
        """m_max_edot: cap of the strain rate of the rate-dependent tangents (before init)."""
        self._call("wf_set_max_strain_rate", float(r))

    def set_mass_mode(self, mode):
        self._call("wf_set_mass_mode", int(mode))

    def add_bcs(self, bcs):
        """bcs: (node, dim, value) triples, or a tuple of three arrays."""
        nodes, dims, vals = _bc_arrays(bcs)
        self._call("wf_add_bc_vel_nodes", nodes.size, nodes, dims, vals)
        self._call("wf_allocate_bcs")

    def add_bc_vel_zone(self, start, end, vel):
        c = C.c_int64()
        self._call("wf_add_bc_vel_zone", np.array(start, float), np.array(end, float),
                   np.array(vel, float), C.byref(c))
        return c.value

    def set_reaction_nodes(self, nodes, dim=2):
        nodes = np.ascontiguousarray(nodes, np.int32)
        self._call("wf_set_reaction_nodes", nodes.size, nodes, int(dim))

    def set_contact_plane(self, z0, vz, kpen, mu, cand_nodes):
        cand = np.ascontiguousarray(cand_nodes, np.int32)
        self._call("wf_set_contact_plane", float(z0), float(vz), float(kpen), float(mu),
                   cand.size, cand)

    def set_dt(self, dt):
        self._call("wf_set_dt", float(dt))

    def set_specimens(self, elem_off, node_off, dts):
        """Batched ensemble: specimen s owns [elem_off[s], elem_off[s+1]) etc."""
        eo = np.ascontiguousarray(elem_off, np.int64)
        no = np.ascontiguousarray(node_off, np.int64)
        dt = np.ascontiguousarray(dts, np.float64)
        self._call("wf_set_specimens", dt.size, eo, no, dt)

    def specimen_reaction(self, spec):
        n = C.c_int64()
        self._call("wf_get_specimen_reaction", int(spec), np.zeros(1), 0, C.byref(n))
        out = np.zeros(max(n.value, 1))
        self._call("wf_get_specimen_reaction", int(spec), out, n.value, C.byref(n))
        return out[: n.value]

    def set_end_time(self, t):
        self._call("wf_set_end_time", float(t))

    # run --------------------------------------------------------------
    def init(self):
        self._call("wf_init")

    def step(self, n=1):
        self._call("wf_run", int(n))

    def run(self, n):
        self._call("wf_run", int(n))

    # adjoint ----------------------------------------------------------
    def adjoint_forward(self, n, every=0):
        """Runs n steps keeping checkpoints every `every` steps (0: ~sqrt(n))."""
        self._call("wf_adjoint_forward", int(n), int(every))

    def adjoint_backward(self, dL_dR, fp32=False):
        """dL/dR of each recorded step -> array [nmat, 3] of dL/d(E, sigma_y0, H)."""
        seed = np.ascontiguousarray(dL_dR, dtype=np.float64)
        grad = np.zeros(3 * self._nmat)
        self._call("wf_adjoint_backward", seed, int(bool(fp32)), grad)
        return grad.reshape(-1, 3)

    # step halves and halo data (slab decomposition) -------------------
    def step_begin(self):
        self._call("wf_step_begin")

    def step_end(self):
        self._call("wf_step_end")

    def halo_forces(self, e0, e1):
        """Element and hourglass forces of elements [e0, e1), flat."""
        out = np.zeros(2 * (e1 - e0) * self.npe * 3)
        self._call("wf_get_halo_forces", int(e0), int(e1), out)
        return out

    def set_halo_forces(self, e0, e1, data):
        data = np.ascontiguousarray(data, np.float64).reshape(-1)
        if data.size != 2 * (e1 - e0) * self.npe * 3:
            raise ValueError("halo forces of the wrong size")
        self._call("wf_set_halo_forces", int(e0), int(e1), data)

    def halo_node_width(self):
        """Values per node of halo_nodes: 12 (FP64 step) or 18 (mixed)."""
        w = C.c_int32()
        self._call("wf_get_halo_node_width", C.byref(w))
        return w.value

    def halo_nodes(self, n0, n1):
        """Node state a step starts from, nodes [n0, n1), flat."""
        out = np.zeros(self.halo_node_width() * (n1 - n0))
        self._call("wf_get_halo_nodes", int(n0), int(n1), out)
        return out

    def set_halo_nodes(self, n0, n1, data):
        data = np.ascontiguousarray(data, np.float64).reshape(-1)
        if data.size != self.halo_node_width() * (n1 - n0):
            raise ValueError("halo node state of the wrong size")
        self._call("wf_set_halo_nodes", int(n0), int(n1), data)

    def solve(self):
        n = C.c_int64()
        self._call("wf_solve", C.byref(n))
        return n.value

    def sync(self):
        self._call("wf_sync")

    @property
    def time(self):
        t = C.c_double()
        s = C.c_int64()
        self._call("wf_get_time", C.byref(t), C.byref(s))
        return t.value

    def min_edge_length(self):
        h = C.c_double()
        self._call("wf_min_edge_length", C.byref(h))
        return h.value

    def set_phase_timing(self, on=True):
        self._call("wf_set_phase_timing", int(bool(on)))

    def phase_times(self, reset=True):
        """(ms[4] of geometry, nodal, element, node phases; steps timed)."""
        ms = np.zeros(4)
        n = C.c_int64()
        self._call("wf_get_phase_times", ms, C.byref(n), int(bool(reset)))
        return ms, n.value

    def set_autotune(self, on=True):
        self._call("wf_set_autotune", int(bool(on)))

    def set_step_mode(self, mode):
        """0 automatic, 1 per-phase kernels, 2 one cluster launch per run, 3 tiled,
        4 column sweep, 5 dataflow step (4 and 5: box meshes)."""
        self._call("wf_set_step_mode", int(mode))

    def set_box_indexing(self, on=True):
        """Box meshes: corners and node lists computed in the kernels (before init)."""
        self._call("wf_set_box_indexing", int(bool(on)))

    def box(self):
        """(nx, ny, nz) of a box mesh the kernels index arithmetically, else zeros."""
        dims = np.zeros(3, np.int32)
        self._call("wf_get_box", dims)
        return tuple(int(v) for v in dims)

    def set_sweep_rows(self, rows):
        """Node rows per column of the column sweep, 4 or 8 (before init)."""
        self._call("wf_set_sweep_rows", int(rows))

    def sweep(self):
        """(columns along x, columns along y, node rows per column, why not swept)."""
        cx, cy, r = C.c_int32(), C.c_int32(), C.c_int32()
        buf = C.create_string_buffer(256)
        self._call("wf_get_sweep", C.byref(cx), C.byref(cy), C.byref(r), buf, 256)
        return cx.value, cy.value, r.value, buf.value.decode()

    def set_flow_tiles(self, tile=512, lag=4):
        """Dataflow step: items per tile and the node update's lag in stages (before init)."""
        self._call("wf_set_flow_tiles", int(tile), int(lag))

    def flow(self):
        """(tiles per step, blocks of the launch, why the mesh has no dataflow step)."""
        t, g = C.c_int32(), C.c_int32()
        buf = C.create_string_buffer(256)
        self._call("wf_get_flow", C.byref(t), C.byref(g), buf, 256)
        return t.value, g.value, buf.value.decode()

    def tiles(self):
        """(tiles, shared nodes, why the mesh was not tiled) of step mode 3."""
        return self.tile_stats()[:2] + (self.tile_stats()[4],)

    def tile_stats(self):
        """(tiles, shared nodes, sum of tile nodes, shared-node list entries, why)."""
        nt, ns = C.c_int32(), C.c_int32()
        tn, ss = C.c_int64(), C.c_int64()
        buf = C.create_string_buffer(256)
        self._call("wf_get_tiles", C.byref(nt), C.byref(ns), C.byref(tn), C.byref(ss), buf, 256)
        return nt.value, ns.value, tn.value, ss.value, buf.value.decode()

    def step_mode(self):
        """(mode the next run uses, cluster blocks, tiles or columns, block size)."""
        m, b, t = C.c_int32(), C.c_int32(), C.c_int32()
        self._call("wf_get_step_mode", C.byref(m), C.byref(b), C.byref(t))
        return m.value, b.value, t.value

    def set_launch_config(self, phase, block, items_per_thread):
        """Launch shape of phase 0/1/2 (items_per_thread 0: persistent grid)."""
        self._call("wf_set_launch_config", int(phase), int(block), int(items_per_thread))

    def launch_config(self, phase):
        """(block size, items per thread, trial ms) chosen for phase 0/1/2."""
        b, e, ms = C.c_int32(), C.c_int32(), C.c_double()
        self._call("wf_get_launch_config", int(phase), C.byref(b), C.byref(e), C.byref(ms))
        return b.value, e.value, ms.value

    def stream_handle(self):
        """The domain's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        p = C.c_void_p()
        self._call("wf_get_stream", C.byref(p))
        return p.value or 0

    def transfer_bytes(self):
        a, b = C.c_int64(), C.c_int64()
        self._call("wf_get_transfer_bytes", C.byref(a), C.byref(b))
        return a.value, b.value

    def launch_count(self):
        n = C.c_int64()
        self._call("wf_get_launch_count", C.byref(n))
        return n.value

    def graph_launches(self):
        """Step graphs replayed since init."""
        n = C.c_int64()
        self._call("wf_get_graph_launches", C.byref(n))
        return n.value

    def prepare_run(self, n):
        """Builds now the step graphs a following run(n) replays (runs nothing)."""
        self._call("wf_prepare_run", int(n))

    # readback ---------------------------------------------------------
    def node_vec(self, name, out=None):
        """A node field as [nn, 3]; `out` (a C-contiguous float64 array of nn * 3
        values, pinned or already written to for the fastest copy) is filled
        instead of a new array."""
        if out is None:
            out = np.zeros(self.nn * 3)
        elif not (out.dtype == np.float64 and out.flags.c_contiguous and out.size == self.nn * 3):
            raise ValueError("out must be a C-contiguous float64 array of nn * 3 values")
        self._call("wf_get_node_field", NODE_VEC[name], out.reshape(-1))
        return out.reshape(-1, 3)

    def node_scalar(self, name):
        out = np.zeros(self.nn)
        self._call("wf_get_node_scalar", NODE_SCALAR[name], out)
        return out

    def elem_scalar(self, name):
        out = np.zeros(self.ne)
        self._call("wf_get_elem_scalar", ELEM_SCALAR[name], out)
        return out

    def elem_tensor(self, name):
        out = np.zeros(self.ne * 6)
        self._call("wf_get_elem_tensor", ELEM_TENSOR[name], out)
        return out.reshape(-1, 6)

    def set_contact_trimesh(self, xyz, tri, vel, mu_static=0.0, mu_dynamic=0.0,
                            penalty_factor=0.1):
        """Rigid triangle-mesh die (setTriMesh + setContactOn + setContactPF)."""
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1)
        tri = np.ascontiguousarray(tri, np.int32).reshape(-1)
        self._call("wf_set_contact_trimesh", xyz.size // 3, xyz, tri.size // 3, tri,
                   np.ascontiguousarray(vel, np.float64), float(mu_static), float(mu_dynamic),
                   float(penalty_factor))

    def set_thermal(self, on=True, T0=20.0):
        """Thermal coupling (setThermalOn + setTemp), FP64 step."""
        self._call("wf_set_thermal", int(bool(on)), float(T0))

    def set_material_thermal(self, mat, k_T, cp_T, exp_T=0.0):
        self._call("wf_set_material_thermal", int(mat), float(k_T), float(cp_T), float(exp_T))

    def set_contact_heat(self, heat_cond, T_die=20.0):
        self._call("wf_set_contact_heat", float(heat_cond), float(T_die))

    def add_contact_trimesh(self, xyz, tri, vel):
        """Another rigid body (TriMesh_d::AddMesh); only body 0 feeds the reaction."""
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1)
        tri = np.ascontiguousarray(tri, np.int32).reshape(-1)
        self._call("wf_add_contact_trimesh", xyz.size // 3, xyz, tri.size // 3, tri,
                   np.ascontiguousarray(vel, np.float64))

    def trimesh_nodes(self):
        n = C.c_int64()
        self._call("wf_get_trimesh_nodes", np.zeros(3), 0, C.byref(n))
        out = np.zeros(3 * max(n.value, 1))
        self._call("wf_get_trimesh_nodes", out, n.value, C.byref(n))
        return out[: 3 * n.value].reshape(-1, 3)

    # input files and output ----------------------------------------------
    def load_deck(self, path):
        """Reads a JSON deck and sets this domain up from it; returns its info."""
        info = WfDeckInfo()
        err = C.create_string_buffer(512)
        st = lib().wf_load_deck(self.h, os.fsencode(path), C.byref(info), err, 512)
        if st != 0:
            raise WfError(st, err.value.decode())
        return Deck._info_dict(info)

    def load_lsdyna(self, path):
        self._call("wf_load_lsdyna", os.fsencode(path))

    def write_vtk(self, path):
        self._call("wf_write_vtk", os.fsencode(path))

    def snapshot(self):
        """Queues a copy of the output fields to pinned host memory; returns its slot."""
        slot = C.c_int32()
        self._call("wf_snapshot", C.byref(slot))
        return slot.value

    def write_snapshot_vtk(self, slot, path):
        """Writes a snapshot (see snapshot()) as wf_write_vtk would have at its step."""
        self._call("wf_write_snapshot_vtk", int(slot), os.fsencode(path))

    def set_energy_history(self, on=True):
        self._call("wf_set_energy_history", int(bool(on)))

    def energies(self):
        """(kinetic energy, accumulated internal energy) after each step."""
        n = C.c_int64()
        self._call("wf_get_energy_history", np.zeros(1), np.zeros(1), 0, C.byref(n))
        k, e = np.zeros(max(n.value, 1)), np.zeros(max(n.value, 1))
        self._call("wf_get_energy_history", k, e, n.value, C.byref(n))
        return k[: n.value], e[: n.value]

    def reaction(self):
        n = C.c_int64()
        self._call("wf_get_reaction_history", np.zeros(1), 0, C.byref(n))
        out = np.zeros(max(n.value, 1))
        self._call("wf_get_reaction_history", out, n.value, C.byref(n))
        return out[: n.value]


def read_nastran(path, flip_normals=False, orient_point=None):
    """Nastran die mesh (wf_read_nastran): (xyz[n, 3], tri[m, 3]) with the
    reference's flipnormals and orientNormals rules (orient_point None: no
    orientation)."""
    nn, nt = C.c_int64(), C.c_int64()
    err = C.create_string_buffer(512)
    pt = None if orient_point is None else (C.c_double * 3)(*[float(v) for v in orient_point])
    args = (os.fsencode(path), int(bool(flip_normals)), pt)
    st = lib().wf_read_nastran(*args, None, 0, None, 0, C.byref(nn), C.byref(nt), err, 512)
    if st != 0:
        raise WfError(st, err.value.decode())
    x = np.zeros(3 * nn.value)
    t = np.zeros(3 * nt.value, np.int32)
    st = lib().wf_read_nastran(*args, x.ctypes.data, nn.value, t.ctypes.data, nt.value,
                               C.byref(nn), C.byref(nt), err, 512)
    if st != 0:
        raise WfError(st, err.value.decode())
    return x.reshape(-1, 3), t.reshape(-1, 3)


class Deck:
    """A JSON deck read on the host (wf_deck_read): the mesh, the material,
    the ordered AddBCVelNode calls and the options, ready to be applied to a
    GPU domain (apply) or to any backend with the same method names (setup)."""

    def __init__(self, path):
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        st = lib().wf_deck_read(os.fsencode(path), C.byref(h), err, 512)
        if st != 0:
            raise WfError(st, err.value.decode())
        self.h = h
        info = WfDeckInfo()
        lib().wf_deck_get_info(self.h, C.byref(info))
        self.info = self._info_dict(info)

    @staticmethod
    def _info_dict(info):
        out = {f: getattr(info, f) for f, _ in WfDeckInfo._fields_
               if f not in ("artif_visc", "stab", "material", "die_vel", "johnson_cook", "gmt",
                            "gmt_range")}
        out["johnson_cook"] = [info.johnson_cook[k] for k in range(8)]
        out["gmt"] = [info.gmt[k] for k in range(8)]
        out["gmt_range"] = [info.gmt_range[k] for k in range(6)]
        out["artif_visc"] = (info.artif_visc[0], info.artif_visc[1])
        out["die_vel"] = tuple(info.die_vel[k] for k in range(3))
        out["stab"] = [getattr(info.stab, f) for f, _ in WfStab._fields_]
        m = info.material
        out["material"] = {f: getattr(m, f) for f, _ in WfMaterial._fields_}
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().wf_deck_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def mesh(self):
        nn, ne, npe = self.info["nn"], self.info["ne"], self.info["npe"]
        x = np.zeros(3 * nn)
        el = np.zeros(ne * npe, np.int32)
        lib().wf_deck_get_mesh(self.h, x, el)
        return x.reshape(-1, 3), el.reshape(-1, npe)

    def bcs(self):
        n = self.info["n_bc"]
        node, dim, val = np.zeros(max(n, 1), np.int64), np.zeros(max(n, 1), np.int32), np.zeros(max(n, 1))
        lib().wf_deck_get_bcs(self.h, node, dim, val)
        return node[:n], dim[:n], val[:n]

    def body(self, b):
        """(xyz[n, 3], tri[m, 3], vel[3]) of rigid body b of a contact deck."""
        nn, nt = C.c_int64(), C.c_int64()
        vel = (C.c_double * 3)()
        st = lib().wf_deck_get_body(self.h, int(b), C.byref(nn), C.byref(nt), vel, None, None)
        if st != 0:
            raise WfError(st, f"no rigid body {b}")
        x = np.zeros(3 * max(nn.value, 1))
        t = np.zeros(3 * max(nt.value, 1), np.int32)
        lib().wf_deck_get_body(self.h, int(b), None, None, None, x.ctypes.data, t.ctypes.data)
        return (x[: 3 * nn.value].reshape(-1, 3), t[: 3 * nt.value].reshape(-1, 3),
                np.array(vel[:]))

    def die(self):
        """(xyz[n, 3], tri[m, 3]) of a contact deck's die (rigid body 0)."""
        x = np.zeros(3 * max(self.info["die_nodes"], 1))
        t = np.zeros(3 * max(self.info["die_tris"], 1), np.int32)
        lib().wf_deck_get_die(self.h, x, t)
        return x[: 3 * self.info["die_nodes"]].reshape(-1, 3), t[: 3 * self.info["die_tris"]].reshape(-1, 3)

    def apply(self, dom):
        st = lib().wf_deck_apply(self.h, dom.h)
        if st != 0:
            raise WfError(st, lib().wf_last_error(dom.h).decode())

    def setup(self, dom):
        """The same calls as wf_deck_apply, through a backend's Python methods."""
        x, el = self.mesh()
        i = self.info
        dom.set_mesh(x, el)
        dom.set_materials([i["material"]])
        if i["material"]["model"] == 2:
            dom.set_johnson_cook(0, *i["johnson_cook"])
        if i["material"]["model"] == 3:
            dom.set_gmt(0, i["gmt"], i["gmt_range"], i["T0"] if i["thermal"] else 0.0)
        dom.add_bcs(self.bcs())
        if i["has_stab"]:
            dom.set_stab(np.array(i["stab"]))
        if i["press_alg"]:
            dom.set_press_algorithm(i["press_alg"])
        if any(i["artif_visc"]):
            dom.set_artif_visc(*i["artif_visc"])
        dom.set_plastic_heat_fraction(i["plheat_frac"])
        dom.set_max_strain_rate(i["max_edot"])
        if i["hourglass"]:
            dom.set_hourglass(i["hourglass"])
        if i["thermal"]:
            dom.set_thermal(True, i["T0"])
            dom.set_material_thermal(0, i["thermal_k"], i["thermal_cp"], i["thermal_exp"])
        if i["contact"]:
            xyz, tri = self.die()
            dom.set_contact_trimesh(xyz, tri, i["die_vel"], i["mu_static"], i["mu_dynamic"],
                                    i["penalty_factor"])
            for b in range(1, i["rigid_bodies"]):
                dom.add_contact_trimesh(*self.body(b))
            if i["thermal"]:
                dom.set_contact_heat(i["heat_cond"], i["die_temp"])
        dom.set_dt(i["dt"])
        dom.set_end_time(i["end_time"])
