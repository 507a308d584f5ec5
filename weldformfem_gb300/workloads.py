"""Synthetic workloads: box meshes, seeded perturbations, materials and BCs.

The reference publishes no benchmark data set; its test decks are small
cubes (validation/*.txt, src/common/main_1_elem_3d.C). The workloads here
are the five configurations of the measurement plan, generated on the host
from a counter-based RNG so that every backend (the CUDA library, the CPU
oracle, the reference compiled from source) receives bit-identical inputs:

  C0  10^3 hexahedra, cube of side 10 mm, hourglass 0.1, 5000 steps
  C1  40x40x60 cells x 6 tetrahedra (576,000), 20x20x30 mm, +-0.15h, 2000 steps
  C2  256x256x128 hexahedra (8.39 M), h = 1 mm, +-0.1h, rigid die, 1000 steps
  C3  1024 independent cubes, n ~ U{6..40}, per-specimen material, 2000 steps
  C4  32^3 hexahedra, 8 octant materials (the C0 cube, h = 0.3125 mm), 4000 steps

Meshes use the numbering of Domain_d::AddBoxLength (Domain_d.C:1136-1504).
Velocity BCs follow the reference drivers: symmetry planes x=0, y=0, z=0
(AddBCVelNode with value 0) and a prescribed top velocity. The time step is
dt = 0.3 * h_min / sqrt(E / rho) with h_min the shortest element edge.
"""
from __future__ import annotations

import dataclasses
from typing import Callable, Optional

import numpy as np

SEED_BASE = 0x5EED0000
_M64 = (1 << 64) - 1

STEEL = dict(model=0, E=200e9, nu=0.3, rho=7850.0, sy0=300e6, H=1e9)


def splitmix64(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """Counter-based splitmix64 stream: value i is mix(seed + (offset+i+1)*golden)."""
    with np.errstate(over="ignore"):
        i = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
        z = np.uint64(seed & _M64) + i * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform_pm1(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """Uniform doubles in [-1, 1) from the top 53 bits of splitmix64."""
    z = splitmix64(seed, n, offset) >> np.uint64(11)
    return z.astype(np.float64) * (2.0 ** -52) - 1.0


def box_counts(L, r):
    """Element counts per axis exactly as AddBoxLength truncates them."""
    return tuple(int(float(L[k]) / (2.0 * float(r))) for k in range(3))


def box_coords(L, r, origin=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Node coordinates of AddBoxLength: repeated addition of 2r (Domain_d.C:1215-1235)."""
    nel = box_counts(L, r)
    xs = []
    for k, n in enumerate(nel):
        v = float(origin[k])
        col = []
        for _ in range(n + 1):
            col.append(v)
            v = v + 2.0 * r
        xs.append(np.array(col))
    zz, yy, xx = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
    return np.stack([xx.ravel(), yy.ravel(), zz.ravel()], axis=1)


def perturb_interior(x: np.ndarray, nel, h: float, frac: float, seed: int) -> np.ndarray:
    """Moves every node not on a boundary face by U[-frac h, +frac h] per axis."""
    nx, ny, nz = (n + 1 for n in nel)
    idx = np.arange(x.shape[0])
    i, j, k = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    interior = (i > 0) & (i < nx - 1) & (j > 0) & (j < ny - 1) & (k > 0) & (k < nz - 1)
    out = x.copy()
    sel = np.nonzero(interior)[0]
    du = uniform_pm1(seed, 3 * sel.size).reshape(-1, 3) * (frac * h)
    out[sel] += du
    return out


def hex_edges():
    return [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4),
            (0, 4), (1, 5), (2, 6), (3, 7)]


TET_EDGES = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


def min_edge_length(x: np.ndarray, elnod: np.ndarray) -> float:
    """Shortest element edge, length = sqrt(dx*dx + dy*dy + dz*dz)."""
    edges = hex_edges() if elnod.shape[1] == 8 else TET_EDGES
    best = np.inf
    for a, b in edges:
        d = x[elnod[:, b]] - x[elnod[:, a]]
        ln = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
        best = min(best, float(ln.min()))
    return best


def box_elnod(nel, tritetra: bool) -> np.ndarray:
    """Connectivity of AddBoxLength (hex x-fastest, optional six-tet split)."""
    nx, ny, nz = nel
    nnodz = (nx + 1) * (ny + 1)
    ez, ey, ex = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ez, ey, ex = ez.ravel(), ey.ravel(), ex.ravel()
    nb1 = nnodz * ez + (nx + 1) * ey + ex
    nb2 = nnodz * ez + (nx + 1) * (ey + 1) + ex
    h = np.stack([nb1, nb1 + 1, nb2 + 1, nb2, nb1 + nnodz, nb1 + nnodz + 1,
                  nb2 + nnodz + 1, nb2 + nnodz], axis=1)
    if not tritetra:
        return h.astype(np.int32)
    T = np.array([[0, 1, 3, 5], [1, 2, 3, 5], [0, 5, 3, 4], [4, 5, 3, 7], [5, 6, 3, 7],
                  [5, 2, 3, 6]])
    return h[:, T].reshape(-1, 4).astype(np.int32)


@dataclasses.dataclass
class Case:
    name: str
    L: tuple
    r: float
    tritetra: bool = False
    perturb: float = 0.0
    seed: int = SEED_BASE
    materials: list = dataclasses.field(default_factory=lambda: [dict(STEEL)])
    elem_mat: Optional[np.ndarray] = None
    bc: str = "sym_top"          # "sym_top": symmetry + top vz; "bottom_z": bottom fixed in z;
    #                              "sym_xy": x and y symmetry planes only
    top_vz: float = -1.0
    hg: float = 0.0
    dt: Optional[float] = None   # None: 0.3 h_min / sqrt(E / rho)
    dt_factor: float = 0.3
    steps: int = 1
    contact: Optional[dict] = None   # dict(v=5.0, kfac=10.0, mu=0.1)
    press_alg: int = 0
    mass_mode: int = 0

    # derived --------------------------------------------------------
    @property
    def nel(self):
        return box_counts(self.L, self.r)

    @property
    def h(self):
        return 2.0 * self.r

    def coords(self) -> np.ndarray:
        x = box_coords(self.L, self.r)
        if self.perturb:
            x = perturb_interior(x, self.nel, self.h, self.perturb, self.seed)
        return x

    def elnod(self) -> np.ndarray:
        return box_elnod(self.nel, self.tritetra)

    @property
    def n_elem(self):
        nx, ny, nz = self.nel
        return nx * ny * nz * (6 if self.tritetra else 1)

    @property
    def n_node(self):
        nx, ny, nz = self.nel
        return (nx + 1) * (ny + 1) * (nz + 1)

    def time_step(self, x=None) -> float:
        if self.dt is not None:
            return float(self.dt)
        if x is None:
            x = self.coords()
        hmin = min_edge_length(x, self.elnod()) if self.perturb else self.h
        m = self.materials[0]
        return self.dt_factor * hmin / np.sqrt(m["E"] / m["rho"])

    def bcs(self, x0=None):
        """Velocity BCs as three arrays (node, dof, value), in node order and,
        per node, x-symmetry, y-symmetry, z-symmetry, top velocity."""
        nx, ny, nz = (n + 1 for n in self.nel)
        idx = np.arange(nx * ny * nz, dtype=np.int64)
        i, j, k = idx % nx, (idx // nx) % ny, idx // (nx * ny)
        if self.bc == "sym_top":
            conds = [(i == 0, 0, 0.0), (j == 0, 1, 0.0), (k == 0, 2, 0.0),
                     (k == nz - 1, 2, float(self.top_vz))]
        elif self.bc == "bottom_z":
            conds = [(k == 0, 2, 0.0)]
        elif self.bc == "sym_xy":
            conds = [(i == 0, 0, 0.0), (j == 0, 1, 0.0)]
        else:
            raise ValueError(self.bc)
        nodes, dims, vals, order = [], [], [], []
        for rank, (mask, dof, val) in enumerate(conds):
            sel = idx[mask]
            nodes.append(sel)
            dims.append(np.full(sel.size, dof, np.int32))
            vals.append(np.full(sel.size, val))
            order.append(sel * 4 + rank)
        perm = np.argsort(np.concatenate(order), kind="stable")
        return (np.concatenate(nodes)[perm], np.concatenate(dims)[perm],
                np.concatenate(vals)[perm])

    def top_nodes(self) -> np.ndarray:
        nx, ny, nz = (n + 1 for n in self.nel)
        return np.arange(nx * ny * (nz - 1), nx * ny * nz, dtype=np.int32)

    def contact_params(self):
        c = self.contact
        m = self.materials[0]
        return dict(z0=float(self.L[2]), vz=-float(c["v"]), kpen=float(c["kfac"]) * m["E"] * self.h,
                    mu=float(c["mu"]))


def apply_options(dom, case: Case, with_bcs=True, x=None, set_dt=True, bcs=None):
    """Everything after the mesh: materials, BCs, options, dt. Returns dt
    (None when set_dt is False: the caller sets it, e.g. from the device
    min-edge reduction after init). `bcs` = case.bcs() when the caller has
    built them already."""
    dom.set_materials(case.materials, case.elem_mat)
    if with_bcs:
        dom.add_bcs(case.bcs() if bcs is None else bcs)
    if case.hg:
        dom.set_hourglass(case.hg)
    if case.press_alg:
        dom.set_press_algorithm(case.press_alg)
    if case.mass_mode and hasattr(dom, "set_mass_mode"):
        dom.set_mass_mode(case.mass_mode)
    if case.contact:
        cp = case.contact_params()
        dom.set_contact_plane(cp["z0"], cp["vz"], cp["kpen"], cp["mu"], case.top_nodes())
    else:
        dom.set_reaction_nodes(case.top_nodes(), 2)
    if not set_dt:
        return None
    if x is None:
        x = case.coords()
    dt = case.time_step(x)
    dom.set_dt(dt)
    return dt


def cfl_dt(case: Case, hmin: float) -> float:
    """dt = factor * h_min / sqrt(E / rho) of the first material."""
    m = case.materials[0]
    return case.dt_factor * hmin / np.sqrt(m["E"] / m["rho"])


def apply(dom, case: Case, x=None, with_bcs=True):
    """Sets up any domain backend (same method names) for `case` and returns dt."""
    dom.add_box(case.L, case.r, case.tritetra)
    if x is None:
        x = case.coords()
    if case.perturb:
        dom.set_nodes(x)
    return apply_options(dom, case, with_bcs, x)


def octant_ids(case: Case) -> np.ndarray:
    """Octant index (0..7) of each hexahedron of a box case, x-fastest bits."""
    nx, ny, nz = case.nel
    ez, ey, ex = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return ((ex.ravel() >= nx // 2).astype(np.int32) + 2 * (ey.ravel() >= ny // 2)
            + 4 * (ez.ravel() >= nz // 2)).astype(np.int32)


def config(cid: int, steps: Optional[int] = None, scale: Optional[tuple] = None) -> Case:
    """The named configurations; `scale` overrides the cell counts (same h)."""
    if cid == 0:
        c = Case("C0 hex 10^3", L=(0.01, 0.01, 0.01), r=0.0005, hg=0.1, steps=5000)
    elif cid == 1:
        c = Case("C1 tet 40x40x60x6", L=(0.02, 0.02, 0.03), r=0.00025, tritetra=True,
                 perturb=0.15, seed=SEED_BASE + 1, steps=2000)
    elif cid == 2:
        c = Case("C2 hex 256x256x128 die", L=(0.256, 0.256, 0.128), r=0.0005, perturb=0.1,
                 seed=SEED_BASE + 2, hg=0.1, bc="bottom_z",
                 contact=dict(v=5.0, kfac=10.0, mu=0.1), steps=1000)
    elif cid == 4:
        c = Case("C4 hex 32^3 octants", L=(0.01, 0.01, 0.01), r=0.00015625, hg=0.1, steps=4000)
        c.materials = [dict(STEEL) for _ in range(8)]
        c.elem_mat = octant_ids(c)
    else:
        raise ValueError(f"unknown configuration {cid}")
    if scale is not None:
        h = c.h
        c.L = tuple(float(n) * h for n in scale)
        c.name = f"{c.name.split()[0]} scaled to {scale[0]}x{scale[1]}x{scale[2]} cells"
        if c.elem_mat is not None:
            c.elem_mat = octant_ids(c)
    if steps is not None:
        c.steps = steps
    return c


def axis_plane_mesh(start, end, dens, flip_normals=False):
    """Rigid plane of triangles normal to z (TriMesh_d::AxisPlaneMesh with
    axis 2, Mesh.C:48-200, as the JSON driver calls it with the block's start
    and dim): (dens+1)^2 nodes at z = start[2], spacing (end[0] - start[0]) /
    dens in x and y from start, two triangles per cell; the normal is +z,
    or -z with flip_normals. Returns (xyz[n, 3], tri[m, 3])."""
    dl = (float(end[0]) - float(start[0])) / dens
    nodes = []
    x2 = float(start[1])
    for j in range(dens + 1):
        x1 = float(start[0])
        for i in range(dens + 1):
            nodes.append((x1, x2, float(start[2])))
            x1 += dl
        x2 += dl
    tri = []
    for j in range(dens):
        for i in range(dens):
            n0 = (dens + 1) * j + i
            n1 = n0 + 1
            n2 = (dens + 1) * (j + 1) + i
            n3 = n2 + 1
            if not flip_normals:
                tri += [(n0, n1, n2), (n1, n3, n2)]
            else:
                tri += [(n0, n2, n1), (n1, n2, n3)]
    return np.array(nodes, dtype=np.float64), np.array(tri, dtype=np.int32)


PARAM_KEYS = ("E", "sy0", "H")


def material_params(case: Case) -> np.ndarray:
    """[nmat, 3] array of (E, sigma_y0, H) of the case's materials."""
    return np.array([[m[k] for k in PARAM_KEYS] for m in case.materials], dtype=np.float64)


def with_params(case: Case, theta) -> Case:
    """Copy of `case` whose materials take (E, sigma_y0, H) from theta[nmat, 3].
    The time step is frozen at the original case's value first, so that
    changing material 0's modulus does not change dt."""
    theta = np.asarray(theta, dtype=np.float64).reshape(-1, 3)
    c = dataclasses.replace(case, materials=[dict(m) for m in case.materials])
    if c.dt is None:
        c.dt = case.time_step()
    for m, row in zip(c.materials, theta):
        for k, v in zip(PARAM_KEYS, row):
            m[k] = float(v)
    return c


def target_factors(case: Case, seed: int = SEED_BASE + 4) -> np.ndarray:
    """Seeded U[0.8, 1.2) factors, one per material parameter (the target
    run of the material-identification problem)."""
    n = len(case.materials) * 3
    return (1.0 + 0.2 * uniform_pm1(seed, n)).reshape(-1, 3)


@dataclasses.dataclass
class Batch:
    """An ensemble of independent specimens run as one batched domain."""
    name: str
    cases: list
    hg: float = 0.1

    def offsets(self):
        eoff = np.zeros(len(self.cases) + 1, np.int64)
        noff = np.zeros(len(self.cases) + 1, np.int64)
        for s, c in enumerate(self.cases):
            eoff[s + 1] = eoff[s] + c.n_elem
            noff[s + 1] = noff[s] + c.n_node
        return eoff, noff

    @property
    def n_elem(self):
        return int(sum(c.n_elem for c in self.cases))

    @property
    def n_node(self):
        return int(sum(c.n_node for c in self.cases))

    def assemble(self):
        """Concatenated mesh, per-element specimen ids, BCs and reaction nodes."""
        eoff, noff = self.offsets()
        xs, els, bn, bd, bv, tops = [], [], [], [], [], []
        for s, c in enumerate(self.cases):
            xs.append(c.coords())
            els.append(c.elnod() + np.int32(noff[s]))
            nodes, dims, vals = c.bcs()
            bn.append(nodes + noff[s])
            bd.append(dims)
            bv.append(vals)
            tops.append(c.top_nodes() + np.int32(noff[s]))
        x = np.concatenate(xs)
        el = np.concatenate(els)
        emat = np.repeat(np.arange(len(self.cases), dtype=np.int32),
                         [c.n_elem for c in self.cases])
        bcs = (np.concatenate(bn), np.concatenate(bd), np.concatenate(bv))
        return x, el, emat, bcs, np.concatenate(tops), eoff, noff

    def dts(self):
        return np.array([c.time_step() for c in self.cases])


def apply_batch(dom, batch: Batch):
    """Sets up a batched domain (one specimen per material); returns dt per specimen."""
    x, el, emat, bcs, tops, eoff, noff = batch.assemble()
    dom.set_mesh(x, el)
    dom.set_materials([c.materials[0] for c in batch.cases], emat)
    dom.add_bcs(bcs)
    dom.set_hourglass(batch.hg)
    dom.set_reaction_nodes(tops, 2)
    dts = batch.dts()
    dom.set_specimens(eoff, noff, dts)
    return dts


def ensemble(n_spec: int = 1024, nmin: int = 6, nmax: int = 40, side: float = 0.01,
             seed: int = SEED_BASE + 3, steps: int = 2000) -> Batch:
    """Config 3: n_spec cubes of side `side`, n ~ U{nmin..nmax} elements per edge,
    E ~ U[70, 210] GPa, sigma_y0 ~ U[200, 500] MPa, H ~ U[0.2, 2] GPa, top velocity
    ~ U[0.5, 5] m/s, nu = 0.3, rho = 7850; symmetry + top-velocity BCs."""
    z = splitmix64(seed, 5 * n_spec).reshape(n_spec, 5)
    u01 = (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    cases = []
    for s in range(n_spec):
        n = nmin + int(z[s, 0] % np.uint64(nmax - nmin + 1))
        r = side / (2.0 * n)
        L = ((n + 0.25) * 2.0 * r,) * 3      # truncates to exactly n cells per edge
        mat = dict(model=0, E=70e9 + 140e9 * u01[s, 1], nu=0.3, rho=7850.0,
                   sy0=200e6 + 300e6 * u01[s, 2], H=0.2e9 + 1.8e9 * u01[s, 3])
        c = Case(f"C3 specimen {s} n={n}", L=L, r=r, hg=0.1, steps=steps,
                 top_vz=-(0.5 + 4.5 * u01[s, 4]))
        c.materials = [mat]
        assert c.nel == (n, n, n)
        cases.append(c)
    return Batch(f"C3 ensemble {n_spec} cubes n~U{{{nmin}..{nmax}}}", cases)
