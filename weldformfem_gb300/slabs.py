"""Slab decomposition of one box mesh over several domains (ranks).

The reference runs one mesh in one domain (assembly over all nodes,
src/common/Matrices.C:42-87; reaction over all contact nodes,
src/explicit/Solver_explicit.C:773). Here a box mesh in the AddBoxLength
numbering (nx x ny x nz hexahedra) is cut into slabs of element layers along
z, one per rank. Rank r owns layers [z0, z1) and holds them with a one-layer
halo on each side, layers [max(z0 - 1, 0), min(z1 + 1, nz)), as a box of its
own: its local element and node numbers keep the global order, so every node
list keeps its global (element-ascending) order.

Each step, per rank:
  step_begin    predictor, geometry, nodal and element phases on the slab;
  exchange      element forces: a halo layer's forces are overwritten with
                those its owner computed (the owner's halo inputs are right);
  step_end      assembly in list order and node update: every node of the
                owned planes, the planes shared with a neighbour included,
                gathers the forces of all its elements, so it is computed as
                in one domain, bit for bit, on both ranks that hold it;
  exchange      node state: a halo plane's state (the start of the next step)
                is overwritten with its owner's.
The time step is the minimum over ranks of the shortest element edge (an
allreduce(min)); the reaction is each rank's sum over the reaction or contact
nodes of the planes it owns (planes [z0, z1), the last rank also plane nz),
added over ranks in rank order.

Engines: any domain object with step_begin, step_end, halo_forces,
set_halo_forces, halo_nodes, set_halo_nodes, reaction (the CUDA
library's Domain, FP64 step; the tests also drive the CPU oracle). Transports:
LocalTransport runs all ranks in one process (one GPU, or the CPU);
DistTransport exchanges through torch.distributed point-to-point messages
(gloo, host buffers) between one process per rank.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import workloads as W


@dataclasses.dataclass
class Slab:
    """One rank's part of an nx x ny x nz box: owned layers [z0, z1), held
    layers [lo, hi) (the owned ones and a one-layer halo on each side)."""
    rank: int
    world: int
    nx: int
    ny: int
    nz: int
    z0: int
    z1: int

    @property
    def lo(self):
        return max(self.z0 - 1, 0)

    @property
    def hi(self):
        return min(self.z1 + 1, self.nz)

    @property
    def pxy(self):
        return (self.nx + 1) * (self.ny + 1)

    def layer(self, k):
        """Local element range [e0, e1) of global layer k."""
        e0 = (k - self.lo) * self.nx * self.ny
        return e0, e0 + self.nx * self.ny

    def plane(self, k):
        """Local node range [n0, n1) of global node plane k."""
        n0 = (k - self.lo) * self.pxy
        return n0, n0 + self.pxy

    def global_nodes(self):
        """Global node range [g0, g1) of the slab's planes lo..hi."""
        return self.lo * self.pxy, (self.hi + 1) * self.pxy

    def owned_planes(self):
        """Node planes whose reaction this rank counts."""
        return range(self.z0, self.z1 + (1 if self.rank == self.world - 1 else 0))


def plan(nx, ny, nz, world):
    """Slabs of nearly equal numbers of layers (at least one each)."""
    if world > nz:
        raise ValueError(f"{world} ranks for {nz} element layers")
    return [Slab(r, world, nx, ny, nz, nz * r // world, nz * (r + 1) // world)
            for r in range(world)]


def setup(dom, case, slab, dt):
    """Sets up a domain backend with the slab's part of a box case (the
    workloads' box configurations): mesh, materials, BCs, hourglass, contact
    candidates or reaction nodes of the owned planes, time step."""
    x = case.coords()
    g0, g1 = slab.global_nodes()
    xs = x[g0:g1]
    el = W.box_elnod((slab.nx, slab.ny, slab.hi - slab.lo), False)
    dom.set_mesh(xs, el)
    dom.set_materials(case.materials,
                      None if case.elem_mat is None else
                      case.elem_mat[slab.lo * slab.nx * slab.ny:slab.hi * slab.nx * slab.ny])
    nodes, dims, vals = case.bcs()
    keep = (nodes >= g0) & (nodes < g1)
    dom.add_bcs((nodes[keep] - g0, dims[keep], vals[keep]))
    if case.hg:
        dom.set_hourglass(case.hg)
    if case.press_alg:
        dom.set_press_algorithm(case.press_alg)
    owned = np.concatenate([np.arange(*slab.plane(k)) for k in slab.owned_planes()]) + g0
    top = case.top_nodes().astype(np.int64)
    mine = top[np.isin(top, owned)] - g0
    if case.contact:
        cp = case.contact_params()
        dom.set_contact_plane(cp["z0"], cp["vz"], cp["kpen"], cp["mu"], mine.astype(np.int32))
    else:
        dom.set_reaction_nodes(mine.astype(np.int32), 2)
    dom.set_dt(dt)


def local_min_edge(case, slab):
    """Shortest element edge of the slab's elements (held layers)."""
    x = case.coords()
    g0, g1 = slab.global_nodes()
    el = W.box_elnod((slab.nx, slab.ny, slab.hi - slab.lo), False)
    return W.min_edge_length(x[g0:g1], el)


class LocalTransport:
    """All ranks in one process: messages are handed over directly."""

    def exchange(self, sends):
        return dict(sends)

    def allreduce_min(self, values):
        return min(values.values())

    def sum_in_rank_order(self, values):
        out = None
        for r in sorted(values):
            out = values[r].copy() if out is None else out + values[r]
        return out


class DistTransport:
    """One process per rank over torch.distributed (point-to-point messages of
    host buffers; gloo)."""

    def __init__(self, rank, world):
        self.rank, self.world = rank, world

    def exchange(self, sends):
        import torch
        import torch.distributed as dist

        reqs, bufs = [], {}
        for (src, dst), arr in sorted(sends.items()):
            if src == self.rank and dst != self.rank:
                reqs.append(dist.isend(torch.from_numpy(np.ascontiguousarray(arr)), dst))
        for (src, dst), arr in sorted(self.expected.items()):
            if dst == self.rank:
                buf = torch.empty(arr, dtype=torch.float64)
                bufs[(src, dst)] = buf
                reqs.append(dist.irecv(buf, src))
        for q in reqs:
            q.wait()
        return {k: v.numpy() for k, v in bufs.items()}

    def allreduce_min(self, values):
        import torch
        import torch.distributed as dist

        t = torch.tensor([values[self.rank]], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MIN)
        return float(t[0])

    def sum_in_rank_order(self, values):
        import torch
        import torch.distributed as dist

        mine = torch.from_numpy(np.ascontiguousarray(values[self.rank], np.float64))
        parts = [torch.empty_like(mine) for _ in range(self.world)]
        dist.all_gather(parts, mine)
        out = parts[0].numpy().copy()
        for p in parts[1:]:
            out = out + p.numpy()
        return out


class SlabRun:
    """Steps the slabs of the ranks this process holds (`domains`: rank ->
    domain set up with setup()) with the halo exchanges between the halves."""

    def __init__(self, slabs, domains, transport):
        self.slabs = {s.rank: s for s in slabs}
        self.doms = domains
        self.tr = transport
        self.npe = 8

    def _recv_shapes(self, kind):
        """(src, dst) -> flat size of each message this process receives."""
        out = {}
        for r in self.doms:
            s = self.slabs[r]
            for nb in (r - 1, r + 1):
                if 0 <= nb < s.world:
                    if kind == "forces":
                        out[(nb, r)] = 2 * s.nx * s.ny * self.npe * 3
                    else:
                        out[(nb, r)] = self.node_size * s.pxy
        return out

    def _exchange(self, kind):
        sends = {}
        for r, d in self.doms.items():
            s = self.slabs[r]
            if kind == "forces":
                # my bottom owned layer to r - 1, my top owned layer to r + 1
                if r > 0:
                    sends[(r, r - 1)] = d.halo_forces(*s.layer(s.z0))
                if r < s.world - 1:
                    sends[(r, r + 1)] = d.halo_forces(*s.layer(s.z1 - 1))
            else:
                # the planes the neighbours hold as halos: z0 + 1 (of r - 1),
                # z1 - 1 (of r + 1)
                if r > 0:
                    sends[(r, r - 1)] = d.halo_nodes(*s.plane(s.z0 + 1))
                if r < s.world - 1:
                    sends[(r, r + 1)] = d.halo_nodes(*s.plane(s.z1 - 1))
        if isinstance(self.tr, DistTransport):
            self.tr.expected = self._recv_shapes(kind)
        got = self.tr.exchange(sends)
        for r, d in self.doms.items():
            s = self.slabs[r]
            for src in (r - 1, r + 1):
                if (src, r) not in got:
                    continue
                data = got[(src, r)]
                if kind == "forces":
                    k = s.z0 - 1 if src == r - 1 else s.z1
                    d.set_halo_forces(*s.layer(k), data)
                else:
                    k = s.z0 - 1 if src == r - 1 else s.z1 + 1
                    d.set_halo_nodes(*s.plane(k), data)

    def step(self, n=1):
        for _ in range(n):
            for d in self.doms.values():
                d.step_begin()
            self._exchange("forces")
            for d in self.doms.values():
                d.step_end()
            self._exchange("nodes")

    def reaction(self):
        """Reaction history summed over ranks in rank order."""
        return self.tr.sum_in_rank_order({r: d.reaction() for r, d in self.doms.items()})

    def node_vec(self, name):
        """The owned planes' values of a node field, by global plane (rank -> array)."""
        out = {}
        for r, d in self.doms.items():
            s = self.slabs[r]
            v = d.node_vec(name)
            planes = list(s.owned_planes())
            n0 = s.plane(planes[0])[0]
            n1 = s.plane(planes[-1])[1]
            out[r] = (planes[0] * s.pxy, v[n0:n1])
        return out

    @property
    def node_size(self):
        d = next(iter(self.doms.values()))
        return d.halo_nodes(0, 1).size
