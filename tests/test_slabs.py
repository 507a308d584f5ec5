"""Slab decomposition of a box mesh (weldformfem_gb300/slabs.py).

The slabs exchange element forces of their halo layers between the step
halves and node state of their halo planes after each step; every node of the
owned planes gathers all its element forces in list order, so the decomposed
run must equal the one-domain run bit for bit in positions, velocities and
displacements. The reaction is summed per rank over its owned planes and
added over ranks in rank order (bitwise equal here: only the top rank's
nodes contribute, in the same order).

CPU tests drive the FP64 oracle as the per-rank engine: in one process, and
as two gloo ranks exchanging through torch.distributed. The GPU test drives
two FP64 domains of the CUDA library in one process and compares them with
one domain of the whole mesh.
"""
import os
import socket

import numpy as np
import pytest

from oracle import orabind as O
from weldformfem_gb300 import slabs as SL
from weldformfem_gb300 import workloads as W

CASES = {"hex-reaction": (0, (4, 3, 7), 120), "die-friction": (2, (5, 4, 8), 120)}


def one_domain(engine, case, steps):
    d = engine()
    W.apply(d, case)
    d.init()
    d.run(steps) if hasattr(d, "run") else d.step(steps)
    return d


def slab_domains(engine, case, plan, dt, ranks):
    doms = {}
    for s in plan:
        if s.rank in ranks:
            d = engine()
            SL.setup(d, case, s, dt)
            d.init()
            doms[s.rank] = d
    return doms


def check_equal(run, whole, fields=("x", "v", "u")):
    for f in fields:
        ref = whole.node_vec(f)
        for _, (g0, v) in run.node_vec(f).items():
            np.testing.assert_array_equal(v, ref[g0:g0 + len(v)], err_msg=f)


def test_plan_covers_layers_and_halos():
    for nz, world in ((7, 2), (8, 3), (5, 5), (130, 4)):
        plan = SL.plan(6, 5, nz, world)
        layers = [k for s in plan for k in range(s.z0, s.z1)]
        assert layers == list(range(nz))
        for s in plan:
            assert s.lo == max(s.z0 - 1, 0) and s.hi == min(s.z1 + 1, nz)
            assert s.layer(s.z0)[0] == (s.z0 - s.lo) * 30
        planes = [k for s in plan for k in s.owned_planes()]
        assert planes == list(range(nz + 1))        # each plane's reaction counted once
    with pytest.raises(ValueError):
        SL.plan(2, 2, 3, 4)


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("world", [2, 3])
def test_oracle_slabs_in_one_process_equal_one_domain(name, world):
    cid, scale, steps = CASES[name]
    case = W.config(cid, scale=scale)
    whole = one_domain(lambda: O.OracleDomain(threads=1), case, steps)
    plan = SL.plan(*case.nel, world)
    tr = SL.LocalTransport()
    dt = case.time_step()
    hmin = tr.allreduce_min({s.rank: SL.local_min_edge(case, s) for s in plan})
    assert hmin == W.min_edge_length(case.coords(), case.elnod())  # allreduce(min) of the CFL
    run = SL.SlabRun(plan, slab_domains(lambda: O.OracleDomain(threads=1), case, plan, dt,
                                        range(world)), tr)
    run.step(steps)
    check_equal(run, whole)
    np.testing.assert_array_equal(run.reaction(), whole.reaction())


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _gloo_worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cid, scale, steps = CASES["die-friction"]
    case = W.config(cid, scale=scale)
    plan = SL.plan(*case.nel, world)
    tr = SL.DistTransport(rank, world)
    hmin = tr.allreduce_min({rank: SL.local_min_edge(case, plan[rank])})
    dt = case.dt_factor * hmin / np.sqrt(case.materials[0]["E"] / case.materials[0]["rho"])
    run = SL.SlabRun(plan, slab_domains(lambda: O.OracleDomain(threads=1), case, plan, dt,
                                        [rank]), tr)
    run.step(steps)
    out[rank] = {"u": run.node_vec("u")[rank], "reaction": run.reaction(), "dt": dt}
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_equal_one_domain():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world, port = 2, free_port()
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_gloo_worker, args=(world, port, out), nprocs=world, join=True)
    cid, scale, steps = CASES["die-friction"]
    case = W.config(cid, scale=scale)
    assert out[0]["dt"] == out[1]["dt"] == case.time_step()
    whole = one_domain(lambda: O.OracleDomain(threads=1), case, steps)
    u = whole.node_vec("u")
    for r in range(world):
        g0, v = out[r]["u"]
        np.testing.assert_array_equal(v, u[g0:g0 + len(v)])
        np.testing.assert_array_equal(out[r]["reaction"], whole.reaction())


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_gpu_mixed_slabs_equal_one_domain(name):
    """The mixed step in halves: three slabs equal one domain of the whole mesh
    run by the per-phase kernels, bit for bit in positions, velocities and
    displacements (every owned node gathers its element forces in list order,
    the halo layers' forces and the halo planes' state coming from their
    owners); the reaction is summed per rank and then in rank order."""
    import weldformfem_gb300 as wf

    cid, scale, steps = CASES[name]
    case = W.config(cid, scale=scale)

    def mixed():
        d = wf.Domain(wf.WF_MIXED)
        return d

    whole = mixed()
    W.apply(whole, case)
    whole.set_step_mode(1)
    whole.init()
    whole.run(steps)
    plan = SL.plan(*case.nel, 3)
    run = SL.SlabRun(plan, slab_domains(mixed, case, plan, case.time_step(), range(3)),
                     SL.LocalTransport())
    run.step(steps)
    check_equal(run, whole)
    assert float(np.max(np.abs(run.reaction() - whole.reaction()))) <= \
        1e-12 * float(np.max(np.abs(whole.reaction())))


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_gpu_slabs_equal_one_domain(name):
    import weldformfem_gb300 as wf

    cid, scale, steps = CASES[name]
    case = W.config(cid, scale=scale)
    whole = one_domain(lambda: wf.Domain(wf.WF_FP64), case, steps)
    plan = SL.plan(*case.nel, 3)
    run = SL.SlabRun(plan, slab_domains(lambda: wf.Domain(wf.WF_FP64), case, plan,
                                        case.time_step(), range(3)), SL.LocalTransport())
    run.step(steps)
    check_equal(run, whole)
    assert float(np.max(np.abs(run.reaction() - whole.reaction()))) <= \
        1e-12 * float(np.max(np.abs(whole.reaction())))
    # the FP64 step equals the oracle too
    o = one_domain(lambda: O.OracleDomain(threads=1), case, steps)
    np.testing.assert_allclose(whole.node_vec("u"), o.node_vec("u"), rtol=0,
                               atol=1e-9 * float(np.max(np.abs(o.node_vec("u")))))
