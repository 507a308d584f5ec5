"""Batched ensemble (config 3): many independent specimens in one domain.

Each specimen is a disjoint sub-mesh with its own material, time step, BCs
and reaction history, and all specimens step in the same launches. Every
node and element computes exactly what it computes in a domain of its own,
so the batched displacements must equal the one-domain-per-specimen runs bit
for bit (both precisions); the per-specimen reaction sums are formed in a
different order and are held to 1e-12. The FP64 batch is also checked
against the oracle specimen by specimen (1e-9, the FP64 parity bar).
"""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from oracle import orabind as O
from tests import helpers as H
from weldformfem_gb300 import workloads as W


def small_ensemble():
    return W.ensemble(n_spec=5, nmin=2, nmax=6, steps=150)


def test_ensemble_generator():
    b = W.ensemble(n_spec=64)
    ns = [c.nel[0] for c in b.cases]
    assert min(ns) >= 6 and max(ns) <= 40 and len(set(ns)) > 10
    assert all(c.nel[0] == c.nel[1] == c.nel[2] for c in b.cases)
    b2 = W.ensemble(n_spec=64)
    assert [c.materials[0]["E"] for c in b.cases] == [c.materials[0]["E"] for c in b2.cases]
    Es = np.array([c.materials[0]["E"] for c in b.cases])
    assert Es.min() >= 70e9 and Es.max() <= 210e9
    x, el, emat, bcs, tops, eoff, noff = small_ensemble().assemble()
    assert el.max() < x.shape[0] and eoff[-1] == el.shape[0] and noff[-1] == x.shape[0]
    for s in range(len(eoff) - 1):
        block = el[eoff[s]:eoff[s + 1]]
        assert block.min() >= noff[s] and block.max() < noff[s + 1]


def solo(case, prec, steps):
    d = wf.Domain(prec)
    W.apply(d, case)
    d.init()
    d.run(steps)
    return d


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [wf.WF_FP64, wf.WF_MIXED], ids=["fp64", "mixed"])
def test_batched_equals_one_domain_per_specimen(prec):
    b = small_ensemble()
    steps = 150
    d = wf.Domain(prec)
    dts = W.apply_batch(d, b)
    d.init()
    d.run(steps)
    u = d.node_vec("u")
    _, noff = b.offsets()
    for s, c in enumerate(b.cases):
        c.dt = float(dts[s])
        one = solo(c, prec, steps)
        np.testing.assert_array_equal(u[noff[s]:noff[s + 1]], one.node_vec("u"))
        r = d.specimen_reaction(s)
        assert r.shape == (steps,)
        assert H.rel_err(r, one.reaction()) <= 1e-12


@pytest.mark.gpu
def test_batched_fp64_matches_oracle():
    b = small_ensemble()
    steps = 150
    d = wf.Domain(wf.WF_FP64)
    dts = W.apply_batch(d, b)
    d.init()
    d.run(steps)
    u = d.node_vec("u")
    pl = d.elem_scalar("pl_strain")
    eoff, noff = b.offsets()
    for s, c in enumerate(b.cases):
        c.dt = float(dts[s])
        o = O.OracleDomain()
        W.apply(o, c)
        o.init()
        o.step(steps)
        assert H.rel_err(u[noff[s]:noff[s + 1]], o.node_vec("u")) <= 1e-9
        assert H.rel_err(pl[eoff[s]:eoff[s + 1]], o.elem_scalar("pl_strain")) <= 1e-9
        assert H.rel_err(d.specimen_reaction(s), o.reaction()) <= 1e-9


@pytest.mark.gpu
def test_batched_fp64_config3_slice_matches_oracle():
    """The first 32 specimens of the config-3 ensemble itself (n ~ U{6..40},
    per-specimen materials and top velocities), 400 steps, FP64 against the
    oracle run of each specimen on its own."""
    full = W.ensemble(n_spec=1024)
    b = W.Batch(full.name, full.cases[:32], full.hg)
    steps = 400
    d = wf.Domain(wf.WF_FP64)
    dts = W.apply_batch(d, b)
    d.init()
    d.run(steps)
    u = d.node_vec("u")
    pl = d.elem_scalar("pl_strain")
    eoff, noff = b.offsets()
    assert eoff[-1] > 200000
    for s, c in enumerate(b.cases):
        c.dt = float(dts[s])
        o = O.OracleDomain()
        W.apply(o, c)
        o.init()
        o.step(steps)
        assert H.rel_err(u[noff[s]:noff[s + 1]], o.node_vec("u")) <= 1e-9, s
        assert H.rel_err(pl[eoff[s]:eoff[s + 1]], o.elem_scalar("pl_strain")) <= 1e-9, s
        assert H.rel_err(d.specimen_reaction(s), o.reaction()) <= 1e-9, s


@pytest.mark.gpu
def test_batched_rejects_bad_tables():
    b = small_ensemble()
    x, el, emat, bcs, tops, eoff, noff = b.assemble()
    d = wf.Domain(wf.WF_MIXED)
    d.set_mesh(x, el)
    bad = noff.copy()
    bad[1] -= 1                      # specimen 0's last node now belongs to specimen 1
    with pytest.raises(wf.WfError) as e:
        d.set_specimens(eoff, bad, b.dts())
    assert e.value.status == 1


@pytest.mark.gpu
def test_specimen_shards_equal_the_whole_batch():
    """bench.py's C3 sharding: each rank runs a contiguous block of the
    specimens as its own batched domain. Every specimen computes exactly what
    it computes in the whole batch, so the shards' displacements and
    per-specimen reactions equal the whole batch's bit for bit."""
    import bench

    full = W.ensemble(n_spec=9, nmin=3, nmax=7, steps=120)
    steps = 120
    whole = wf.Domain(wf.WF_MIXED)
    W.apply_batch(whole, full)
    whole.init()
    whole.run(steps)
    u = whole.node_vec("u")
    _, noff = full.offsets()
    world = 2
    for rank in range(world):
        lo, hi = bench.shard(len(full.cases), rank, world)
        part = W.Batch(full.name, full.cases[lo:hi], full.hg)
        d = wf.Domain(wf.WF_MIXED)
        W.apply_batch(d, part)
        d.init()
        d.run(steps)
        np.testing.assert_array_equal(d.node_vec("u"), u[noff[lo]:noff[hi]])
        for s in range(hi - lo):
            np.testing.assert_array_equal(d.specimen_reaction(s), whole.specimen_reaction(lo + s))
