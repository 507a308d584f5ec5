"""Node-to-element lists of meshes large enough for the multithreaded host
build (element chunks counted and placed in element order) and for the
device build of wf_init (count, scan, atomic placement, per-list sort): both
identical to a stable sort of the element-node entries by node, i.e.
element-ascending lists as setNodElem builds them (Domain_d.C:1508-1611).
Before wf_init the lists come from the host build, after it from the device
tables."""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from weldformfem_gb300 import workloads as W


def expected(flat, npe, nn):
    order = np.argsort(flat, kind="stable")
    cnt = np.bincount(flat, minlength=nn)
    return order // npe, order % npe, np.concatenate([[0], np.cumsum(cnt)[:-1]]), cnt


def check(d, flat, npe, nn):
    elnod, nodel, loc, off, cnt = d.conn()
    np.testing.assert_array_equal(elnod.reshape(-1), flat)
    for got, want in zip((nodel, loc, off, cnt), expected(flat, npe, nn)):
        np.testing.assert_array_equal(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("cid,scale", [(0, (110, 110, 100)), (1, (100, 100, 110))])
def test_node_lists_of_a_large_mesh(cid, scale):
    c = W.config(cid, scale=scale)
    flat = c.elnod().reshape(-1)
    npe = c.elnod().shape[1]
    assert c.n_node > (1 << 20)      # several host chunks, many scan tiles
    d = wf.Domain(wf.WF_MIXED)
    d.set_mesh(c.coords(), c.elnod())
    check(d, flat, npe, c.n_node)     # host build
    d = wf.Domain(wf.WF_MIXED)
    d.set_mesh(c.coords(), c.elnod())
    W.apply_options(d, c)
    d.set_autotune(False)
    d.init()
    check(d, flat, npe, c.n_node)     # device build


@pytest.mark.gpu
def test_device_lists_of_a_renumbered_mesh():
    """Nodes renumbered at random and elements shuffled: lists of uneven
    length whose entries the atomic placement scatters; the sort restores the
    element-ascending order, and the FP64 displacements stay bitwise the
    oracle's (the node gathers add in list order)."""
    from oracle import orabind as O

    c = W.config(1, scale=(6, 5, 7))
    rng = np.random.default_rng(W.SEED_BASE + 31)
    x, el = c.coords(), c.elnod()
    perm = rng.permutation(c.n_node)          # new id of each node
    inv = np.argsort(perm)
    x2 = x[inv]
    el2 = perm[el][rng.permutation(el.shape[0])].astype(np.int32)
    npe = el2.shape[1]
    bcs = [(int(perm[n]), int(k), float(v)) for n, k, v in zip(*c.bcs())]
    dt = c.time_step(x)

    def setup(dom):
        dom.set_mesh(x2, el2)
        dom.set_materials(c.materials)
        dom.add_bcs(bcs)
        dom.set_reaction_nodes(perm[c.top_nodes()].astype(np.int32), 2)
        dom.set_dt(dt)
        dom.init()
        return dom

    d = setup(wf.Domain(wf.WF_FP64))
    check(d, el2.reshape(-1), npe, c.n_node)
    o = setup(O.OracleDomain())
    for dom in (d, o):
        dom.step(40)
    np.testing.assert_array_equal(d.node_vec("u"), o.node_vec("u"))
    # the reaction is a reduction over the node set (the device adds block
    # partials, the oracle adds in list order): equal to rounding
    np.testing.assert_allclose(d.reaction(), o.reaction(), rtol=1e-13, atol=0)


@pytest.mark.gpu
def test_set_mesh_rejects_unknown_nodes_and_lists_follow_a_new_mesh():
    c = W.config(0, scale=(3, 3, 3))
    x, el = c.coords(), c.elnod()
    d = wf.Domain(wf.WF_MIXED)
    for v in (c.n_node, -1):
        bad = el.copy()
        bad[5, 2] = v
        with pytest.raises(wf.WfError) as e:
            d.set_mesh(x, bad)
        assert e.value.status == wf.WF_ERR_ARG
    d.set_mesh(x, el)
    check(d, el.reshape(-1), 8, c.n_node)
    el2 = np.ascontiguousarray(el[::-1])          # same node count, other lists
    d.set_mesh(x, el2)
    check(d, el2.reshape(-1), 8, c.n_node)
