"""Node-to-element lists of a mesh large enough for the multithreaded host
build (each thread owns a node range and scans the connectivity in element
order): identical to a stable sort of the element-node entries by node, i.e.
element-ascending lists as setNodElem builds them (Domain_d.C:1508-1611)."""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from weldformfem_gb300 import workloads as W


@pytest.mark.gpu
@pytest.mark.parametrize("cid,scale", [(0, (110, 110, 100)), (1, (100, 100, 110))])
def test_node_lists_of_a_large_mesh(cid, scale):
    c = W.config(cid, scale=scale)
    d = wf.Domain(wf.WF_MIXED)
    d.set_mesh(c.coords(), c.elnod())
    elnod, nodel, loc, off, cnt = d.conn()
    flat = c.elnod().reshape(-1)
    npe = c.elnod().shape[1]
    assert c.n_node > (1 << 20)      # at least two node ranges
    order = np.argsort(flat, kind="stable")
    np.testing.assert_array_equal(nodel, order // npe)
    np.testing.assert_array_equal(loc, order % npe)
    np.testing.assert_array_equal(cnt, np.bincount(flat, minlength=c.n_node))
    np.testing.assert_array_equal(off, np.concatenate([[0], np.cumsum(cnt)[:-1]]))
