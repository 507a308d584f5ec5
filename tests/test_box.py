"""Box-mesh indexing of the mixed per-phase kernels (GPU).

On a mesh in the AddBoxLength numbering the geometry, nodal, element and node
kernels compute element corners and node lists from the indices instead of
reading the connectivity and list arrays. The lists come out in the same
(element-ascending) order and every sum runs in that order, so the run must
equal the run that reads the arrays bit for bit, reaction history included.
"""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from tests import helpers as H
from weldformfem_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CASES = {
    "die-contact": lambda: W.config(2, scale=(40, 36, 24)),
    "cube-hourglass-plastic": lambda: W.config(0, scale=(20, 20, 20)),
    "octants": lambda: W.config(4, scale=(16, 16, 16)),
}


def run(case, box, steps, set_mesh=False, hollomon=False, mode=1):
    d = wf.Domain(wf.WF_MIXED)
    if set_mesh:
        x = case.coords()
        d.set_mesh(x, case.elnod())
        W.apply_options(d, case, x=x)
    else:
        W.apply(d, case)
    if hollomon:
        d.set_materials([H.HOLLOMON])
    d.set_box_indexing(box)
    d.set_step_mode(mode)
    d.init()
    d.run(steps)
    d.sync()
    return d


@pytest.mark.parametrize("name", list(CASES))
def test_box_indexing_equals_arrays_bitwise(name):
    case = CASES[name]()
    a = run(case, True, 300)
    b = run(case, False, 300)
    assert a.box() == case.nel and b.box() == (0, 0, 0)
    for f in ("x", "v", "u", "a"):
        np.testing.assert_array_equal(a.node_vec(f), b.node_vec(f), err_msg=f)
    np.testing.assert_array_equal(a.elem_scalar("pl_strain"), b.elem_scalar("pl_strain"))
    np.testing.assert_array_equal(a.reaction(), b.reaction())


def test_box_indexing_general_law_and_uploaded_mesh():
    case = W.config(0, scale=(12, 12, 12))
    a = run(case, True, 800, set_mesh=True, hollomon=True)
    b = run(case, False, 800, hollomon=True)
    assert a.box() == (12, 12, 12)
    assert a.elem_scalar("pl_strain").max() > 0.0
    for f in ("x", "v", "u"):
        np.testing.assert_array_equal(a.node_vec(f), b.node_vec(f), err_msg=f)


def test_box_indexing_in_tiled_steps():
    """The tiled step's shared-node kernel indexes the box too."""
    case = W.config(2, scale=(24, 20, 16))
    a = run(case, True, 200, mode=3)
    b = run(case, False, 200, mode=1)
    for f in ("x", "v", "u"):
        np.testing.assert_array_equal(a.node_vec(f), b.node_vec(f), err_msg=f)


def test_non_box_numbering_reads_the_arrays():
    case = W.config(0, scale=(8, 8, 8))
    x = case.coords()
    el = case.elnod()[::-1].copy()          # elements listed backwards: not the box numbering
    d = wf.Domain(wf.WF_MIXED)
    d.set_mesh(x, el)
    W.apply_options(d, case, x=x)
    d.init()
    assert d.box() == (0, 0, 0)
    d.run(10)
    d.sync()
    t = wf.Domain(wf.WF_MIXED)
    W.apply(t, W.config(1, scale=(4, 4, 4)))
    t.init()
    assert t.box() == (0, 0, 0)             # tetrahedra


@pytest.mark.parametrize("cid,scale", [(2, (40, 36, 24)), (0, (20, 20, 20)), (2, (70, 9, 3))])
def test_min_edge_length_over_grid_edges_equals_element_edges(cid, scale):
    """Box meshes take the shortest edge over the grid edges (each once); the
    value is the element loop's bit for bit, and the oracle's."""
    case = W.config(cid, scale=scale)
    a = run(case, True, 0)
    b = run(case, False, 0)
    assert a.box() == case.nel and b.box() == (0, 0, 0)
    ha, hb = a.min_edge_length(), b.min_edge_length()
    assert ha == hb
    assert ha == W.min_edge_length(case.coords(), case.elnod())


def test_node_vec_into_caller_buffer():
    case = W.config(0, scale=(6, 6, 6))
    d = run(case, True, 30)
    want = d.node_vec("u")
    buf = np.full(case.n_node * 3, np.nan)
    got = d.node_vec("u", out=buf)
    assert got.base is buf or got is buf or np.shares_memory(got, buf)
    np.testing.assert_array_equal(got, want)
    with pytest.raises(ValueError):
        d.node_vec("u", out=np.zeros(case.n_node * 3, np.float32))


def test_direct_displacement_readback_equals_export():
    """Mixed positions and displacements read straight from the state equal
    those of the full FP64 export bit for bit."""
    case = W.config(2, scale=(24, 20, 16))
    d = run(case, True, 40)
    u1, x1 = d.node_vec("u"), d.node_vec("x")      # direct
    d.elem_scalar("pl_strain")                       # exports every field
    np.testing.assert_array_equal(d.node_vec("u"), u1)
    np.testing.assert_array_equal(d.node_vec("x"), x1)
