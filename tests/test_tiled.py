"""Tiled element + assembly step (step mode 3) against the per-phase step (GPU).

On meshes numbered like AddBoxLength's, the tiled kernels sum every node's
element forces in the per-phase gather's order and use the same element and
node arithmetic, so positions, velocities and displacements must equal the
per-phase run bit for bit; the reaction history is summed over the nodes in
another order and is held to 1e-12. On a renumbered mesh the interior sums
run in corner order instead of list order: the result is then compared with
the FP64 oracle under the mixed-precision bounds of tests/test_mixed.py, and
two tiled runs must agree bit for bit (determinism).
"""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from oracle import orabind as O
from tests import helpers as H
from weldformfem_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CASES = {
    "die-contact": lambda: W.config(2, scale=(24, 20, 16)),
    "cube-hourglass-plastic": lambda: W.config(0, scale=(16, 16, 16)),
    "octants": lambda: W.config(4, scale=(16, 16, 16)),
}


def run(case, mode, steps, x=None, elnod=None, hollomon=False):
    d = wf.Domain(wf.WF_MIXED)
    if elnod is None:
        W.apply(d, case, x=x)
    else:
        d.set_mesh(x, elnod)
        W.apply_options(d, case, x=x)
    if hollomon:
        d.set_materials([H.HOLLOMON])
    d.set_step_mode(mode)
    d.init()
    d.run(steps)
    d.sync()
    return d


@pytest.mark.parametrize("name", list(CASES))
def test_tiled_equals_per_phase_bitwise(name):
    case = CASES[name]()
    steps = 300
    t = run(case, 3, steps)
    p = run(case, 1, steps)
    assert t.step_mode()[0] == 3 and p.step_mode()[0] == 1
    ntiles, nshared, why = t.tiles()
    assert ntiles > 0 and nshared > 0 and why == ""
    for f in ("x", "v", "u", "a"):
        np.testing.assert_array_equal(t.node_vec(f), p.node_vec(f), err_msg=f)
    np.testing.assert_array_equal(t.elem_scalar("pl_strain"), p.elem_scalar("pl_strain"))
    np.testing.assert_array_equal(t.elem_tensor("tau"), p.elem_tensor("tau"))
    assert H.rel_err(t.reaction(), p.reaction()) <= 1e-12


def test_tiled_general_law_equals_per_phase_bitwise():
    case = W.config(0, scale=(12, 12, 12))
    t = run(case, 3, 800, hollomon=True)
    p = run(case, 1, 800, hollomon=True)
    assert t.elem_scalar("pl_strain").max() > 0.0
    for f in ("x", "v", "u"):
        np.testing.assert_array_equal(t.node_vec(f), p.node_vec(f), err_msg=f)


def test_tile_counts():
    case = W.config(2, scale=(24, 20, 16))
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, case)
    d.set_step_mode(3)
    d.init()
    mode, ntiles, threads = d.step_mode()
    assert mode == 3 and ntiles == d.tiles()[0] and threads == 512
    # 24 x 20 x 16 cells in cubes of 8: 3 x 3 x 2 bins, the y row of 20 cut 8 + 8 + 4
    assert ntiles == 18


def renumbered(case, seed=7):
    """The case's mesh with nodes and elements renumbered by a seeded shuffle."""
    rng = np.random.default_rng(seed)
    x = case.coords()
    el = case.elnod()
    pn = rng.permutation(x.shape[0])        # new id of old node i: inv[i]
    inv = np.empty_like(pn)
    inv[pn] = np.arange(pn.size)
    pe = rng.permutation(el.shape[0])
    return x[pn], inv[el[pe]].astype(np.int32), pn


def test_renumbered_mesh_tiles_and_matches_fp64():
    """Frictionless die (with friction the FP32 and FP64 runs part ways in the
    sliding direction, see tests/test_mixed.py), renumbered nodes and elements."""
    case = W.config(2, scale=(24, 20, 16))
    case.contact = dict(case.contact, mu=0.0)
    x, el, pn = renumbered(case)
    case_r = case
    steps = 200
    # BCs, reaction and contact nodes follow the renumbering: set them by hand
    nodes, dims, vals = case.bcs()
    inv = np.empty_like(pn)
    inv[pn] = np.arange(pn.size)

    def setup(dom):
        dom.set_mesh(x, el)
        dom.set_materials(case_r.materials)
        dom.add_bcs((inv[nodes], dims, vals))
        dom.set_hourglass(case_r.hg)
        cp = case_r.contact_params()
        dom.set_contact_plane(cp["z0"], cp["vz"], cp["kpen"], cp["mu"], inv[case.top_nodes()])
        dom.set_dt(case.time_step())

    runs = []
    for _ in range(2):
        d = wf.Domain(wf.WF_MIXED)
        setup(d)
        d.set_step_mode(3)
        d.init()
        assert d.tiles()[0] > 0
        d.run(steps)
        runs.append(d)
    np.testing.assert_array_equal(runs[0].node_vec("u"), runs[1].node_vec("u"))
    np.testing.assert_array_equal(runs[0].reaction(), runs[1].reaction())
    o = O.OracleDomain()
    setup(o)
    o.init()
    o.step(steps)
    assert H.rel_err(runs[0].node_vec("u"), o.node_vec("u")) <= 1e-4
    assert H.rel_err(runs[0].reaction(), o.reaction()) <= 1e-3


def test_rotated_element_is_not_tiled_and_falls_back():
    """An element whose nodes are listed from another corner shares a node
    with a neighbour at the same corner index: the mesh is not tiled, a tiled
    run is refused and the automatic mode runs the per-phase kernels."""
    case = W.config(0, scale=(16, 16, 16))
    x = case.coords()
    el = case.elnod().copy()
    e = 16 * 16 * 8 + 16 * 8 + 8
    el[e] = el[e][[1, 2, 3, 0, 5, 6, 7, 4]]     # the same hexahedron, turned about z
    d = wf.Domain(wf.WF_MIXED)
    d.set_mesh(x, el)
    W.apply_options(d, case, x=x)
    d.set_step_mode(3)
    d.init()
    ntiles, _, why = d.tiles()
    assert ntiles == 0 and "same corner" in why
    assert d.step_mode()[0] == 1            # reported: the kernels a run could use
    with pytest.raises(wf.WfError) as err:
        d.run(1)
    assert err.value.status == wf.WF_ERR_UNSUPPORTED
    d.set_step_mode(0)                      # automatic: per-phase kernels
    d.run(20)
    d.sync()


def test_tiles_are_built_only_for_mode_3():
    case = W.config(0, scale=(16, 16, 16))
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, case)
    d.init()
    assert d.tiles()[0] == 0 and "step mode 3" in d.tiles()[2]


def test_tetrahedra_are_not_tiled():
    case = W.config(1, scale=(6, 5, 8))
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, case)
    d.init()
    assert d.tiles() == (0, 0, "tetrahedra")
    assert d.step_mode()[0] in (1, 2)


def test_tiled_phase_timing_and_graph_runs_agree():
    case = W.config(2, scale=(24, 20, 16))
    a = run(case, 3, 70)                     # graphs of 32 + 32 + 6 steps
    b = wf.Domain(wf.WF_MIXED)
    W.apply(b, case)
    b.set_step_mode(3)
    b.init()
    b.set_phase_timing(True)                 # direct launches with events
    b.run(70)
    ms, n = b.phase_times()
    assert n == 70 and np.all(ms > 0)
    np.testing.assert_array_equal(a.node_vec("u"), b.node_vec("u"))
    np.testing.assert_array_equal(a.reaction(), b.reaction())
