"""The box-mesh steps against the per-phase step (GPU): the column sweep (step
mode 4) and the dataflow step (step mode 5).

Both compute every element force with the per-phase element arithmetic and
add each node's eight element forces in list order (the sweep: the four of the
layer below carried from the previous layer, then the four of the layer
above; the dataflow step: the per-phase node gather itself), so positions,
velocities, accelerations, displacements, tau and eps_p must equal the
per-phase run (mode 1) bit for bit; the reaction history is summed over the
nodes in another order and is held to 1e-12. The sweep reads one buffer of
each pair it shares with neighbouring columns and writes the other, and the
dataflow step counts in one of two counter sets: runs of every length (direct
launches, graph remainders of odd and even length, 32-step graphs) and
switches of mode between runs must use the current ones.
"""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from tests import helpers as H
from weldformfem_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CASES = {
    # 41 x 37 nodes per plane: 2 x 5 columns of 8 rows, rings on both sides
    "die-contact-friction": lambda: W.config(2, scale=(40, 36, 24)),
    "cube-hourglass-plastic": lambda: W.config(0, scale=(20, 20, 20)),
    "octants": lambda: W.config(4, scale=(16, 16, 16)),
    # 71 nodes along x: three columns of 23-24 nodes; three element layers
    "wide-thin": lambda: W.config(2, scale=(70, 9, 3)),
}


GMT_MAT = dict(model=3, E=200e9, nu=0.3, rho=7850.0, sy0=250e6)
GMT = dict(c=[-2e-4, 0.2, 1200e6, -1.5e-3, 1e-4, 0.02, -1e-5, -2e-3],
           range=[0.01, 2.0, 1e-2, 1e5, 0.0, 1500.0], T=300.0)


def run(case, mode, steps, rows=8, hollomon=False, energy=False, runs=None, flow=None,
        gmt=False):
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, case)
    if hollomon:
        d.set_materials([H.HOLLOMON])
    if gmt:
        d.set_materials([GMT_MAT])
        d.set_gmt(0, GMT["c"], GMT["range"], GMT["T"])
    if energy:
        d.set_energy_history(True)
    d.set_sweep_rows(rows)
    if flow:
        d.set_flow_tiles(*flow)
    d.set_step_mode(mode)
    d.init()
    for n in (runs or [steps]):
        d.run(n)
    d.sync()
    return d


def assert_same_state(a, b, fields=("x", "v", "u", "a")):
    for f in fields:
        np.testing.assert_array_equal(a.node_vec(f), b.node_vec(f), err_msg=f)
    np.testing.assert_array_equal(a.elem_scalar("pl_strain"), b.elem_scalar("pl_strain"))
    np.testing.assert_array_equal(a.elem_tensor("tau"), b.elem_tensor("tau"))
    assert H.rel_err(a.reaction(), b.reaction()) <= 1e-12


@pytest.mark.parametrize("rows", [8, 4])
@pytest.mark.parametrize("name", list(CASES))
def test_sweep_equals_per_phase_bitwise(name, rows):
    case = CASES[name]()
    s = run(case, 4, 300, rows=rows)
    p = run(case, 1, 300)
    assert s.step_mode()[0] == 4 and p.step_mode()[0] == 1
    cx, cy, r, why = s.sweep()
    nx, ny, _ = case.nel
    assert why == "" and r == rows
    assert cx == -(-(nx + 1) // 31) and cy == -(-(ny + 1) // rows)
    assert s.step_mode()[1:] == (cx * cy, 32 * (rows + 1))
    assert_same_state(s, p)


@pytest.mark.parametrize("flow", [(512, 4), (256, 1), (2048, 8)], ids=str)
@pytest.mark.parametrize("name", list(CASES))
def test_flow_equals_per_phase_bitwise(name, flow):
    case = CASES[name]()
    f = run(case, 5, 300, flow=flow)
    p = run(case, 1, 300)
    assert f.step_mode()[0] == 5
    tiles, grid, why = f.flow()
    nx, ny, nz = case.nel
    exy, pxy, t = nx * ny, (nx + 1) * (ny + 1), flow[0]

    def cdiv(a, b):
        return -(-a // b)
    # element and node-update tiles (the geometry and nodal phases run as
    # their own kernels before the launch)
    want = nz * cdiv(exy, t) + (nz + 1) * cdiv(pxy, t)
    assert why == "" and tiles == want and grid > 0
    assert f.step_mode()[1:] == (grid, 256)
    assert_same_state(f, p)


@pytest.mark.parametrize("mode", [4, 5])
@pytest.mark.parametrize("law", ["hollomon", "gmt"])
def test_general_law_equals_per_phase_bitwise(mode, law):
    case = W.config(0, scale=(12, 12, 12))
    case.top_vz = -20.0
    s = run(case, mode, 400, **{law: True})
    p = run(case, 1, 400, **{law: True})
    assert s.elem_scalar("pl_strain").max() > 0.0
    assert_same_state(s, p)


@pytest.mark.parametrize("mode", [4, 5])
def test_run_lengths_and_parity(mode):
    """Runs of 1 step (direct launch), odd and even graph remainders and
    32-step graphs: each leaves the state in the buffers, and the counters in
    the set, that the next run uses."""
    case = CASES["die-contact-friction"]()
    runs = [1, 2, 37, 64, 5, 1, 33]
    s = run(case, mode, 0, runs=runs)
    p = run(case, 1, sum(runs))
    assert_same_state(s, p)
    # a readback between runs of odd length reads the current buffers
    s2 = run(case, mode, 0, runs=[3])
    p2 = run(case, 1, 3)
    np.testing.assert_array_equal(s2.node_vec("x"), p2.node_vec("x"))
    s2.run(6)
    p2.run(6)
    assert_same_state(s2, p2)


def test_mode_switches_between_runs():
    case = CASES["cube-hourglass-plastic"]()
    s = wf.Domain(wf.WF_MIXED)
    W.apply(s, case)
    s.init()
    for mode, n in ((4, 11), (1, 7), (5, 21), (4, 3), (5, 5), (1, 3), (0, 9)):
        s.set_step_mode(mode)
        s.run(n)
    s.sync()
    p = run(case, 1, 59)
    assert_same_state(s, p)


@pytest.mark.parametrize("mode", [4, 5])
def test_energy_history(mode):
    case = CASES["cube-hourglass-plastic"]()
    s = run(case, mode, 120, energy=True)
    p = run(case, 1, 120, energy=True)
    assert_same_state(s, p)
    es, ep = s.energies(), p.energies()
    for a, b in zip(es, ep):
        np.testing.assert_array_equal(np.asarray(a), np.asarray(b))


def test_selection():
    # 257 x 257 nodes per plane (C2's): 9 x 33 columns, enough to fill the GPU
    wide = W.config(0, scale=(256, 256, 2))
    w = wf.Domain(wf.WF_MIXED)
    W.apply(w, wide)
    w.init()
    assert w.step_mode()[0] == 4                   # automatic: the column sweep
    big = W.config(0, scale=(16, 16, 16))          # above the cluster run's 3000 elements
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, big)
    d.init()
    assert d.sweep()[:2] == (1, 3)                 # swept, but 3 columns leave the GPU idle:
    assert d.step_mode()[0] == 1                   # automatic: the per-phase kernels
    d.set_step_mode(4)
    assert d.step_mode()[0] == 4
    d.set_step_mode(5)
    assert d.step_mode()[0] == 5
    d.set_step_mode(1)
    assert d.step_mode()[0] == 1
    f = wf.Domain(wf.WF_FP64)
    W.apply(f, big)
    f.init()
    assert f.step_mode()[0] == 1 and f.sweep()[0] == 0 and f.flow()[0] == 0
    for mode in (4, 5):
        f.set_step_mode(mode)
        with pytest.raises(wf.WfError) as e:
            f.run(1)
        assert e.value.status == wf.WF_ERR_UNSUPPORTED
    # tetrahedra and a renumbered mesh have neither
    t = wf.Domain(wf.WF_MIXED)
    W.apply(t, W.config(1, scale=(6, 5, 8)))
    t.init()
    assert t.sweep()[0] == 0 and "box" in t.sweep()[3]
    assert t.flow()[0] == 0 and "box" in t.flow()[2]
    x = big.coords()
    el = big.elnod()[::-1].copy()
    r = wf.Domain(wf.WF_MIXED)
    r.set_mesh(x, el)
    W.apply_options(r, big, x=x)
    r.set_step_mode(5)
    r.init()
    assert r.step_mode()[0] == 1 and "box" in r.flow()[2]
    for mode in (4, 5):
        r.set_step_mode(mode)
        with pytest.raises(wf.WfError) as e:
            r.run(1)
        assert e.value.status == wf.WF_ERR_UNSUPPORTED
    with pytest.raises(wf.WfError):
        d.set_sweep_rows(4)                         # after init
    with pytest.raises(wf.WfError):
        d.set_flow_tiles(512, 4)
    n = wf.Domain(wf.WF_MIXED)
    with pytest.raises(wf.WfError):
        n.set_sweep_rows(6)
    for bad in ((300, 4), (128, 4), (512, 0), (512, 17)):
        with pytest.raises(wf.WfError):
            n.set_flow_tiles(*bad)


@pytest.mark.parametrize("nel", [(1, 1, 5), (31, 1, 3), (30, 7, 2), (32, 9, 1), (2, 40, 3),
                                 (62, 17, 2)], ids=str)
@pytest.mark.parametrize("mode", [4, 5])
def test_ragged_and_thin_boxes(nel, mode):
    """Columns of one node, a single element layer, rows that end mid-column,
    widths at the 31-node column limit and just past it: the sweep and the
    dataflow step still equal the per-phase step bit for bit."""
    case = W.config(0, scale=nel)
    s = run(case, mode, 60)
    p = run(case, 1, 60)
    assert s.step_mode()[0] == mode
    assert_same_state(s, p)
