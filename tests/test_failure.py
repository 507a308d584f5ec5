"""Non-finite force detection reaches the caller (GPU).

The reference loop clears a non-finite assembled internal force to zero and
prints it (src/explicit/Solver_explicit.C:777-785). The node kernels clear it
the same way and raise a device flag with the smallest offending node id;
the first wf_sync after the run reports WF_ERR_NONFINITE and clears the flag.
The failure is made on the host: a NaN prescribed velocity or a NaN
coordinate goes in through the public entry points. Nothing faults on the
GPU: the kernels only compute with NaN values.
"""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from weldformfem_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def small_case():
    return W.config(0, scale=(4, 4, 4))


@pytest.mark.parametrize("prec", [wf.WF_FP64, wf.WF_MIXED], ids=["fp64", "mixed"])
def test_clean_run_syncs_ok(prec):
    d = wf.Domain(prec)
    W.apply(d, small_case())
    d.init()
    d.run(40)
    d.sync()                          # no exception: nothing was cleared
    assert np.all(np.isfinite(d.node_vec("u")))


@pytest.mark.parametrize("prec,mode", [(wf.WF_FP64, 1), (wf.WF_MIXED, 1), (wf.WF_MIXED, 2),
                                       (wf.WF_MIXED, 4), (wf.WF_MIXED, 5)],
                         ids=["fp64", "mixed-per-phase", "mixed-cluster", "mixed-sweep",
                              "mixed-flow"])
def test_nan_velocity_bc_is_reported(prec, mode):
    case = small_case()
    d = wf.Domain(prec)
    d.add_box(case.L, case.r, case.tritetra)
    nodes, dims, vals = case.bcs()
    top = case.top_nodes()
    bad = int(top[len(top) // 2])
    sel = np.nonzero((nodes == bad) & (dims == 2))[0]
    assert sel.size == 1
    vals = vals.copy()
    vals[sel[0]] = np.nan
    W.apply_options(d, case, with_bcs=False)
    d.add_bcs((nodes, dims, vals))
    if prec == wf.WF_MIXED:
        d.set_step_mode(mode)
    d.init()
    d.run(5)                          # queued: the run itself reports nothing yet
    with pytest.raises(wf.WfError) as e:
        d.sync()
    assert e.value.status == wf.WF_ERR_NONFINITE
    msg = str(e.value)
    assert "node" in msg
    first = int(msg.split("first at node ")[1].split(")")[0])
    # the smallest node of an element around the NaN node
    assert 0 <= first <= bad
    # reported once: a sync with no run in between is clean
    d.sync()
    # the cleared forces keep the state as the reference leaves it; more
    # steps raise the flag again
    d.run(2)
    with pytest.raises(wf.WfError) as e:
        d.sync()
    assert e.value.status == wf.WF_ERR_NONFINITE


def test_nan_coordinate_is_reported_by_solve():
    case = small_case()
    x = case.coords()
    x[len(x) // 2, 0] = np.nan        # an interior node
    d = wf.Domain(wf.WF_FP64)
    d.add_box(case.L, case.r, case.tritetra)
    d.set_nodes(x)
    W.apply_options(d, case, x=case.coords())
    d.init()
    d.set_end_time(3.5 * case.time_step())
    with pytest.raises(wf.WfError) as e:
        d.solve()                      # wf_solve syncs and reports
    assert e.value.status == wf.WF_ERR_NONFINITE
