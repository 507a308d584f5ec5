"""Single-cluster runs of the mixed-precision step (wf_set_step_mode 2).

A whole run is one launch of one thread-block cluster whose blocks own fixed
element and node ranges and meet at cluster barriers between the phases. The
per-element and per-node arithmetic is the per-phase kernels', so the state
after N steps must be bitwise the per-phase (graph) run's; the reaction is
summed in another order (FP64 sums of FP32 contributions), 1e-12 relative.
"""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from tests import helpers as H
from weldformfem_gb300 import workloads as W


def cases():
    c0 = W.config(0)                       # 10^3 hexahedra, hourglass, symmetry + top velocity
    tet = W.config(1, scale=(6, 6, 8))     # 1728 perturbed tetrahedra
    die = W.config(2, scale=(12, 12, 6))   # 864 perturbed hexahedra, rigid plane die
    hol = W.config(0, scale=(7, 9, 11))
    hol.materials = [dict(model=1, E=200e9, nu=0.3, rho=7850.0, sy0=300e6, hol_K=600e6,
                          hol_m=0.2)]
    return {"c0": (c0, 400), "tet": (tet, 300), "die": (die, 300), "hollomon": (hol, 300)}


def run(case, steps, mode):
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, case)
    d.set_step_mode(mode)
    d.init()
    d.run(steps // 2)
    d.run(steps - steps // 2)        # two runs: the state carries across launches
    return d


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c0", "tet", "die", "hollomon"])
def test_cluster_run_matches_per_phase_kernels(name):
    case, steps = cases()[name]
    a = run(case, steps, 1)
    b = run(case, steps, 2)
    assert a.step_mode()[0] == 1
    mode, blocks, bs = b.step_mode()
    assert mode == 2 and blocks >= 2 and bs in (64, 128, 256)
    for f in ("x", "u", "v", "a"):
        np.testing.assert_array_equal(b.node_vec(f), a.node_vec(f), err_msg=f)
    np.testing.assert_array_equal(b.elem_scalar("pl_strain"), a.elem_scalar("pl_strain"))
    np.testing.assert_array_equal(b.elem_tensor("sigma"), a.elem_tensor("sigma"))
    ra, rb = a.reaction(), b.reaction()
    assert ra.shape == rb.shape == (steps,)
    assert H.rel_err(rb, ra) <= 1e-12
    assert np.abs(ra).max() > 0
    # one predictor and one cluster launch per run
    assert b.launch_count() == 4


@pytest.mark.gpu
def test_automatic_mode_and_fallbacks():
    case, _ = cases()["c0"]
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, case)
    d.init()
    assert d.step_mode()[0] == 2            # 1000 elements: cluster run
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, case)
    d.set_energy_history(True)
    d.init()
    assert d.step_mode()[0] == 1            # energy history: no cluster run; per-phase kernels
    d.set_step_mode(2)
    with pytest.raises(wf.WfError) as e:
        d.run(4)
    assert e.value.status == wf.WF_ERR_UNSUPPORTED
    d = wf.Domain(wf.WF_FP64)
    W.apply(d, case)
    d.init()
    assert d.step_mode()[0] == 1            # FP64 always runs per phase
    big = W.config(0, scale=(16, 16, 16))   # 4096 elements: above the automatic limit
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, big)
    d.init()
    assert d.step_mode()[0] == 1            # too few sweep columns: per-phase kernels
    d.set_step_mode(3)                      # tiles are built by init: not after it
    assert d.step_mode()[0] == 1
    t = wf.Domain(wf.WF_MIXED)
    W.apply(t, big)
    t.set_step_mode(3)
    t.init()
    assert t.step_mode()[0] == 3            # tiled hexahedra
    d.set_step_mode(2)
    assert d.step_mode()[0] == 2
    with pytest.raises(wf.WfError):
        d.set_step_mode(6)

