"""Energy history (Domain_d::computeEnergies after every step).

The oracle's energies are pinned bit-for-bit to the reference's own
computeEnergies in tests/test_oracle.py (golden fixtures). Here the GPU
history is checked against the oracle: FP64 within 1e-9 relative (the sums
run in a different order), mixed precision within 1e-3.
"""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from oracle import orabind as O
from tests import helpers as H
from weldformfem_gb300 import workloads as W

CASES = {
    "hex4_hg": (lambda: W.config(0, scale=(4, 4, 4)), 300),
    "tet3x3x4": (lambda: W.config(1, scale=(3, 3, 4)), 300),
    "octants4": (lambda: W.config(4, scale=(4, 4, 4)), 300),
}


def oracle_energies(case, steps):
    o = O.OracleDomain()
    W.apply(o, case)
    o.init()
    o.step(steps)
    return o.energies()


def gpu_energies(case, steps, prec, timed=False):
    d = wf.Domain(prec)
    d.set_energy_history(True)
    W.apply(d, case)
    d.init()
    if timed:
        d.set_phase_timing(True)
    d.run(steps)
    return d.energies()


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_fp64_energies_match_oracle(name):
    mk, steps = CASES[name]
    ko, eo = oracle_energies(mk(), steps)
    kg, eg = gpu_energies(mk(), steps, wf.WF_FP64)
    assert kg.shape == (steps,)
    assert H.rel_err(kg, ko) <= 1e-9
    assert H.rel_err(eg, eo) <= 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_mixed_energies_close_to_oracle(name):
    mk, steps = CASES[name]
    ko, eo = oracle_energies(mk(), steps)
    kg, eg = gpu_energies(mk(), steps, wf.WF_MIXED)
    assert H.rel_err(kg, ko) <= 1e-3
    assert H.rel_err(eg, eo) <= 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [wf.WF_FP64, wf.WF_MIXED], ids=["fp64", "mixed"])
def test_graph_and_direct_launches_agree(prec):
    mk, _ = CASES["hex4_hg"]
    a = gpu_energies(mk(), 70, prec)               # two 32-step graphs + 6 direct steps
    b = gpu_energies(mk(), 70, prec, timed=True)   # direct launches only
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.gpu
def test_energy_history_must_be_enabled_before_init():
    d = wf.Domain(wf.WF_FP64)
    W.apply(d, CASES["hex4_hg"][0]())
    d.init()
    with pytest.raises(wf.WfError) as e:
        d.energies()
    assert e.value.status == 2
    with pytest.raises(wf.WfError) as e:
        d.set_energy_history(True)
    assert e.value.status == 2
