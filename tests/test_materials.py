"""Material laws beyond linear hardening on the GPU: Johnson-Cook and GMT.

The oracle's restatements are pinned bit-for-bit to the reference's own
CalcStressStrain (Material_::Init_JohnsonCook; CalcGMTYieldStress and
CalcGMTTangentModulus with the Material_ fields they read) by the
hex_johnson_cook and hex_gmt fixtures in tests/test_oracle.py. Here the GPU
paths are checked against the oracle on the same inputs: FP64 within 1e-9
relative (log, exp and pow of the device and the host libm can differ by an
ulp), mixed precision within the mixed-path bounds in each of its step modes.
"""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from oracle import orabind as O
from tests import helpers as H
from weldformfem_gb300 import workloads as W

JC_MAT = dict(model=2, E=200e9, nu=0.3, rho=7850.0, sy0=250e6)
JC = [400e6, 0.35, 0.02, 1.0, 1.0, 1500.0, 20.0, 300.0]
GMT_MAT = dict(model=3, E=200e9, nu=0.3, rho=7850.0, sy0=250e6)
# n1, n2, C1, C2, m1, m2, I1, I2; e, edot and T ranges; temperature
GMT = dict(c=[-2e-4, 0.2, 1200e6, -1.5e-3, 1e-4, 0.02, -1e-5, -2e-3],
           range=[0.01, 2.0, 1e-2, 1e5, 0.0, 1500.0], T=300.0)


def cases():
    h = W.config(0, scale=(3, 3, 4))
    h.perturb = 0.1
    h.seed = W.SEED_BASE + 9
    h.top_vz = -5.0
    h.materials = [dict(JC_MAT)]
    t = W.config(1, scale=(3, 3, 4))
    t.top_vz = -3.0
    t.materials = [dict(JC_MAT)]
    return {"hex": (h, 400), "tet": (t, 300)}


def oracle(case, steps):
    o = O.OracleDomain()
    H.setup(o, case, {"jc": JC})
    o.init()
    o.step(steps)
    return o


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["hex", "tet"])
def test_johnson_cook_fp64_matches_oracle(name):
    case, steps = cases()[name]
    o = oracle(case, steps)
    assert o.elem_scalar("pl_strain").max() > 0.005   # the runs are well into yield
    d = wf.Domain(wf.WF_FP64)
    H.setup(d, case, {"jc": JC})
    d.init()
    d.run(steps)
    for kind, f in [("node_vec", "u"), ("elem_scalar", "pl_strain"), ("elem_scalar", "sigma_y"),
                    ("elem_tensor", "sigma")]:
        assert H.rel_err(getattr(d, kind)(f), getattr(o, kind)(f)) <= 1e-9, f
    assert H.rel_err(d.reaction(), o.reaction()) <= 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["hex", "tet"])
def test_johnson_cook_mixed(name):
    case, steps = cases()[name]
    o = oracle(case, steps)
    d = wf.Domain(wf.WF_MIXED)
    H.setup(d, case, {"jc": JC})
    d.init()
    d.run(steps)
    assert H.rel_err(d.node_vec("u"), o.node_vec("u")) <= 1e-4
    assert H.rel_err(d.elem_scalar("pl_strain"), o.elem_scalar("pl_strain")) <= 1e-2
    assert H.rel_err(d.reaction(), o.reaction()) <= 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [wf.WF_FP64, wf.WF_MIXED])
def test_johnson_cook_strain_rate_cap(prec):
    """m_max_edot below the element rates (the hex_jc_rate_cap fixture pins
    the oracle to the reference): the GPU against the oracle with the same
    cap, FP64 within 1e-9 and mixed within its bounds."""
    case, steps = cases()["hex"]
    extra = {"jc": JC, "max_edot": 50.0}
    o = O.OracleDomain()
    H.setup(o, case, extra)
    o.init()
    o.step(steps)
    d = wf.Domain(prec)
    H.setup(d, case, extra)
    d.init()
    d.run(steps)
    tol = 1e-9 if prec == wf.WF_FP64 else 1e-4
    assert H.rel_err(d.node_vec("u"), o.node_vec("u")) <= tol
    assert H.rel_err(d.elem_scalar("pl_strain"), o.elem_scalar("pl_strain")) <= (
        1e-9 if prec == wf.WF_FP64 else 1e-2)


@pytest.mark.gpu
def test_johnson_cook_needs_its_constants():
    case, _ = cases()["hex"]
    d = wf.Domain(wf.WF_FP64)
    W.apply(d, case)
    with pytest.raises(wf.WfError) as e:
        d.init()
    assert e.value.status == 2
    d2 = wf.Domain(wf.WF_FP64)
    c2 = W.config(0, scale=(2, 2, 2))
    W.apply(d2, c2)
    with pytest.raises(wf.WfError) as e:
        d2.set_johnson_cook(0, *JC)
    assert e.value.status == 2


def test_johnson_cook_deck(tmp_path):
    import json
    deck = {"Configuration": {"simTime": 1e-6, "cflFactor": 0.3},
            "Materials": [{"type": "JohnsonCook", "const": [400e6, 0.35, 0.02, 1.0],
                           "density0": 7850.0, "youngsModulus": 200e9, "poissonsRatio": 0.3,
                           "yieldStress0": 250e6}],
            "DomainBlocks": [{"type": "Box", "dim": [0.002, 0.002, 0.002],
                              "elemLength": 0.001}]}
    p = tmp_path / "jc.json"
    p.write_text(json.dumps(deck))
    k = wf.Deck(str(p))
    assert k.info["material"]["model"] == 2 and k.info["material"]["sy0"] == 250e6
    assert k.info["johnson_cook"] == [400e6, 0.35, 0.02, 1.0, 1.0, 1.0e10, 0.0, 0.0]


def gmt_cases():
    h = W.config(0, scale=(3, 3, 4))
    h.perturb = 0.1
    h.seed = W.SEED_BASE + 19
    h.top_vz = -5.0
    h.materials = [dict(GMT_MAT)]
    t = W.config(1, scale=(3, 3, 4))
    t.top_vz = -3.0
    t.materials = [dict(GMT_MAT)]
    # a box of hexahedra (no perturbation) large enough for the per-phase,
    # column-sweep and dataflow steps
    b = W.config(0, scale=(12, 12, 12))
    b.top_vz = -20.0
    b.materials = [dict(GMT_MAT)]
    return {"hex": (h, 400), "tet": (t, 300), "box": (b, 300)}


def gmt_oracle(case, steps):
    o = O.OracleDomain()
    H.setup(o, case, {"gmt": GMT})
    o.init()
    o.step(steps)
    return o


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["hex", "tet", "box"])
def test_gmt_fp64_matches_oracle(name):
    case, steps = gmt_cases()[name]
    o = gmt_oracle(case, steps)
    assert o.elem_scalar("pl_strain").max() > 0.005   # well into yield, past e_min
    d = wf.Domain(wf.WF_FP64)
    H.setup(d, case, {"gmt": GMT})
    d.init()
    d.run(steps)
    for kind, f in [("node_vec", "u"), ("elem_scalar", "pl_strain"), ("elem_scalar", "sigma_y"),
                    ("elem_tensor", "sigma")]:
        assert H.rel_err(getattr(d, kind)(f), getattr(o, kind)(f)) <= 1e-9, f
    assert H.rel_err(d.reaction(), o.reaction()) <= 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("name,mode", [("hex", 0), ("hex", 1), ("tet", 0), ("tet", 1),
                                       ("box", 1), ("box", 4), ("box", 5)])
def test_gmt_mixed(name, mode):
    """FP32 GMT (the law's temperature terms reduced once on the host) in the
    automatic mode (the cluster run for these sizes), the per-phase kernels,
    the column sweep and the dataflow step."""
    case, steps = gmt_cases()[name]
    o = gmt_oracle(case, steps)
    d = wf.Domain(wf.WF_MIXED)
    H.setup(d, case, {"gmt": GMT})
    if mode:
        d.set_step_mode(mode)
    d.init()
    d.run(steps)
    assert H.rel_err(d.node_vec("u"), o.node_vec("u")) <= 1e-4
    assert H.rel_err(d.elem_scalar("pl_strain"), o.elem_scalar("pl_strain")) <= 1e-2
    assert H.rel_err(d.reaction(), o.reaction()) <= 1e-3


@pytest.mark.gpu
def test_gmt_argument_checks():
    case, _ = gmt_cases()["hex"]
    d = wf.Domain(wf.WF_FP64)
    W.apply(d, case)
    with pytest.raises(wf.WfError) as e:          # constants never set
        d.init()
    assert e.value.status == 2
    d = wf.Domain(wf.WF_FP64)
    W.apply(d, case)
    for rng in ([0.0, 2.0, 1e-2, 1e5, 0.0, 1500.0],      # e_min = 0: the law is 0 * inf
                [0.01, 2.0, 1e5, 1e-2, 0.0, 1500.0]):    # er_min > er_max
        with pytest.raises(wf.WfError) as e:
            d.set_gmt(0, GMT["c"], rng, 300.0)
        assert e.value.status == 1
    with pytest.raises(wf.WfError) as e:          # material 0 of another model
        j = wf.Domain(wf.WF_FP64)
        W.apply(j, W.config(0, scale=(2, 2, 2)))
        j.set_gmt(0, GMT["c"], GMT["range"], 300.0)
    assert e.value.status == 2


def test_gmt_deck(tmp_path):
    """The GMT deck keys (main.C:466-493, 548-553) and NortonHoff's rejection."""
    import json
    mat = {"type": "GMT", "const": GMT["c"], "strRange": [0.01, 2.0],
           "strdotRange": [1e-2, 1e5], "density0": 7850.0, "youngsModulus": 200e9,
           "poissonsRatio": 0.3, "yieldStress0": 250e6}
    deck = {"Configuration": {"simTime": 1e-6, "cflFactor": 0.3}, "Materials": [mat],
            "DomainBlocks": [{"type": "Box", "dim": [0.002, 0.002, 0.002],
                              "elemLength": 0.001}]}
    p = tmp_path / "gmt.json"
    p.write_text(json.dumps(deck))
    k = wf.Deck(str(p))
    assert k.info["material"]["model"] == 3
    assert k.info["gmt"] == GMT["c"]
    assert k.info["gmt_range"] == [0.01, 2.0, 1e-2, 1e5, 0.0, 1.0e10]   # tempRange default
    mat["type"] = "NortonHoff"
    p.write_text(json.dumps(deck))
    with pytest.raises(wf.WfError) as e:
        wf.Deck(str(p))
    assert e.value.status == 5


def test_plasticity_options_deck(tmp_path):
    """Configuration.plHeatFrac and maxStrRate (main.C:218, 228) and their
    defaults."""
    import json
    mat = {"type": "Bilinear", "const": [2.0e9], "density0": 7850.0, "youngsModulus": 200e9,
           "poissonsRatio": 0.3, "yieldStress0": 300e6}
    deck = {"Configuration": {"simTime": 1e-6, "cflFactor": 0.3}, "Materials": [mat],
            "DomainBlocks": [{"type": "Box", "dim": [0.002, 0.002, 0.002],
                              "elemLength": 0.001}]}
    p = tmp_path / "opts.json"
    p.write_text(json.dumps(deck))
    k = wf.Deck(str(p))
    assert k.info["plheat_frac"] == 0.9 and k.info["max_edot"] == 1.0e6
    deck["Configuration"].update(plHeatFrac=0.6, maxStrRate=50.0)
    p.write_text(json.dumps(deck))
    k = wf.Deck(str(p))
    assert k.info["plheat_frac"] == 0.6 and k.info["max_edot"] == 50.0
    deck["Configuration"]["plHeatFrac"] = 1.5
    p.write_text(json.dumps(deck))
    with pytest.raises(wf.WfError) as e:
        wf.Deck(str(p))
    assert e.value.status == 1
