"""Mixed-precision CUDA path against the FP64 oracle (GPU).

The mixed path computes element arithmetic in FP32 (positions as compensated
float pairs, reaction sums in FP64), so it is not bit-compatible; these tests
bound its error against the FP64 oracle on the same inputs. Tolerances
(max |mixed - fp64| / max |fp64|): displacement 1e-4, reaction history 1e-3,
equivalent plastic strain 1e-2 (elements at the yield onset switch branch
with O(eps_f32) changes of the trial stress).

With Coulomb friction the sliding force points along -v_t / |v_t| (the
reference's law, Contact.C:277-283); where the tangential velocity is near
zero that direction is set by rounding, so FP32 and FP64 runs part ways in
the lateral rigid-body motion of a block held only by friction. The
frictional case therefore bounds the reaction history (the contact normal
force, 1e-3) and the RMS displacement error (1e-3) rather than the maximum.
"""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from oracle import orabind as O
from tests import helpers as H
from weldformfem_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def errors(case, steps):
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, case)
    d.init()
    d.run(steps)
    o = O.OracleDomain()
    W.apply(o, case)
    o.init()
    o.step(steps)
    return {"u": H.rel_err(d.node_vec("u"), o.node_vec("u")),
            "x": H.rel_err(d.node_vec("x"), o.node_vec("x")),
            "reaction": H.rel_err(d.reaction(), o.reaction()),
            "pl": H.rel_err(d.elem_scalar("pl_strain"), o.elem_scalar("pl_strain")),
            "sigma": H.rel_err(d.elem_tensor("sigma"), o.elem_tensor("sigma"))}


def frictionless(case):
    case.contact = dict(case.contact, mu=0.0)
    return case


@pytest.mark.parametrize("case,steps", [
    (W.config(0), 2000),                                  # config 0 hexahedra + hourglass
    (W.config(1, scale=(8, 8, 12)), 800),                 # perturbed tetrahedra
    (frictionless(W.config(2, scale=(16, 16, 8))), 600),  # perturbed hexahedra, rigid die
], ids=["hex_c0", "tet", "die_frictionless"])
def test_mixed_error_vs_fp64(case, steps):
    e = errors(case, steps)
    assert e["u"] <= 1e-4, e
    assert e["x"] <= 1e-6, e
    assert e["reaction"] <= 1e-3, e
    assert e["pl"] <= 1e-2, e


def test_mixed_error_vs_fp64_with_friction():
    case = W.config(2, scale=(16, 16, 8))
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, case)
    d.init()
    d.run(600)
    o = O.OracleDomain()
    W.apply(o, case)
    o.init()
    o.step(600)
    u, uo = d.node_vec("u"), o.node_vec("u")
    rms = np.sqrt(np.mean((u - uo) ** 2)) / np.sqrt(np.mean(uo ** 2))
    assert rms <= 1e-3
    assert H.rel_err(d.reaction(), o.reaction()) <= 1e-3


def test_mixed_deterministic():
    case = W.config(2, scale=(12, 12, 6))
    outs = []
    for _ in range(2):
        d = wf.Domain(wf.WF_MIXED)
        W.apply(d, case)
        d.init()
        d.run(100)
        outs.append((d.node_vec("x"), d.reaction()))
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


def test_mixed_rejects_unsupported_options():
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, W.config(1, scale=(2, 2, 2)))
    stab = np.zeros(10)
    stab[0] = 0.5
    d.set_stab(stab)
    with pytest.raises(wf.WfError) as e:
        d.init()
    assert e.value.status == 5
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, W.config(1, scale=(2, 2, 2)))
    d.set_press_algorithm(1)
    with pytest.raises(wf.WfError) as e:
        d.init()
    assert e.value.status == 5


def run_pair(case, steps, av=None):
    out = []
    for dom in (wf.Domain(wf.WF_MIXED), O.OracleDomain()):
        W.apply(dom, case)
        if av:
            dom.set_artif_visc(*av)
        dom.init()
        dom.run(steps) if hasattr(dom, "run") else dom.step(steps)
        out.append(dom)
    return out


@pytest.mark.parametrize("cid,scale", [(0, (6, 6, 6)), (1, (4, 4, 6)), (0, (16, 16, 16))],
                         ids=["hex-cluster", "tet-cluster", "hex-per-phase"])
def test_mixed_artificial_viscosity_vs_fp64(cid, scale):
    """calcArtificialViscosity in FP32: within the mixed path's bounds of the
    FP64 oracle with the same viscosity, and ten times closer to it than the
    mixed run without viscosity is (coefficients large enough for the viscous
    stress to show in the reaction)."""
    case = W.config(cid, scale=scale)
    case.perturb = 0.1
    case.seed = W.SEED_BASE + 11
    case.materials = [dict(H.HOLLOMON)]
    m, o = run_pair(case, 300, av=(50.0, 10.0))
    assert H.rel_err(m.node_vec("u"), o.node_vec("u")) <= 1e-4
    e_av = H.rel_err(m.reaction(), o.reaction())
    assert e_av <= 1e-3
    plain, _ = run_pair(case, 300)
    assert e_av < 0.1 * H.rel_err(plain.reaction(), o.reaction())


def test_autotuned_and_default_launch_shapes_agree_bitwise():
    """The autotuner only changes launch shapes; results are identical (the
    per-phase step, whose three kernels are all tuned)."""
    case = W.config(2, scale=(20, 18, 10))
    outs = []
    for tune in (True, False):
        d = wf.Domain(wf.WF_MIXED)
        W.apply(d, case)
        d.set_step_mode(1)
        d.set_autotune(tune)
        d.init()
        d.run(64)
        outs.append((d.node_vec("x"), d.reaction(), d.elem_scalar("pl_strain")))
        if tune:
            for phase in range(3):
                bs, ept, ms = d.launch_config(phase)
                assert bs in (64, 128, 256) and ept in (0, 1, 2, 4) and ms > 0.0
    # every shape by hand, persistent grids (items per thread 0) included
    for bs, ept in ((64, 0), (256, 0), (128, 4)):
        d = wf.Domain(wf.WF_MIXED)
        W.apply(d, case)
        d.set_step_mode(1)
        d.set_autotune(False)
        d.init()
        for phase in range(3):
            d.set_launch_config(phase, bs, ept)
        d.run(64)
        outs.append((d.node_vec("x"), d.reaction(), d.elem_scalar("pl_strain")))
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a, b)


def test_mixed_full_c2_without_friction_over_the_whole_run():
    """Configuration 2 at full size (8.39 M hexahedra, rigid die) over all its
    1000 steps, mixed against FP64 on the same inputs, with the friction
    coefficient set to 0: displacement and reaction within 1e-4 (max-norm),
    plastic strain within 1e-2. (With friction the sliding direction of the
    top-face nodes is decided by rounding; bench.py reports that case's
    max-norm and RMS errors.)"""
    case = W.config(2)
    case.contact = dict(case.contact, mu=0.0)
    x = case.coords()
    out = {}
    for prec in (wf.WF_MIXED, wf.WF_FP64):
        d = wf.Domain(prec)
        W.apply(d, case, x=x)
        d.init()
        d.run(case.steps)
        out[prec] = (d.node_vec("u"), d.reaction(), d.elem_scalar("pl_strain"))
        del d
    (um, rm, pm), (uf, rf, pf) = out[wf.WF_MIXED], out[wf.WF_FP64]
    assert pf.max() > 1e-3                         # plastic by the end
    assert H.rel_err(um, uf) <= 1e-4
    assert H.rel_err(rm, rf) <= 1e-4
    assert H.rel_err(pm, pf) <= 1e-2
