"""Adjoint (reverse mode) of the FP64 step: material gradients of the
reaction history.

The loss is the material-identification objective of the 32^3 octant cube,
on a 4^3 version of it: L = sum_s (R_s - R*_s)^2 with R* from a run whose 24
octant parameters (E, sigma_y0, H of 8 materials) are scaled by seeded
U[0.8, 1.2) factors. The GPU gradient is checked against central finite
differences (relative step 1e-6) of the CPU oracle, the FP64 restatement of
the reference step, in log-parameter form theta_i dL/dtheta_i so that E,
sigma_y0 and H are comparable: within 1e-3 of the largest component. The FP32
reverse is checked against the FP64 reverse.
"""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from oracle import orabind as O
from tests import helpers as H
from weldformfem_gb300 import adjoint as A
from weldformfem_gb300 import workloads as W

STEPS = 300
REL_STEP = 1e-6
TOL_FD = 1e-3
TOL_FP32 = 1e-2


def small_case():
    c = W.config(4, steps=STEPS, scale=(4, 4, 4))
    c.dt = c.time_step()
    return c


def oracle_reaction(case, theta, steps=STEPS):
    o = O.OracleDomain()
    W.apply(o, W.with_params(case, theta))
    o.init()
    o.step(steps)
    return o.reaction()


def test_param_helpers():
    c = small_case()
    th = W.material_params(c)
    assert th.shape == (8, 3)
    f = W.target_factors(c)
    assert f.shape == (8, 3) and f.min() >= 0.8 and f.max() < 1.2
    np.testing.assert_array_equal(f, W.target_factors(c))
    c2 = W.with_params(c, th * f)
    assert c2.dt == c.dt and c2.materials[3]["sy0"] == th[3, 1] * f[3, 1]
    assert c.materials[3]["sy0"] == th[3, 1]          # the original is untouched


@pytest.fixture(scope="module")
def problem():
    c = small_case()
    th0 = W.material_params(c)
    Rstar = oracle_reaction(c, th0 * W.target_factors(c))
    return c, th0, Rstar


@pytest.fixture(scope="module")
def fd_gradient(problem):
    c, th0, Rstar = problem
    g = np.zeros_like(th0)
    for i in range(th0.shape[0]):
        for k in range(3):
            h = REL_STEP * th0[i, k]
            tp, tm = th0.copy(), th0.copy()
            tp[i, k] += h
            tm[i, k] -= h
            Lp = np.sum((oracle_reaction(c, tp) - Rstar) ** 2)
            Lm = np.sum((oracle_reaction(c, tm) - Rstar) ** 2)
            g[i, k] = (Lp - Lm) / (2 * h)
    return g


def log_grad_err(g, ref, th):
    a, b = g * th, ref * th
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.gpu
def test_adjoint_matches_finite_differences(problem, fd_gradient):
    c, th0, Rstar = problem
    R, d = A.solve_with_adjoint(c, th0, STEPS, every=16)
    assert H.rel_err(R, oracle_reaction(c, th0)) <= 1e-9
    g = d.adjoint_backward(2.0 * (R - Rstar))
    err = log_grad_err(g, fd_gradient, th0)
    print(f"adjoint vs central FD (log-parameter, max-normalised): {err:.3e}")
    assert err <= TOL_FD
    # every material parameter matters in this problem
    assert np.all(np.abs(fd_gradient * th0) > 1e-6 * np.abs(fd_gradient * th0).max())


@pytest.mark.gpu
def test_fp32_reverse_against_fp64(problem):
    c, th0, Rstar = problem
    R, d = A.solve_with_adjoint(c, th0, STEPS)
    seed = 2.0 * (R - Rstar)
    g64 = d.adjoint_backward(seed)
    g32 = d.adjoint_backward(seed, fp32=True)
    err = log_grad_err(g32, g64, th0)
    print(f"FP32 reverse vs FP64 reverse (log-parameter, max-normalised): {err:.3e}")
    assert err <= TOL_FP32


@pytest.mark.gpu
def test_checkpoint_interval_does_not_change_gradient(problem):
    c, th0, Rstar = problem
    grads = []
    for every in (1, 7, 0, STEPS, -1):   # -1: every step kept, no recompute
        R, d = A.solve_with_adjoint(c, th0, STEPS, every=every)
        grads.append(d.adjoint_backward(2.0 * (R - Rstar)))
    for g in grads[1:]:
        np.testing.assert_array_equal(g, grads[0])


@pytest.mark.gpu
@pytest.mark.parametrize("every", [32, -1])
def test_backward_restores_final_state_and_repeats(problem, every):
    c, th0, Rstar = problem
    R, d = A.solve_with_adjoint(c, th0, STEPS, every=every)
    u = d.node_vec("u")
    pl = d.elem_scalar("pl_strain")
    seed = np.random.default_rng(7).standard_normal(STEPS)
    g1 = d.adjoint_backward(seed)
    np.testing.assert_array_equal(d.node_vec("u"), u)
    np.testing.assert_array_equal(d.elem_scalar("pl_strain"), pl)
    np.testing.assert_array_equal(d.reaction(), R)
    np.testing.assert_array_equal(d.adjoint_backward(seed), g1)
    # linear in the seed
    np.testing.assert_allclose(d.adjoint_backward(3.0 * seed), 3.0 * g1, rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_torch_autograd_wrapper(problem):
    torch = pytest.importorskip("torch")
    c, th0, Rstar = problem
    theta = torch.tensor(th0, dtype=torch.float64, requires_grad=True)
    R = A.ReactionHistory.apply(theta, c, STEPS, 0, False)
    loss = ((R - torch.from_numpy(Rstar)) ** 2).sum()
    loss.backward()
    Rn, d = A.solve_with_adjoint(c, th0, STEPS)
    np.testing.assert_array_equal(R.detach().numpy(), Rn)
    np.testing.assert_array_equal(theta.grad.numpy(), d.adjoint_backward(2.0 * (Rn - Rstar)))


@pytest.mark.gpu
def test_adjoint_rejects_unsupported():
    c = small_case()
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, c)
    d.init()
    with pytest.raises(wf.WfError) as e:
        d.adjoint_forward(10)
    assert e.value.status == 5
    d = wf.Domain(wf.WF_FP64)
    W.apply(d, c)
    d.init()
    with pytest.raises(wf.WfError) as e:
        d.adjoint_backward(np.zeros(10))
    assert e.value.status == 2
    d.adjoint_forward(10)
    d.run(1)
    with pytest.raises(wf.WfError) as e:
        d.adjoint_backward(np.zeros(10))
    assert e.value.status == 2


@pytest.mark.gpu
def test_adjoint_full_c4_against_oracle_finite_differences():
    """Configuration 4 as specified (32^3 hexahedra, 8 octant materials, 4000
    steps, checkpoints every 64 steps): two gradient components against
    central differences of the CPU oracle (the FP64 restatement of the
    reference step), each within 1e-3 of the difference quotient."""
    c = W.config(4)
    c.dt = c.time_step()
    n = c.steps
    th0 = W.material_params(c)
    Rstar = oracle_reaction(c, th0 * W.target_factors(c), n)
    R, d = A.solve_with_adjoint(c, th0, n, every=64)
    assert H.rel_err(R, oracle_reaction(c, th0, n)) <= 1e-9
    g = d.adjoint_backward(2.0 * (R - Rstar))
    for i, k in ((0, 0), (5, 1)):          # E of octant 0, sigma_y0 of octant 5
        h = REL_STEP * th0[i, k]
        tp, tm = th0.copy(), th0.copy()
        tp[i, k] += h
        tm[i, k] -= h
        Lp = np.sum((oracle_reaction(c, tp, n) - Rstar) ** 2)
        Lm = np.sum((oracle_reaction(c, tm, n) - Rstar) ** 2)
        gfd = (Lp - Lm) / (2 * h)
        assert abs(g[i, k] - gfd) <= 1e-3 * abs(gfd), (i, k, g[i, k], gfd)
