"""Material gradients of the reaction history through the hand-written adjoint.

`solve_with_adjoint` runs the FP64 step with checkpoints (wf_adjoint_forward)
and returns the reaction history with the domain that can reverse it
(wf_adjoint_backward). `ReactionHistory` wraps the pair as a
torch.autograd.Function over the material table theta[nmat, 3] = (E,
sigma_y0, H): the forward builds and runs a domain, the backward maps
dL/dR to dL/dtheta on the GPU. Every forward builds a fresh domain, so one
graph may call it several times.
"""
from __future__ import annotations

import numpy as np

from . import WF_FP64, Domain
from . import workloads as W


def solve_with_adjoint(case: W.Case, theta=None, steps=None, every=0):
    """Runs `case` (materials from theta[nmat, 3] when given) for `steps`
    steps with checkpoints; returns (reaction history, domain)."""
    c = case if theta is None else W.with_params(case, theta)
    d = Domain(WF_FP64)
    W.apply(d, c)
    d.init()
    d.adjoint_forward(int(steps if steps is not None else c.steps), int(every))
    return d.reaction(), d


def _autograd_function():
    import torch

    class ReactionHistory(torch.autograd.Function):
        """R = ReactionHistory.apply(theta, case, steps, every, fp32)."""

        @staticmethod
        def forward(ctx, theta, case, steps, every=0, fp32=False):
            R, dom = solve_with_adjoint(case, theta.detach().cpu().numpy(), steps, every)
            ctx.dom = dom
            ctx.fp32 = bool(fp32)
            ctx.device = theta.device
            return torch.from_numpy(R).to(theta.device)

        @staticmethod
        def backward(ctx, grad_R):
            seed = grad_R.detach().to("cpu", torch.float64).numpy()
            g = ctx.dom.adjoint_backward(seed, ctx.fp32)
            return torch.from_numpy(g).to(ctx.device), None, None, None, None

    return ReactionHistory


def __getattr__(name):
    if name == "ReactionHistory":
        fn = _autograd_function()
        globals()["ReactionHistory"] = fn
        return fn
    raise AttributeError(name)
