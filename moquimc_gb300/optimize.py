"""Spot-weight optimisation on a Dij matrix: dose = D.w through the differentiable Dij operator.

The objective is a quadratic prescription dose in a target plus a one-sided quadratic penalty above
a maximum dose in an organ; the weights take projected-gradient steps (w >= 0).  moqui itself stops
at writing the matrix (save_sparse_file, moqui/base/environments/mqi_tps_env.hpp:1905-1930); this is
the plan-optimisation loop its Dij output feeds, with the gradient from the hand-written D^T.g
kernel rather than from a dense matrix.
"""
from __future__ import annotations

import numpy as np

from . import dij as dijmod


def make_objective(torch, target, organ, prescription: float = 2.0, organ_max: float = 0.5):
    """f(dose) = sum_target (d - p)^2 + sum_organ max(d - m, 0)^2 (boolean CUDA masks)."""
    tgt_idx = torch.nonzero(target).squeeze(1)
    org_idx = torch.nonzero(organ).squeeze(1)

    def f(dose):
        dt = dose.index_select(0, tgt_idx)
        do = dose.index_select(0, org_idx)
        return ((dt - prescription) ** 2).sum() + (torch.relu(do - organ_max) ** 2).sum()

    return f


def lipschitz(op, target, organ, iters: int = 20, seed: int = 0) -> float:
    """Largest eigenvalue of 2 D^T M D (M the union of the masks) by power iteration."""
    import torch

    g = torch.Generator(device="cuda").manual_seed(seed)
    mask = (target | organ).double()
    v = torch.rand(op.n_spots, device="cuda", dtype=torch.float64, generator=g)
    lam = 1.0
    for _ in range(iters):
        v = op.rmatvec(mask * op.matvec(v))
        lam = float(v.norm())
        if lam == 0.0:
            raise RuntimeError("the Dij matrix has no dose in the target or organ")
        v = v / lam
    return 2.0 * lam


def projected_gradient(op, objective, w0, iters: int = 100, step: float | None = None, lip: float | None = None):
    """iters steps of w <- max(w - step * grad f(D.w), 0); returns (w, objective history)."""
    import torch

    w = w0.clone()
    step = step if step is not None else 1.0 / lip
    hist = []
    for _ in range(iters):
        wv = w.detach().requires_grad_(True)
        f = objective(dijmod.dose(op, wv))
        f.backward()
        with torch.no_grad():
            w = torch.clamp(wv - step * wv.grad, min=0.0)
        hist.append(f.detach())
    return w, torch.stack(hist)


def fd_check(op, objective, w, spots, h: float = 1e-3, dtype=None):
    """Relative errors of the autograd gradient (computed in `dtype`) against central finite
    differences with step h on the given spots, the objective evaluated with the FP64 product."""
    import torch

    dtype = dtype or w.dtype
    wv = w.detach().to(dtype).requires_grad_(True)
    f = objective(dijmod.dose(op, wv))
    f.backward()
    grad = wv.grad.double().cpu().numpy()[spots]
    w64 = w.detach().double()
    fd = np.empty(len(spots))
    for i, s in enumerate(spots):
        e = torch.zeros_like(w64)
        e[int(s)] = h
        fd[i] = (float(objective(op.matvec(w64 + e))) - float(objective(op.matvec(w64 - e)))) / (2.0 * h)
    scale = np.abs(fd).max() if np.abs(fd).max() > 0 else 1.0
    rel = np.abs(grad - fd) / np.maximum(np.abs(fd), 1e-9 * scale)
    return rel, grad, fd
