"""Test-harness autograd wrappers over the C ABI (not part of the package).

`FEulerFn` is a torch.autograd.Function whose forward is gbmv_feuler (FP64) and whose
backward is the hand-written VJP gbmv_feuler_vjp; `rk4_loss_and_grad` integrates the
semi-discrete Euler system with classical RK4 and differentiates a loss through the steps,
recomputing each segment of `checkpoint_every` steps from its checkpointed initial state in
the backward pass (torch.utils.checkpoint) instead of storing every stage.
"""
from __future__ import annotations

import torch
from torch.utils.checkpoint import checkpoint


class FEulerFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, hydro, *w):
        w = [x.contiguous() for x in w]
        wdot = [torch.empty_like(x) for x in w]
        rc = hydro.fEuler(0.0, w, wdot, 0)
        if rc != 0:
            raise RuntimeError(f"fEuler returned {rc}")
        ctx.hydro = hydro
        ctx.save_for_backward(*w)
        return tuple(wdot)

    @staticmethod
    def backward(ctx, *v):
        w = ctx.saved_tensors
        v = [x.contiguous() if x is not None else torch.zeros_like(w[i]) for i, x in enumerate(v)]
        u = [torch.empty_like(x) for x in w]
        ctx.hydro.fEuler_vjp(0.0, list(w), v, u)
        return (None, *u)


def rhs(hydro, w):
    return list(FEulerFn.apply(hydro, *w))


def rk4_step(hydro, dt, *w):
    w = list(w)
    k1 = rhs(hydro, w)
    k2 = rhs(hydro, [a + (0.5 * dt) * b for a, b in zip(w, k1)])
    k3 = rhs(hydro, [a + (0.5 * dt) * b for a, b in zip(w, k2)])
    k4 = rhs(hydro, [a + dt * b for a, b in zip(w, k3)])
    return tuple(a + (dt / 6.0) * (b + 2.0 * c + 2.0 * d + e)
                 for a, b, c, d, e in zip(w, k1, k2, k3, k4))


def _segment(hydro, dt, nsteps):
    def run(*w):
        for _ in range(nsteps):
            w = rk4_step(hydro, dt, *w)
        return w
    return run


def integrate(hydro, w0, dt, nsteps, checkpoint_every=None):
    w = tuple(w0)
    done = 0
    while done < nsteps:
        m = min(checkpoint_every or nsteps, nsteps - done)
        seg = _segment(hydro, dt, m)
        if checkpoint_every:
            w = checkpoint(seg, *w, use_reentrant=False)
        else:
            w = seg(*w)
        done += m
    return w


def rho2_integral(w, cell_volume):
    return (w[0] * w[0]).sum() * cell_volume


def loss_and_grad(hydro, w0, dt, nsteps, cell_volume, checkpoint_every=10):
    """Returns (L, dL/dw0) for L = integral of rho^2 at t = nsteps * dt."""
    leaves = [x.detach().clone().requires_grad_(True) for x in w0]
    w = integrate(hydro, leaves, dt, nsteps, checkpoint_every)
    L = rho2_integral(w, cell_volume)
    grads = torch.autograd.grad(L, leaves)
    return float(L.detach()), [g.detach() for g in grads]


def loss_only(hydro, w0, dt, nsteps, cell_volume):
    with torch.no_grad():
        w = integrate(hydro, [x.clone() for x in w0], dt, nsteps)
        return float(rho2_integral(w, cell_volume))
