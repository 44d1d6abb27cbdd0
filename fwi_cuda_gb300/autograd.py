"""torch.autograd view of the engine: model arrays -> L2 misfit, with the
backward pass supplied by the engine's hand-written adjoint (psv_gradient).

Test harness only (finite-difference checks, gradient-based experiments);
the FWI drivers call the C ABI directly.  The forward pass runs one FWI
gradient of every shot on the plan (forward, residual, time-reversed
adjoint with the imaging condition of src/cpu/n_kernel_lib_PSV.cpp:439-484)
and returns the reference's misfit L2 = 1/2 dt sum (u_mod - u_obs)^2
(adjsrc2, :580-600).  backward returns the summed per-shot imaging terms
(before energy preconditioning) oriented as +dL2/dm: the reference's CPU
path accumulates exactly that (grad -= ...), the CUDA path its negative.

Measured against central finite differences (tests/test_gpu_autograd.py,
101 x 201 model, 50 points): the lam term matches dL2/dlam to about 2 %
point by point; the mu term correlates at 0.998 with a scale near 1.2 (mu
enters the stencil through harmonic averages at staggered points, the
imaging condition is a point estimate); the reference's density term does
not follow dL2/drho.

A plan created with adjoint="exact" (FP64) returns instead the derivative
of L2 itself, from the hand-transposed discrete adjoint of the time loop
(PSV_ADJOINT_EXACT), on every cell of the grid.
"""
from __future__ import annotations

import numpy as np
import torch


def _full(sv, a):
    """Snapshot-window array -> full grid (zeros elsewhere)."""
    out = np.zeros((sv.nz, sv.nx))
    out[sv.snap_z1:sv.snap_z2 + 1:sv.snap_dz, sv.snap_x1:sv.snap_x2 + 1:sv.snap_dx] = a
    return out


class FWIMisfit(torch.autograd.Function):
    """FWIMisfit.apply(lam, mu, rho, plan) -> L2 (0-d float64 tensor).

    lam, mu, rho: [nz][nx] tensors (any device; copied to the host); plan:
    an engine.Plan holding the observed traces.  Every shot must fit one
    batch (max_batch 0 or >= nshot) so that its imaging term is readable.
    """

    @staticmethod
    def forward(ctx, lam, mu, rho, plan):
        sv = plan.sv
        m = [t.detach().to("cpu", torch.float64).numpy() for t in (lam, mu, rho)]
        plan.set_model(*m)
        plan.reset_gradient()
        L2, glob = plan.gradient(fetch=True)
        orient = -1.0 if sv.imaging_sign > 0 else 1.0  # -> +dL2/dm
        if getattr(plan, "adjoint", "reference") == "exact":
            g = [orient * x for x in glob]
        else:
            g = [np.zeros((sv.nz, sv.nx)) for _ in range(3)]
            for s in range(sv.nshot):
                o = plan.shot_gradient(s)
                for k, name in enumerate(("grad_lam", "grad_mu", "grad_rho")):
                    g[k] += orient * _full(sv, o[name])
        ctx.save_for_backward(*[torch.from_numpy(x).to(t.device, t.dtype)
                                for x, t in zip(g, (lam, mu, rho))])
        return torch.tensor(L2, dtype=torch.float64, device=lam.device)

    @staticmethod
    def backward(ctx, grad_out):
        gl, gm, gr = ctx.saved_tensors
        return grad_out * gl, grad_out * gm, grad_out * gr, None


def misfit(plan, lam, mu, rho):
    """L2 misfit of the model on `plan`, differentiable in lam, mu, rho."""
    return FWIMisfit.apply(lam, mu, rho, plan)
