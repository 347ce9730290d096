"""A thin ``torch.autograd.Function`` over getConc and its CUDA adjoint.

Used by the gradient-check harness only: the forward is ``scft_get_conc``
(cuda_scft.cu:61-138) on a context, the backward is ``scft_adjoint`` (the
hand-written reverse sweep of the propagator march with contour
checkpointing).  Tensors are float64 on the host; the library moves them to
and from the device.
"""
from __future__ import annotations

import torch


class GetConc(torch.autograd.Function):
    """(wA, wB, box[3]) -> (phiA, phiB, Q) of one context.

    ``wa``/``wb``: float64 ``[batch, Nz, Ny, Nx]``; ``box``: float64 ``[3]``
    (lx, ly, lz, shared by the batch).  ``Q``: ``[batch]``."""

    @staticmethod
    def forward(fctx, wa, wb, box, scft_ctx, checkpoint_every=0):
        c = scft_ctx
        c.set_box(*(float(v) for v in box.detach().cpu().tolist()))
        c.set_w(wa.detach().cpu().numpy(), wb.detach().cpu().numpy())
        c.get_conc()
        fctx.scft = c
        fctx.checkpoint_every = checkpoint_every
        fctx.save_for_backward(wa, wb, box)
        return (torch.from_numpy(c.pha), torch.from_numpy(c.phb), torch.from_numpy(c.Q()))

    @staticmethod
    def backward(fctx, g_pha, g_phb, g_Q):
        wa, wb, box = fctx.saved_tensors
        c = fctx.scft
        # the context may have moved on since the forward: restore its inputs
        c.set_box(*(float(v) for v in box.detach().cpu().tolist()))
        c.set_w(wa.detach().cpu().numpy(), wb.detach().cpu().numpy())
        want_L = bool(fctx.needs_input_grad[2])
        ga, gb, gL = c.adjoint(g_pha.detach().cpu().numpy(), g_phb.detach().cpu().numpy(),
                               g_Q.detach().cpu().numpy(), want_L=want_L,
                               checkpoint_every=fctx.checkpoint_every)
        gbox = torch.from_numpy(gL.sum(axis=0)) if want_L else None
        return torch.from_numpy(ga), torch.from_numpy(gb), gbox, None, None


def free_energy(wa, wb, box, scft_ctx, chiN: float, checkpoint_every: int = 0):
    """F of Free (cuda_scft.cu:190-221) per instance, differentiable in
    (wA, wB, box): chiN<phiA phiB> - <wA' phiA + wB phiB> - ln Q, with wA' the
    mean-free wA that getConc works with (cuda_scft.cu:71)."""
    pha, phb, Q = GetConc.apply(wa, wb, box, scft_ctx, checkpoint_every)
    dims = tuple(range(1, wa.dim()))
    wa_mf = wa - wa.mean(dim=dims, keepdim=True)
    return ((chiN * pha * phb).mean(dim=dims) - (wa_mf * pha + wb * phb).mean(dim=dims)
            - torch.log(Q))


__all__ = ["GetConc", "free_energy"]
