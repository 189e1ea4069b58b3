"""torch.autograd binding of the MP2 adjoint: ``mp2_energy(gao, C, nocc, eps)`` returns a 0-d
tensor whose backward calls jues_rmp2_adjoint (the library computes E, dE/dgao and dE/dC in one
pass; no autograd graph is built through the contraction)."""
import numpy as np

from .MollerPlesset import rmp2_adjoint


def _torch():
    import torch
    return torch


def mp2_energy(gao, C, nocc, eps, precision="fp64"):
    torch = _torch()

    class _MP2(torch.autograd.Function):
        @staticmethod
        def forward(ctx, g, Cm):
            gn = g.detach().cpu().numpy()
            cn = Cm.detach().cpu().numpy()
            e = np.asarray(eps.detach().cpu().numpy() if hasattr(eps, "detach") else eps)
            E, gb, cb = rmp2_adjoint(gao=gn, C=cn, nocc=int(nocc), eps=e, precision=precision,
                                     want_gao=g.requires_grad, want_C=Cm.requires_grad)
            ctx.save_for_backward(*(torch.as_tensor(x) if x is not None else torch.zeros(0)
                                    for x in (gb, cb)))
            ctx.flags = (gb is not None, cb is not None)
            return torch.tensor(E, dtype=torch.float64)

        @staticmethod
        def backward(ctx, Ebar):
            gb, cb = ctx.saved_tensors
            return (Ebar * gb if ctx.flags[0] else None, Ebar * cb if ctx.flags[1] else None)

    return _MP2.apply(gao, C)
