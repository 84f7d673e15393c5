"""torch.autograd binding of the adjoint: the gap-field objective as a
differentiable function of the design region's per-voxel eps.

    F = GapFieldObjective.apply(eps, fields, design_lo, objective, n_steps, checkpoint_every)

eps is a 3-D tensor [nz_d][ny_d][nx_d] (any device; the stepper copies it to
its own buffers); F is a 0-d float64 tensor, and F.backward() fills eps.grad
with dF/d(eps) from the library's discrete adjoint (sj_adjoint_gradient).
One instance (instance 0 of `fields`) per call.
"""
import numpy as np
import torch

from .spec import Design


class GapFieldObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, eps, fields, design_lo, objective, n_steps, checkpoint_every=200):
        e = eps.detach().to("cpu", torch.float64).numpy()
        fields.set_design(Design(tuple(design_lo), np.ascontiguousarray(e)), inst=0)
        F, grads = fields.adjoint_gradient([objective], n_steps, checkpoint_every)
        ctx.save_for_backward(torch.from_numpy(grads[0]).to(eps.device, eps.dtype))
        return torch.tensor(F[0], dtype=torch.float64, device=eps.device)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out.to(g.dtype) * g, None, None, None, None, None
