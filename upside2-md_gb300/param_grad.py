"""Parameter gradients of the GB300 engine behind torch.autograd.

`FrameEnergy` maps one node's parameters to the mean potential over the frames
held by a `Batch` (one protein replicated, one frame per system).  The forward
pass uploads the parameters and evaluates every frame in one batched launch
sequence.  The backward pass returns the engine's own adjoint dE/d(param):
the per-edge kernels that accumulate spline-coefficient derivatives with the
current edge sensitivities (the reference's get_param_deriv path:
src/interaction_graph.h:406-416 with src/bead_interaction.h:87-131 for the
rotamer pair splines, src/environment.cpp:789-833 for the nonlinear
environment coupling), summed over the batch and divided by the frame count.

PyTorch is only the differentiation interface here; the arithmetic runs in the
engine's sm_103a kernels.
"""
import numpy as np
import torch


class FrameEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, param, batch, node):
        shape = tuple(param.shape)
        batch.set_param(node, param.detach().to("cpu", torch.float32).numpy())
        energy, _ = batch.evaluate(want_deriv=False)
        grad = batch.param_deriv(node, shape).astype(np.float64) / batch.n_sys
        ctx.save_for_backward(torch.from_numpy(grad).to(param.device))
        ctx.param_dtype = param.dtype
        return torch.tensor(float(np.mean(energy)), dtype=torch.float64, device=param.device)

    @staticmethod
    def backward(ctx, grad_out):
        (grad,) = ctx.saved_tensors
        return (grad_out * grad).to(ctx.param_dtype), None, None


def mean_energy(param, batch, node):
    """Mean potential over the batch's frames, differentiable in `param`."""
    return FrameEnergy.apply(param, batch, node)
