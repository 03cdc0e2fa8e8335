"""torch.autograd binding of hmf_solve_adjoint (include/hmf.h).

`hmf_loss(solver, data, alpha, truth)` returns the scalar
L = -(1/V) sum_i log(max(u_{leaf(truth_i)}(i), eps)) of the solver's final
leaf labels as a torch tensor whose backward yields dL/d(data) and
dL/d(alpha).  The library runs the whole reverse pass inside the forward call
(the states it needs are on the device only then), so backward only scales
the stored gradients by the incoming gradient.  No counterpart in the
reference, which has no gradients.
"""
from __future__ import annotations

import torch

from .segmentation import HMFSolver


class _HMFLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, data, alpha, solver, truth, checkpoint_every, eps):
        if not data.is_cuda:
            raise TypeError("data must be a CUDA tensor [n_leaves, VZ, VY, VX]")
        leaves = solver.leaves
        if data.shape[0] != len(leaves):
            raise ValueError("data holds %d leaves, the tree has %d" % (data.shape[0], len(leaves)))
        vols = [data[j].detach().to(torch.float32).contiguous() for j in range(len(leaves))]
        for leaf, vol in zip(leaves, vols):
            solver.set_data(leaf, vol)
        alpha_h = alpha.detach().to(torch.float64).cpu().tolist()
        for v, a in enumerate(alpha_h):
            if solver.parent[v] >= 0:
                solver.set_smoothness_scalar(v, a)
        stream = torch.cuda.current_stream(data.device)
        loss = solver.solve_adjoint(truth, checkpoint_every=checkpoint_every, eps=eps, stream=stream)
        grads = torch.empty((len(leaves),) + tuple(data.shape[1:]), dtype=torch.float64, device=data.device)
        for j, leaf in enumerate(leaves):
            solver.data_gradient(leaf, out=grads[j], stream=stream)
        torch.cuda.current_stream(data.device).synchronize()
        ctx.save_for_backward(grads.to(data.dtype),
                              torch.as_tensor(solver.alpha_gradient(), dtype=alpha.dtype, device=alpha.device))
        del vols
        return torch.tensor(loss, dtype=torch.float64, device=data.device)

    @staticmethod
    def backward(ctx, grad_loss):
        gD, ga = ctx.saved_tensors
        g = grad_loss.to(device=gD.device, dtype=gD.dtype)
        return gD * g, ga * grad_loss.to(device=ga.device, dtype=ga.dtype), None, None, None, None


def hmf_loss(solver: HMFSolver, data: torch.Tensor, alpha: torch.Tensor, truth, checkpoint_every: int = 0,
             eps: float = 1e-6) -> torch.Tensor:
    """Loss of a REF_CUDA solve with gradients w.r.t. the leaf data terms
    (`data`, [n_leaves, VZ, VY, VX] in `solver.leaves` order, on the GPU) and
    the per-vertex smoothness weights (`alpha`, [n_nodes]; the root's entry is
    unused).  The solver's parameters and smoothness images must be set."""
    return _HMFLoss.apply(data, alpha, solver, truth, int(checkpoint_every), float(eps))
