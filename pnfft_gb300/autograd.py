"""pnfft_trafo as a torch.autograd.Function over the C ABI.

    f = trafo(f_hat, x)         f_j = sum_k f_hat_k exp(-2 pi i k.x_j) (NFFT)

Backward, with g = dL/df in PyTorch's convention (2 dL/d conj(f)):
  * d/d f_hat = adj(g): the adjoint NFFT (spreading B^T, F^H, D^T);
  * d/d x_j   = Re(conj(g_j) grad f(x_j)), grad f from the interpolation with
                the window-derivative kernel (PNFFT_COMPUTE_GRAD_F, AD).
The node binning computed in the forward pass is reused by the backward pass
(the nodes are declared fixed between the two).

f_hat: complex tensor in the plan's layout (N0 x N1 x N2, or flat); x: (M, 3)
real tensor on the same CUDA device.  Results have f_hat's dtype; the device
path is the plan's (FP32-mixed or FP64).
"""
import torch

from . import COMPUTE_F, COMPUTE_GRAD_F, Plan  # noqa: F401


class NfftTrafo(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f_hat, x, plan):
        fh = f_hat.reshape(-1).to(torch.complex128).contiguous()
        xd = x.detach().to(torch.float64).contiguous()
        plan._nodes_for(xd.shape[0])
        from . import load
        load().pnfft_gb300_nodes_set_fixed(plan._nodes, 1)  # new coordinates: bin once, reuse in backward
        plan._fixed = True
        f, _, _ = plan.trafo_device(xd, fh, COMPUTE_F, fixed_nodes=True)
        ctx.plan = plan
        ctx.shape = f_hat.shape
        ctx.dtype = f_hat.dtype
        ctx.xdtype = x.dtype
        ctx.save_for_backward(fh, xd)
        return f.to(f_hat.dtype)

    @staticmethod
    def backward(ctx, g):
        fh, xd = ctx.saved_tensors
        plan = ctx.plan
        g = g.to(torch.complex128).contiguous()
        grad_fhat = grad_x = None
        if ctx.needs_input_grad[0]:
            a = plan.adj_device(xd, g, fixed_nodes=True)
            grad_fhat = a.to(ctx.dtype).reshape(ctx.shape)
        if ctx.needs_input_grad[1]:
            _, gf, _ = plan.trafo_device(xd, fh, COMPUTE_GRAD_F, fixed_nodes=True)
            grad_x = (torch.conj(g)[:, None] * gf).real.to(ctx.xdtype)
        return grad_fhat, grad_x, None


def trafo(f_hat, x, plan):
    """Differentiable NFFT: f (M,) = trafo(f_hat, x) on `plan`."""
    return NfftTrafo.apply(f_hat, x, plan)
