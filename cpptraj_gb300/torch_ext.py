"""torch.autograd.Function over the C ABI: all-pairs RMSD with a hand-written
CUDA backward (gbr_rmsd_backward).

    from cpptraj_gb300.torch_ext import allpairs_rmsd
    tri = allpairs_rmsd(xyz)          # xyz: [F, N, 3] float32 CUDA tensor, requires_grad
    tri.sum().backward()              # xyz.grad = dL/dxyz

The forward returns the upper triangle in cpptraj's TRI order.  The backward
recomputes every pair's rotation on the GPU instead of storing it.
"""
from __future__ import annotations

import torch

from . import gbrmsd


class AllPairsRMSD(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, mass, precision, device_index):
        if not xyz.is_cuda or xyz.dtype != torch.float32:
            raise TypeError("allpairs_rmsd needs a float32 CUDA tensor")
        xyz = xyz.contiguous()
        h = gbrmsd.default_handle(device_index)
        h.set_stream(torch.cuda.current_stream(xyz.device).cuda_stream)
        out = h.allpairs(xyz, tgt_mass=mass, precision=precision)
        ctx.save_for_backward(xyz)
        ctx.mass = mass
        ctx.device_index = device_index
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (xyz,) = ctx.saved_tensors
        h = gbrmsd.default_handle(ctx.device_index)
        h.set_stream(torch.cuda.current_stream(xyz.device).cuda_stream)
        g = grad_out.contiguous().to(torch.float32)
        grad = torch.empty_like(xyz)
        h.backward(xyz, mass=ctx.mass, g=g, grad=grad)
        return grad, None, None, None


def allpairs_rmsd(xyz: torch.Tensor, mass=None, precision: str = "tc") -> torch.Tensor:
    """Differentiable all-pairs best-fit RMSD (TRI order) of one frame set."""
    dev = xyz.device.index if xyz.device.index is not None else torch.cuda.current_device()
    return AllPairsRMSD.apply(xyz, mass, precision, dev)
