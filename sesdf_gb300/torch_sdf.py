"""Optional torch binding: the SES signed distance and the SES area as differentiable
functions.

    sdf = ses_sdf(atoms, queries, probe_radius=1.4)
    area = ses_area(atoms, probe_radius=1.4)   # scalar tensor, A^2

atoms is a CUDA float32 tensor [n, 4] (x, y, z, vdW radius), queries a CUDA
float32 tensor [m, 3]. The forward pass builds the full surface (sesgb_build_device)
and evaluates sesgb_sdf; the backward pass calls sesgb_sdf_backward, which searches
the active primitives again and returns d L / d atoms [n, 4] (coordinates and radii).
The queries receive no gradient. Both passes run on the current CUDA stream.
"""
from __future__ import annotations

import torch

from .api import SesBuild


class SesSdf(torch.autograd.Function):
    @staticmethod
    def forward(ctx, atoms: torch.Tensor, queries: torch.Tensor, probe_radius: float = 1.4):
        if not atoms.is_cuda or atoms.dtype != torch.float32 or atoms.dim() != 2 or atoms.shape[1] != 4:
            raise ValueError("atoms must be a CUDA float32 tensor [n, 4]")
        a = atoms.detach().contiguous()
        q = queries.detach().contiguous().to(torch.float32)
        stream = torch.cuda.current_stream().cuda_stream
        g = SesBuild(a.cpu().numpy(), probe_radius, "full")
        g.build_device(a.data_ptr(), stream)
        out = torch.empty(q.shape[0], dtype=torch.float32, device=a.device)
        g.sdf(q.data_ptr(), q.shape[0], out.data_ptr(), None, stream)
        ctx.build = g
        ctx.save_for_backward(q)
        ctx.n = a.shape[0]
        return out

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        (q,) = ctx.saved_tensors
        g = ctx.build
        go = grad_out.detach().contiguous().to(torch.float32)
        grad = torch.empty((ctx.n, 4), dtype=torch.float32, device=q.device)
        g.sdf_backward(q.data_ptr(), q.shape[0], go.data_ptr(), grad.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.current_stream().synchronize()
        g.close()
        return grad, None, None


def ses_sdf(atoms: torch.Tensor, queries: torch.Tensor, probe_radius: float = 1.4) -> torch.Tensor:
    return SesSdf.apply(atoms, queries, probe_radius)


class SesArea(torch.autograd.Function):
    """Total SES area of the build's primitives; backward: sesgb_ses_area_backward."""

    @staticmethod
    def forward(ctx, atoms: torch.Tensor, probe_radius: float = 1.4):
        if not atoms.is_cuda or atoms.dtype != torch.float32 or atoms.dim() != 2 or atoms.shape[1] != 4:
            raise ValueError("atoms must be a CUDA float32 tensor [n, 4]")
        a = atoms.detach().contiguous()
        stream = torch.cuda.current_stream().cuda_stream
        g = SesBuild(a.cpu().numpy(), probe_radius, "full")
        g.build_device(a.data_ptr(), stream)
        area = g.ses_area(None, stream)["total"]
        ctx.build = g
        ctx.n = a.shape[0]
        ctx.device = a.device
        return torch.tensor(area, dtype=torch.float32, device=a.device)

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        g = ctx.build
        gs = float(grad_out.detach().cpu())
        grad = torch.empty((ctx.n, 4), dtype=torch.float32, device=ctx.device)
        g.ses_area_backward(grad.data_ptr(), (gs, gs, gs), torch.cuda.current_stream().cuda_stream)
        torch.cuda.current_stream().synchronize()
        g.close()
        return grad, None


def ses_area(atoms: torch.Tensor, probe_radius: float = 1.4) -> torch.Tensor:
    return SesArea.apply(atoms, probe_radius)
