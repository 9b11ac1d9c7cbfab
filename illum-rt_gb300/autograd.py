"""Differentiable closest hits for PyTorch, over the C-ABI.

``closest_hits(tracer, vpos, tris, rays)`` returns (t, beta, gamma, ref) for every ray, with t,
beta and gamma differentiable with respect to the vertex positions ``vpos`` [nv, 3] and the rays
[n, 8] (origin in columns 0-2, direction in 4-6). The hit triangle of each ray is held fixed:
the forward pass builds the BVH from the current vertices (with the reference builder on the
host, or with builder="gpu" with the GPU builder straight from the device tensor, which avoids
the round trip through host memory when the vertices change every step, or with
builder="refit", which refits the tree the tracer already holds for this mesh to the current
vertices and builds on the GPU only the first time) and traces with the selected tracer; the backward pass (grt_adjoint) recomputes each intersection
from the vertices and propagates dL/d(t, beta, gamma) to the three vertices and the ray.
Misses (t = FLT_MAX) get no gradient; mask them out of the loss.
"""
from __future__ import annotations

import numpy as np
import torch


def _topology_key(tris, nv: int):
    """Identity of a mesh's topology for the refit cache: the vertex and triangle counts and a
    64-bit digest of the triangle array's contents (index and value of every word mixed, summed
    modulo 2^64), so that a different triangle array, or an array edited in place, never reuses
    a tree built for other triangles. Tensors are digested on their own device."""
    if isinstance(tris, torch.Tensor):
        t = tris.detach().reshape(-1).to(torch.int64) & 0xFFFFFFFF
        i = torch.arange(1, t.numel() + 1, dtype=torch.int64, device=t.device)
    else:
        a = np.ascontiguousarray(tris, np.uint32).reshape(-1)
        t = torch.from_numpy(a.astype(np.int64))
        i = torch.arange(1, a.size + 1, dtype=torch.int64)
    w = i * -7046029254386353131  # odd 64-bit multiplier; products wrap modulo 2^64
    h1 = int(((t + 0x632BE5AB) * w).sum())
    h2 = int(((t ^ (w >> 29)) * (w | 1) * 0x2545F491).sum())
    return (int(nv), int(t.numel()), h1, h2)


class _ClosestHits(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vpos, rays, tracer, tris, builder):
        with torch.no_grad():
            stream = torch.cuda.current_stream(rays.device).cuda_stream
            if builder in ("gpu", "refit"):
                v4 = torch.ones((vpos.shape[0], 4), dtype=torch.float32, device=vpos.device)
                v4[:, :3] = vpos.detach()
                t4 = tris if isinstance(tris, torch.Tensor) else torch.from_numpy(
                    np.ascontiguousarray(tris, np.uint32).view(np.int32))
                key = _topology_key(tris, vpos.shape[0]) if builder == "refit" else None
                if builder == "refit" and getattr(tracer, "_refit_key", None) == key:
                    tracer.refit(v4, stream=stream)
                else:
                    tracer.build_device(v4, t4.to(vpos.device).contiguous(), stream=stream)
                    tracer._refit_key = key if builder == "refit" else None
            elif builder == "reference":
                v4 = np.ones((vpos.shape[0], 4), np.float32)
                v4[:, :3] = vpos.detach().cpu().numpy()
                tracer.build(v4, tris)
            else:
                raise ValueError(f"unknown builder {builder!r}")
            hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device=rays.device)
            tracer.trace(rays.detach(), hits, False, stream)
            tracer.check(stream)
        ctx.save_for_backward(vpos, rays, hits)
        ctx.tracer = tracer
        ref = hits[:, 3].view(torch.int32)
        ctx.mark_non_differentiable(ref)
        return hits[:, 0].clone(), hits[:, 1].clone(), hits[:, 2].clone(), ref.clone()

    @staticmethod
    def backward(ctx, gt, gb, gg, _gref):
        vpos, rays, hits = ctx.saved_tensors
        n = rays.shape[0]
        z = torch.zeros(n, dtype=torch.float32, device=rays.device)
        grad3 = torch.stack([gt if gt is not None else z, gb if gb is not None else z,
                             gg if gg is not None else z], dim=1).contiguous()
        grad_v = torch.zeros((vpos.shape[0], 3), dtype=torch.float32, device=rays.device)
        grad_r = torch.empty((n, 8), dtype=torch.float32, device=rays.device)
        stream = torch.cuda.current_stream(rays.device).cuda_stream
        ctx.tracer.adjoint(rays.detach().contiguous(), hits, grad3, grad_v, grad_r,
                           vpos=vpos.detach().contiguous(), stream=stream)
        return (grad_v if ctx.needs_input_grad[0] else None, grad_r if ctx.needs_input_grad[1] else None,
                None, None, None)


def closest_hits(tracer, vpos: torch.Tensor, tris, rays: torch.Tensor, builder: str = "reference"):
    """(t, beta, gamma, ref) of each ray, differentiable in vpos [nv, 3] and rays [n, 8].
    builder: "reference" (host build, hits bit-identical to the reference tracer with an exact
    tracer), "gpu" (GPU build; hits equal except near-ties) or "refit" (the tracer's tree
    refitted to the current vertices when it was built for triangles of the same contents, else
    a GPU build; hits equal except near-ties)."""
    return _ClosestHits.apply(vpos, rays, tracer, tris, builder)
