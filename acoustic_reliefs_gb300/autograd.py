"""torch.autograd bindings of the GPU diffusion coefficient and its adjoint gradient.

``DiffusionCoefficient`` wraps ``DiffBEM.gradient`` (acoustics3d_cpp/src/acoustics3d.cpp:199-234,
adjoint.cpp:24-242) as a differentiable function of the heights of the differentiable vertices:
the heights stay in device memory, and the value and gradient are written by the library's
kernels into device tensors on torch's current stream, so an optimizer step makes no host round
trip of the gradient (the reference's ``acoustic_gradient`` copies it through NumPy,
acoustics_opt.py:37-60).

Two modes, mirroring the store-or-recompute choice of ``recompute_matrices``:
  "store"     (default) the forward pass runs the forward solves and the adjoint together and keeps
              the gradient for backward;
  "recompute" the forward pass computes only the value; backward runs forward and adjoint again.

``reduction`` "sum" returns the band sum, as ``DiffBEM.gradient`` does; "mean" the band mean, as
``DiffBEM.value`` does (acoustics3d.cpp:128 vs :224-233). The gradient is always that of the value
returned.

``eval_uv`` / ``heights_from_texture`` restate the reference's bilinear texture sampling
(acoustics_opt.py:24-34) in torch, so that autograd carries the gradient from vertex heights back to
a texture (the scatter of acoustics_opt.py:43-56).
"""
from __future__ import annotations

import torch

from .acoustics3d import DiffBEM

__all__ = ["DiffusionCoefficient", "diffusion_coefficient", "eval_uv", "heights_from_texture"]


def _run(bem: DiffBEM, h: torch.Tensor, want_grad: bool):
    c = torch.empty((), dtype=torch.float64, device=h.device)
    stream = torch.cuda.current_stream(h.device).cuda_stream
    if want_grad:
        g = torch.empty_like(h)
        bem.gradient_dev(h.data_ptr(), c.data_ptr(), g.data_ptr(), stream)
        return c, g
    bem.value_dev(h.data_ptr(), c.data_ptr(), stream)
    return c * bem.n_bands, None  # value_dev gives the band mean


class DiffusionCoefficient(torch.autograd.Function):
    """c = DiffusionCoefficient.apply(heights, bem, mode, reduction); heights: (HH,) CUDA tensor."""

    @staticmethod
    def forward(ctx, heights: torch.Tensor, bem: DiffBEM, mode: str = "store", reduction: str = "sum"):
        if not heights.is_cuda:
            raise ValueError("heights must be a CUDA tensor")
        if mode not in ("store", "recompute"):
            raise ValueError(f"mode must be 'store' or 'recompute', not {mode!r}")
        if reduction not in ("sum", "mean"):
            raise ValueError(f"reduction must be 'sum' or 'mean', not {reduction!r}")
        h = heights.detach().to(torch.float64).contiguous()
        scale = 1.0 if reduction == "sum" else 1.0 / bem.n_bands
        store = mode == "store" and ctx.needs_input_grad[0]
        c, g = _run(bem, h, store)
        ctx.bem, ctx.scale, ctx.in_dtype = bem, scale, heights.dtype
        ctx.save_for_backward(h, g if store else None)
        return (c * scale).to(heights.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        h, g = ctx.saved_tensors
        if g is None:
            _, g = _run(ctx.bem, h, True)
        return (grad_out.to(torch.float64) * ctx.scale * g).to(ctx.in_dtype), None, None, None


def diffusion_coefficient(heights: torch.Tensor, bem: DiffBEM, mode: str = "store",
                          reduction: str = "sum") -> torch.Tensor:
    return DiffusionCoefficient.apply(heights, bem, mode, reduction)


def eval_uv(tex: torch.Tensor, uvs: torch.Tensor) -> torch.Tensor:
    """Bilinear sample of an (h, w) texture at (n, 2) uv coordinates, (0, 0) at the top-left texel's
    corner, indices clamped at the far edges (acoustics_opt.py:24-34)."""
    h, w = tex.shape
    u = uvs[:, 0].to(tex.dtype) * w - 0.5
    v = uvs[:, 1].to(tex.dtype) * h - 0.5
    # numpy.modf splits toward zero; negative fractions are wrapped to 1 + f as the reference does
    ui_t, vi_t = torch.trunc(u), torch.trunc(v)
    uf, vf = u - ui_t, v - vi_t
    uf = torch.where(uf < 0, 1 + uf, uf)
    vf = torch.where(vf < 0, 1 + vf, vf)
    ui = ui_t.to(torch.int64).clamp_min(0)
    vi = vi_t.to(torch.int64).clamp_min(0)
    ui1 = (ui + 1).clamp_max(w - 1)
    vi1 = (vi + 1).clamp_max(h - 1)
    return ((1 - vf) * (1 - uf) * tex[vi, ui] + (1 - vf) * uf * tex[vi, ui1] + vf * (1 - uf) * tex[vi1, ui] +
            vf * uf * tex[vi1, ui1])


def heights_from_texture(tex: torch.Tensor, diff_uvs: torch.Tensor) -> torch.Tensor:
    """Heights of the differentiable vertices sampled from a heightmap texture (differentiable)."""
    return eval_uv(tex, diff_uvs)
