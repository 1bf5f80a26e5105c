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

``TexMap`` / ``eval_uv`` / ``heights_from_texture`` run the reference's bilinear texture sampling
(acoustics_opt.py:23-33) and its transpose, the texture gradient of acoustic_gradient
(acoustics_opt.py:44-57), as CUDA kernels of the library (``ac3d_texmap_*``), so that autograd
carries the gradient from vertex heights back to a texture on the device; both directions are
bitwise the reference's NumPy results.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib as _L
from .acoustics3d import AC3DError, DiffBEM

__all__ = ["DiffusionCoefficient", "diffusion_coefficient", "TexMap", "eval_uv", "heights_from_texture"]


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


class TexMap:
    """Bilinear lookup of an (H, W) heightmap texture at fixed uv points, (0, 0) at the top-left
    texel's corner, indices clamped at the far edges (eval_uv, acoustics_opt.py:23-33), and its
    transpose. The texel indices and weights are built once for the uv set; ``tm(tex)`` is
    differentiable with respect to ``tex`` (a CUDA tensor)."""

    def __init__(self, uvs, shape):
        uv = uvs.detach().cpu().numpy() if isinstance(uvs, torch.Tensor) else uvs
        uv = np.ascontiguousarray(np.asarray(uv, dtype=np.float64).reshape(-1, 2))
        self.H, self.W = int(shape[0]), int(shape[1])
        self.n = len(uv)
        h = ctypes.c_void_p()
        rc = _L.lib().ac3d_texmap_create(ctypes.byref(h), _L.ptr(uv), self.n, self.H, self.W)
        if rc != _L.OK:
            raise AC3DError(rc, "invalid uvs or texture size, or no CUDA device")
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _L.lib().ac3d_texmap_destroy(h)
            except Exception:
                pass
            self._h = None

    def _stream(self, t: torch.Tensor) -> int:
        if not t.is_cuda:
            raise ValueError("the texture must be a CUDA tensor")
        return torch.cuda.current_stream(t.device).cuda_stream

    def sample(self, tex: torch.Tensor) -> torch.Tensor:
        """Heights (n,) FP64 from an (H, W) texture (no autograd)."""
        t = tex.detach().to(torch.float64).contiguous()
        if tuple(t.shape) != (self.H, self.W):
            raise ValueError(f"texture shape {tuple(t.shape)} != {(self.H, self.W)}")
        out = torch.empty(self.n, dtype=torch.float64, device=t.device)
        rc = _L.lib().ac3d_texmap_sample_dev(self._h, ctypes.c_void_p(t.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                             ctypes.c_void_p(self._stream(t)))
        if rc != _L.OK:
            raise AC3DError(rc, "texture lookup failed")
        return out

    def scatter(self, grad: torch.Tensor) -> torch.Tensor:
        """Texture gradient (H, W) FP64 from per-point gradients (n,)."""
        g = grad.detach().to(torch.float64).contiguous()
        if g.numel() != self.n:
            raise ValueError(f"gradient length {g.numel()} != {self.n}")
        out = torch.empty((self.H, self.W), dtype=torch.float64, device=g.device)
        rc = _L.lib().ac3d_texmap_scatter_dev(self._h, ctypes.c_void_p(g.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                              ctypes.c_void_p(self._stream(g)))
        if rc != _L.OK:
            raise AC3DError(rc, "texture scatter failed")
        return out

    def __call__(self, tex: torch.Tensor) -> torch.Tensor:
        return _TexSample.apply(tex, self)


class _TexSample(torch.autograd.Function):
    @staticmethod
    def forward(ctx, tex: torch.Tensor, tm: TexMap):
        ctx.tm, ctx.dtype = tm, tex.dtype
        return tm.sample(tex).to(tex.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        return ctx.tm.scatter(grad_out).to(ctx.dtype), None


def eval_uv(tex: torch.Tensor, uvs) -> torch.Tensor:
    """Bilinear sample of an (h, w) CUDA texture at (n, 2) uv coordinates (acoustics_opt.py:23-33),
    differentiable with respect to ``tex``. Builds the lookup for ``uvs`` on each call; hold a
    ``TexMap`` to reuse it."""
    return TexMap(uvs, tex.shape)(tex)


def heights_from_texture(tex: torch.Tensor, diff_uvs) -> torch.Tensor:
    """Heights of the differentiable vertices sampled from a heightmap texture (differentiable)."""
    return eval_uv(tex, diff_uvs)
