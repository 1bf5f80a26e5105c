"""torch.autograd binding: texture sampling on CPU, the GPU coefficient/gradient through autograd.

The texture lookup and its transpose are checked against the NumPy restatement of
acoustics_opt.py:24-56 in ``meshes``; the autograd function against ``DiffBEM.gradient`` (itself
checked against the oracle's adjoint in test_gpu_parity)."""
import numpy as np
import pytest
import torch

from acoustic_reliefs_gb300 import meshes
from acoustic_reliefs_gb300.autograd import diffusion_coefficient, eval_uv, heights_from_texture


def _uvs(n, seed):
    rng = np.random.default_rng(seed)
    uv = rng.uniform(0.0001, 0.9999, size=(n, 2))
    uv[:4] = [[0.0001, 0.0001], [0.9999, 0.9999], [0.0001, 0.9999], [0.5, 0.5]]  # corners, centre
    return uv


def test_eval_uv_matches_numpy_lookup():
    tex = np.random.default_rng(1).uniform(0, 0.1, size=(24, 32))
    uv = _uvs(500, 2)
    got = eval_uv(torch.from_numpy(tex), torch.from_numpy(uv)).numpy()
    np.testing.assert_allclose(got, meshes.sample_heightmap(tex, uv), rtol=0, atol=1e-15)


def test_eval_uv_backward_is_reference_scatter():
    tex = torch.from_numpy(np.random.default_rng(3).uniform(0, 0.1, size=(16, 16))).requires_grad_(True)
    uv = _uvs(300, 4)
    w = np.random.default_rng(5).normal(size=len(uv))
    (heights_from_texture(tex, torch.from_numpy(uv)) * torch.from_numpy(w)).sum().backward()
    np.testing.assert_allclose(tex.grad.numpy(), meshes.scatter_to_heightmap((16, 16), uv, w), rtol=0, atol=1e-12)


def _bem():
    from acoustic_reliefs_gb300.acoustics3d import DiffBEM
    R = meshes.relief(0.3, 0.3, 0.05, 10, 2, 10, 0, meshes.smooth_heightmap(16, 2))
    bem = DiffBEM(16, 1.5, [1000.0, 2000.0], 2, 1e-6, 1e-6, 1e-9, (0.0, 100.0, 0.0), 50, 15, False,
                  precision="fp64")
    bem.silent = True
    bem.precompute(R.Ps, R.Es, R.diff_pts)
    return bem, R


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["store", "recompute"])
@pytest.mark.parametrize("reduction", ["sum", "mean"])
def test_autograd_matches_gradient(gpu_lib, mode, reduction):
    bem, R = _bem()
    x = np.random.default_rng(6).uniform(0, 0.02, size=len(R.diff_pts))
    c_ref, g_ref = bem.gradient(x)
    scale = 1.0 if reduction == "sum" else 0.5
    h = torch.tensor(x, device="cuda", requires_grad=True)
    c = diffusion_coefficient(h, bem, mode, reduction)
    c.backward()
    assert abs(c.item() - scale * c_ref) <= 1e-10 * max(1.0, abs(c_ref))
    np.testing.assert_allclose(h.grad.cpu().numpy(), scale * g_ref, rtol=0,
                               atol=1e-9 * max(1.0, np.abs(g_ref).max()))


@pytest.mark.gpu
def test_autograd_texture_chain_matches_reference_glue(gpu_lib):
    """loss = 1 - c(eval_uv(tex)): tex.grad equals -(scatter of DiffBEM.gradient), which is what
    acoustic_gradient (acoustics_opt.py:37-60) hands to the optimizer."""
    bem, R = _bem()
    tex_np = np.random.default_rng(9).uniform(0, 0.02, size=(16, 16))
    tex = torch.tensor(tex_np, device="cuda", requires_grad=True)
    uv = torch.tensor(R.uvs, device="cuda")
    loss = 1 - diffusion_coefficient(heights_from_texture(tex, uv), bem)
    loss.backward()
    x = meshes.sample_heightmap(tex_np, R.uvs)
    c_ref, g_ref = bem.gradient(x)
    assert abs(loss.item() - (1 - c_ref)) <= 1e-10
    want = -meshes.scatter_to_heightmap(tex_np.shape, R.uvs, g_ref)
    np.testing.assert_allclose(tex.grad.cpu().numpy(), want, rtol=0, atol=1e-9 * max(1.0, np.abs(want).max()))
