"""torch.autograd binding: the device texture lookup and its transpose, and the GPU
coefficient / gradient through autograd.

The texture lookup and its transpose (ac3d_texmap_*) are checked bitwise against the NumPy
restatement of acoustics_opt.py:23-57 in ``meshes``; the autograd function against
``DiffBEM.gradient`` (itself checked against the oracle's adjoint in test_gpu_parity)."""
import numpy as np
import pytest
import torch

from acoustic_reliefs_gb300 import meshes
from acoustic_reliefs_gb300.autograd import TexMap, diffusion_coefficient, eval_uv, heights_from_texture


def _uvs(n, seed):
    rng = np.random.default_rng(seed)
    uv = rng.uniform(0.0001, 0.9999, size=(n, 2))
    # corners, centre, the texture's edges and texel centres
    uv[:8] = [[0.0001, 0.0001], [0.9999, 0.9999], [0.0001, 0.9999], [0.5, 0.5], [0.0, 0.0], [1.0, 1.0],
              [0.0, 1.0], [1.0 / 64, 3.0 / 64]]
    return uv


@pytest.mark.gpu
def test_eval_uv_matches_numpy_lookup(gpu_lib):
    tex = np.random.default_rng(1).uniform(0, 0.1, size=(24, 32))
    uv = _uvs(500, 2)
    got = eval_uv(torch.tensor(tex, device="cuda"), torch.from_numpy(uv)).cpu().numpy()
    assert np.array_equal(got, meshes.sample_heightmap(tex, uv))


@pytest.mark.gpu
def test_eval_uv_backward_is_reference_scatter(gpu_lib):
    tex = torch.tensor(np.random.default_rng(3).uniform(0, 0.1, size=(16, 16)), device="cuda", requires_grad=True)
    uv = _uvs(300, 4)
    w = np.random.default_rng(5).normal(size=len(uv))
    (heights_from_texture(tex, uv) * torch.tensor(w, device="cuda")).sum().backward()
    assert np.array_equal(tex.grad.cpu().numpy(), meshes.scatter_to_heightmap((16, 16), uv, w))


@pytest.mark.gpu
def test_texmap_reuse_on_the_relief(gpu_lib):
    """A TexMap built once serves every step: the 64 x 64 relief's 4225 top vertices."""
    R = meshes.relief_20k(0)
    tm = TexMap(R.uvs, (64, 64))
    for seed in range(3):
        tex = np.random.default_rng(seed).uniform(0, 0.1, size=(64, 64))
        h = tm.sample(torch.tensor(tex, device="cuda")).cpu().numpy()
        assert np.array_equal(h, meshes.sample_heightmap(tex, R.uvs))
    g = np.random.default_rng(9).normal(size=len(R.uvs))
    assert np.array_equal(tm.scatter(torch.tensor(g, device="cuda")).cpu().numpy(),
                          meshes.scatter_to_heightmap((64, 64), R.uvs, g))


def test_texmap_needs_cuda_tensors():
    """No CPU fallback: a CPU texture is rejected before any work (the library must be built)."""
    pytest.importorskip("ctypes")
    from acoustic_reliefs_gb300 import _lib
    try:
        _lib.lib()
    except RuntimeError:
        pytest.skip("library not built")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(Exception):
        eval_uv(torch.zeros(4, 4, dtype=torch.float64), np.full((2, 2), 0.5))


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
