"""GPU: the multi-incidence objective (ac3d_gradient_multi): loss = 1 - mean over frequencies x
plane-wave directions of the single-frequency diffusion coefficient at the receivers, with its
adjoint gradient over the differentiable heights (adjoint.cpp:24-242 per frequency and direction;
here the directions of a frequency share one H-matrix, block solves in both orientations and
every shape-derivative evaluation).

* Against the single-direction path (DiffBEM.gradient, one band of one frequency per call): the
  loss within 1e-6 and the gradient within 1e-4 relative L2 of the mean of the singles (both
  solve to 1e-8, through different Krylov paths).
* Central finite differences (h = 1e-5 m) on an exact operator (radius factor 1e3: every block is
  near, nothing is approximated by ACA) in FP64: each checked derivative within 1e-3 relative of
  the largest checked derivative. ACA's pivot choice is not a smooth function of the heights, so
  finite differences of an H-matrix objective measure pivot switches, not the derivative.
* Mixed precision against FP64 on the same case: gradient within 1e-3 relative L2.
"""
import numpy as np
import pytest

from acoustic_reliefs_gb300 import meshes
from acoustic_reliefs_gb300.acoustics3d import DiffBEM

pytestmark = pytest.mark.gpu


def _dirs(n, seed):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d[:, 1] = -np.abs(d[:, 1]) - 0.5
    d[0] = [0.0, -1.0, 0.0]
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def _bem(R, freq, precision, factor=2.0, leaf=32, tol=1e-8, direction=(0.0, -1.0, 0.0)):
    bem = DiffBEM(leaf, factor, [freq], 1, 1e-6, 1e-6, tol, precision=precision, incident=("plane", direction))
    bem.silent = True
    bem.set_listeners(meshes.semicircle(10.0, 91))
    bem.precompute(R.Ps, R.Es, R.diff_pts)
    return bem


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_multi_equals_mean_of_singles(gpu_lib, precision):
    R = meshes.relief(0.6, 0.6, 0.05, 16, 4, 16, 0, meshes.smooth_heightmap(64, 1))
    x = np.random.default_rng(2).uniform(0.0, 0.01, size=len(R.diff_pts))
    freqs = [800.0, 1600.0]
    dirs = _dirs(5, 7)
    bem = _bem(R, freqs[0], precision)
    bem.set_krylov("gmres")
    loss, g, cf = bem.gradient_multi(x, freqs, dirs)
    assert cf.shape == (2, 5) and np.all(np.isfinite(g))
    cs, gs = [], []
    for f in freqs:
        for d in dirs:
            b = _bem(R, f, precision, direction=d)
            c1, g1 = b.gradient(x)
            cs.append(c1)
            gs.append(g1)
    assert abs(loss - (1 - np.mean(cs))) < 1e-6
    np.testing.assert_allclose(cf.reshape(-1), cs, atol=1e-6)
    gref = -np.mean(gs, axis=0)
    assert np.linalg.norm(g - gref) / np.linalg.norm(gref) < 1e-4


@pytest.fixture(scope="module")
def exact_case():
    R = meshes.relief(0.3, 0.3, 0.05, 6, 2, 6, 0, meshes.smooth_heightmap(16, 3))
    x = np.random.default_rng(5).uniform(0.0, 0.01, size=len(R.diff_pts))
    return R, x


def test_multi_gradient_finite_differences(gpu_lib, exact_case):
    R, x = exact_case
    freqs = [1500.0, 3000.0]
    dirs = _dirs(3, 11)
    bem = _bem(R, freqs[0], "fp64", factor=1e3, tol=1e-12)
    loss, g, _ = bem.gradient_multi(x, freqs, dirs)
    rng = np.random.default_rng(9)
    idx = rng.choice(len(x), size=min(16, len(x)), replace=False)
    h = 1e-5
    fd = []
    for i in idx:
        e = np.zeros_like(x)
        e[i] = h
        lp = bem.gradient_multi(x + e, freqs, dirs)[0]
        lm = bem.gradient_multi(x - e, freqs, dirs)[0]
        fd.append((lp - lm) / (2 * h))
    fd = np.array(fd)
    scale = np.max(np.abs(fd))
    assert scale > 0
    assert np.max(np.abs(g[idx] - fd)) < 1e-3 * scale


def test_multi_gradient_mixed_vs_fp64(gpu_lib, exact_case):
    R, x = exact_case
    freqs = [1500.0, 3000.0]
    dirs = _dirs(3, 11)
    g64 = _bem(R, freqs[0], "fp64", factor=1e3, tol=1e-10).gradient_multi(x, freqs, dirs)[1]
    g32 = _bem(R, freqs[0], "mixed", factor=1e3, tol=1e-10).gradient_multi(x, freqs, dirs)[1]
    assert np.linalg.norm(g32 - g64) / np.linalg.norm(g64) < 1e-3



def test_multi_gradient_tensor_cores(gpu_lib):
    """The transposed block solves with the tensor-core dot pass give the gradient of the
    CUDA-core run within 1e-5 relative L2 (every solve to 1e-8)."""
    R = meshes.relief(0.6, 0.6, 0.05, 16, 4, 16, 0, meshes.smooth_heightmap(64, 1))
    x = np.random.default_rng(4).uniform(0.0, 0.01, size=len(R.diff_pts))
    dirs = _dirs(9, 5)
    out = {}
    for tc in (True, False):
        bem = _bem(R, 1200.0, "mixed")
        bem.set_krylov("gmres")
        bem.set_tensor_cores(tc)
        out[tc] = bem.gradient_multi(x, [1200.0], dirs)
    assert abs(out[True][0] - out[False][0]) < 1e-7
    assert np.linalg.norm(out[True][1] - out[False][1]) / np.linalg.norm(out[False][1]) < 1e-5
