"""Full-size cases, checked through properties that need no oracle run at that size.

* The 200k-triangle relief (0.9 m, 256 x 256 heightmap, 210240 triangles) at 4 kHz with 16
  plane-wave directions as one block solve: every column converges, and the first column equals
  the single-right-hand-side solve of the same direction.
* The 80k-triangle relief (0.9 m, 128 x 128 heightmap, 81024 triangles, 37445 differentiable
  vertices) at 1 kHz, receivers on a 10 m semicircle: the adjoint gradient runs at full size, the
  coefficient it returns is the one value() returns, and storing or recomputing the matrices
  (recompute_matrices, adjoint.cpp:148-196) gives the same gradient."""
import numpy as np
import pytest

from acoustic_reliefs_gb300 import meshes
from acoustic_reliefs_gb300.acoustics3d import DiffBEM

from tests import cases

pytestmark = pytest.mark.gpu


def _dirs(n, seed):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d[:, 1] = -np.abs(d[:, 1]) - 0.5
    d[0] = [0.0, -1.0, 0.0]
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def test_block_solve_200k_triangles_4khz(gpu_lib):
    R = meshes.relief(0.9, 0.9, 0.05, 40, 7, 40, 3, meshes.smooth_heightmap(256, 0))
    assert len(R.Es) == 210240
    Ls = meshes.semicircle(10.0, 181)
    dirs = _dirs(16, 3)
    bem = DiffBEM(32, 2.0, [4000.0], 1, 1e-4, 1e-4, 1e-8, precision="mixed")
    bem.silent = True
    bem.set_mesh(R.Ps, R.Es)
    P = bem.pvals_multi(4000.0, dirs, Ls)
    st = bem.stats()
    assert P.shape == (16, 181) and np.all(np.isfinite(P))
    assert st["converged"] == 1 and st["solves"] == 16 and st["rel_residual"] <= 1e-8
    bem.set_incident("plane", dirs[0])
    y = bem.pvals(4000.0, Ls)
    assert bem.stats()["rel_residual"] <= 1e-8
    # both at relative residual 1e-8 on the same H-matrix
    assert cases.rel_l2(P[0], y) < 1e-5


def test_gradient_80k_triangles(gpu_lib):
    R = meshes.relief(0.9, 0.9, 0.05, 48, 7, 48, 2, meshes.smooth_heightmap(128, 0))
    assert len(R.Es) == 81024
    x = np.random.default_rng(4).uniform(0.0, 0.01, size=len(R.diff_pts))
    out = {}
    for recompute in (False, True):
        bem = DiffBEM(32, 2.0, [1000.0], 1, 1e-4, 1e-4, 1e-6, recompute_matrices=recompute, precision="mixed",
                      incident=("plane", (0.0, -1.0, 0.0)))
        bem.silent = True
        bem.set_listeners(meshes.semicircle(10.0, 181))
        bem.precompute(R.Ps, R.Es, R.diff_pts)
        c, g = bem.gradient(x)
        out[recompute] = (c, g, bem.value(x))
    c, g, v = out[False]
    assert 0.0 < c < 1.0 and np.all(np.isfinite(g)) and np.any(g != 0.0)
    assert abs(v - c) <= 1e-10  # one band: the band mean of value() is the band sum of gradient()
    c2, g2, _ = out[True]
    assert abs(c2 - c) <= 1e-10
    np.testing.assert_allclose(g2, g, rtol=0, atol=1e-10 * np.max(np.abs(g)))


def test_gradient_multi_80k_triangles_37_directions(gpu_lib):
    """The multi-incidence gradient at full size: the 0.9 m relief with a 128 x 128 heightmap
    (81024 triangles), 1, 2 and 4 kHz, 37 incidence angles in the xy plane, receivers on a 10 m
    semicircle: loss = 1 - mean coefficient and its gradient over all 37445 differentiable heights
    in one call. The coefficients agree with single-direction forward solves, and the gradient is
    finite."""
    import time
    R = meshes.relief(0.9, 0.9, 0.05, 48, 7, 48, 2, meshes.smooth_heightmap(128, 0))
    assert len(R.Es) == 81024
    th = np.radians(np.linspace(-90.0, 90.0, 37))
    dirs = np.stack([np.sin(th), -np.cos(th), np.zeros_like(th)], 1)
    freqs = [1000.0, 2000.0, 4000.0]
    x = np.random.default_rng(4).uniform(0.0, 0.01, size=len(R.diff_pts))
    bem = DiffBEM(32, 2.0, [1000.0], 1, 1e-4, 1e-4, 1e-6, precision="mixed")
    bem.silent = True
    bem.set_krylov("gmres")
    bem.set_listeners(meshes.semicircle(10.0, 181))
    bem.precompute(R.Ps, R.Es, R.diff_pts)
    t0 = time.perf_counter()
    loss, g, cf = bem.gradient_multi(x, freqs, dirs)
    dt = time.perf_counter() - t0
    st = bem.stats()
    print(f"37 directions x 3 frequencies on 81024 triangles: {dt:.2f} s, loss {loss:.6f}, "
          f"{st['solves']} solves, {st['iterations']} iterations")
    assert cf.shape == (3, 37) and np.all(np.isfinite(g)) and np.linalg.norm(g) > 0
    assert abs(loss - (1.0 - cf.mean())) < 1e-12
    for fi, di in ((0, 0), (2, 18)):
        b = DiffBEM(32, 2.0, [freqs[fi]], 1, 1e-4, 1e-4, 1e-6, precision="mixed", incident=("plane", dirs[di]))
        b.silent = True
        b.set_krylov("gmres")
        b.set_listeners(meshes.semicircle(10.0, 181))
        b.precompute(R.Ps, R.Es, R.diff_pts)
        assert abs(b.value(x) - cf[fi, di]) < 1e-4
