"""use_actual / sphere(actual=True): the exact-operator path (adjoint.cpp:33-83,148-170;
sphere.h:65-69) against the oracle's dense FP64 direct solve.

The reference solves the dense system by QR; the GPU path runs the same tree with every leaf pair
a dense FP64 block and BiCGSTAB to 1e-12, so the tolerances below are set by that residual
(coefficients 1e-9 absolute, gradients and pressures 1e-7 relative), far below the H-matrix
path's ACA-level agreement."""
import numpy as np
import pytest

from acoustic_reliefs_gb300 import meshes

from tests import cases

pytestmark = pytest.mark.gpu


def _pair(oracle_lib, precision="mixed"):
    from acoustic_reliefs_gb300.acoustics3d import DiffBEM
    R = meshes.relief(0.3, 0.3, 0.05, 10, 2, 10, 0, meshes.smooth_heightmap(16, 2))
    kw = dict(cluster_size=16, radius_factor=1.5, freq_bands=[1000.0, 2000.0], n_freqs=2, approx_ACA_tol=1e-4,
              Q_ACA_tol=1e-4, solver_tol=1e-6, src_pt=(0.0, 100.0, 0.0), listener_radius=50, listener_ds=15)
    gpu = DiffBEM(**kw, precision=precision)
    gpu.silent = True
    orc = oracle_lib.OracleDiffBEM(**kw)
    gpu.precompute(R.Ps, R.Es, R.diff_pts)
    orc.precompute(R.Ps, R.Es, R.diff_pts)
    gpu.use_actual = True
    orc.use_actual = True
    return gpu, orc, R


def test_use_actual_values_and_gradient_vs_oracle_dense(oracle_lib, gpu_lib):
    gpu, orc, R = _pair(oracle_lib)
    vg, vo = np.array(gpu.values()), np.array(orc.values())
    assert np.max(np.abs(vg - vo)) <= 1e-9
    x = np.random.default_rng(11).uniform(0, 0.02, size=len(R.diff_pts))
    assert abs(gpu.value(x) - orc.value(x)) <= 1e-9
    cg, gg = gpu.gradient(x)
    co, go = orc.gradient(x)
    assert abs(cg - co) <= 1e-9
    np.testing.assert_allclose(gg, go, rtol=0, atol=1e-7 * np.max(np.abs(go)))


def test_use_actual_is_scoped_to_the_coefficient_calls(oracle_lib, gpu_lib):
    """pvals keeps the H-matrix under use_actual (acoustics3d.cpp:236-280 ignores the flag), and
    switching the flag off returns the H-matrix coefficient exactly."""
    gpu, _, _ = _pair(oracle_lib)
    Ls = meshes.semicircle(5.0, 61)
    y_on = gpu.pvals(1500.0, Ls)
    c_exact = gpu.band_value(1000.0)
    gpu.use_actual = False
    y_off = gpu.pvals(1500.0, Ls)
    c_h = gpu.band_value(1000.0)
    assert np.array_equal(y_on, y_off)
    gpu.use_actual = True
    assert gpu.band_value(1000.0) == c_exact
    gpu.use_actual = False
    assert gpu.band_value(1000.0) == c_h
    assert abs(c_h - c_exact) < 1e-3  # H-matrix vs exact operator: ACA-level difference


def test_use_actual_follows_set_points(oracle_lib, gpu_lib):
    gpu, orc, R = _pair(oracle_lib)
    P2 = R.Ps.copy()
    P2[:, 1] *= 1.1
    gpu.set_points(P2)
    orc.Ps0 = P2.copy()
    assert abs(gpu.band_value(2000.0) - orc.band_value(2000.0)) <= 1e-9


def test_sphere_actual_vs_oracle_dense_and_mie(oracle_lib, gpu_lib):
    from acoustic_reliefs_gb300.acoustics3d import sphere
    c = cases.sphere_c1()
    LL, lrad = 90, 5.0
    y = sphere((c["Ps"], c["Es"]), c["freq"], LL, lrad, actual=True)
    m = oracle_lib.Mesh(c["Ps"], c["Es"], 128, 1.5)
    k = oracle_lib.wavenumber(c["freq"])
    th = np.arange(LL) / LL * 2 * np.pi
    Ls = np.stack([lrad * np.cos(th), np.zeros(LL), -lrad * np.sin(th)], axis=1)
    x = np.linalg.solve(m.dense_boundary(k), -m.rhs(k, (1.0, 0.0, 0.0), 1))
    y_ref = m.dense_listener(k, Ls) @ x
    assert cases.rel_l2(y, y_ref) <= 1e-7
    y_h = sphere((c["Ps"], c["Es"]), c["freq"], LL, lrad)
    assert cases.rel_l2(y_h, y_ref) <= 1e-6  # the H-matrix path at tolerance 1e-10
