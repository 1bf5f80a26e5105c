"""GPU parity: the CUDA path through the C-ABI against the FP64 oracle (golden fixtures and live
oracle runs) and the analytic Mie series. Tolerances: pressures 1e-4 relative L2, diffusion
coefficients 1e-3 absolute, per the accuracy contract of the path."""
import os

import numpy as np
import pytest

from acoustic_reliefs_gb300.acoustics3d import DiffBEM
from tests import cases

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
P_TOL = 1e-4


def gpu_pressures(c, precision, listener="dense"):
    bem = DiffBEM(c["leaf"], c["factor"], [c["freq"]], 1, c["aca_tol"], c["aca_tol"], c["tol"],
                  precision=precision, incident=("plane", c["vec"]), listener=listener)
    bem.silent = True
    _, Es = bem.set_mesh(c["Ps"], c["Es"])
    y = bem.pvals(c["freq"], c["Ls"])
    return y, bem, Es


@pytest.mark.parametrize("precision,listener", [("fp64", "dense"), ("mixed", "dense"), ("fp64", "aca"),
                                                ("mixed", "aca")])
def test_sphere_c1_vs_oracle_and_mie(gpu_lib, precision, listener):
    g = np.load(os.path.join(GOLDEN, "sphere_c1.npz"))
    c = cases.sphere_c1()
    y, bem, Es = gpu_pressures(c, precision, listener)
    assert np.array_equal(Es, g["Es_tree"])
    ref = g["y_oracle"] if listener == "aca" else g["y_oracle_dense"]
    assert cases.rel_l2(y, ref) < P_TOL
    assert cases.rel_l2(y, g["y_mie"]) < 2e-2
    st = bem.stats()
    assert st["converged"] == 1 and st["rel_residual"] <= c["tol"]


@pytest.mark.parametrize("precision,listener", [("fp64", "dense"), ("mixed", "dense"), ("mixed", "aca")])
def test_relief_vs_oracle(gpu_lib, precision, listener):
    g = np.load(os.path.join(GOLDEN, "relief_small.npz"))
    c = cases.relief_small()
    y, bem, Es = gpu_pressures(c, precision, listener)
    assert np.array_equal(Es, g["Es_tree"])
    ref = g["y_oracle_aca"] if listener == "aca" else g["y_oracle"]
    assert cases.rel_l2(y, ref) < P_TOL
    st = bem.stats()
    assert st["converged"] == 1 and st["rel_residual"] <= c["tol"]


def test_relief_surface_values_fp64(gpu_lib):
    g = np.load(os.path.join(GOLDEN, "relief_small.npz"))
    c = cases.relief_small()
    bem = DiffBEM(c["leaf"], c["factor"], [c["freq"]], 1, c["aca_tol"], c["aca_tol"], c["tol"], precision="fp64",
                  incident=("plane", c["vec"]))
    bem.silent = True
    bem.set_mesh(c["Ps"], c["Es"])
    x = bem.surface_vals(c["freq"])
    assert cases.rel_l2(x, g["x_oracle"]) < P_TOL


def test_repeatable_bitwise(gpu_lib):
    c = cases.relief_small()
    y1, _, _ = gpu_pressures(c, "mixed")
    y2, _, _ = gpu_pressures(c, "mixed")
    assert np.array_equal(y1, y2)


def small_diffbem(oracle_lib, precision, recompute=False, listener="dense", tol=1e-6, factor=1.5):
    R = cases.meshes.relief(0.3, 0.3, 0.05, 10, 2, 10, 0, cases.meshes.smooth_heightmap(16, 2))
    kw = dict(cluster_size=16, radius_factor=factor, freq_bands=[1000.0, 2000.0], n_freqs=3, approx_ACA_tol=tol,
              Q_ACA_tol=tol, solver_tol=1e-9, src_pt=(0.0, 100.0, 0.0), listener_radius=50, listener_ds=15,
              recompute_matrices=recompute)
    gpu = DiffBEM(**kw, precision=precision, listener=listener)
    gpu.silent = True
    orc = oracle_lib.OracleDiffBEM(**kw)
    Ps, Es = gpu.precompute(R.Ps, R.Es, R.diff_pts)
    orc.precompute(R.Ps, R.Es, R.diff_pts)
    return gpu, orc, R


@pytest.mark.parametrize("precision,listener", [("fp64", "dense"), ("mixed", "dense"), ("fp64", "aca")])
def test_diffbem_values_vs_oracle(oracle_lib, gpu_lib, precision, listener):
    gpu, orc, R = small_diffbem(oracle_lib, precision, listener=listener)
    vg = gpu.values()
    vo = orc.values()
    assert np.max(np.abs(np.array(vg) - np.array(vo))) < 1e-3
    assert abs(gpu.band_value(1000.0) - vo[0]) < 1e-3
    x = np.random.default_rng(5).uniform(0, 0.02, size=len(R.diff_pts))
    assert abs(gpu.value(x) - orc.value(x)) < 1e-3
    assert abs(gpu.value() - np.mean(vo)) < 1e-3


@pytest.mark.parametrize("precision,recompute,listener", [("fp64", False, "dense"), ("fp64", True, "dense"),
                                                          ("mixed", False, "dense"), ("fp64", False, "aca"),
                                                          ("fp64", True, "aca")])
def test_gradient_vs_oracle(oracle_lib, gpu_lib, precision, recompute, listener):
    gpu, orc, R = small_diffbem(oracle_lib, precision, recompute, listener)
    x = np.random.default_rng(6).uniform(0, 0.02, size=len(R.diff_pts))
    cg, gg = gpu.gradient(x)
    co, go = orc.gradient(x)
    assert abs(cg - co) < 1e-3
    assert np.linalg.norm(gg - go) / np.linalg.norm(go) < 1e-3


def test_gradient_vs_finite_differences(oracle_lib, gpu_lib):
    """Central differences (h = 1e-5 m) of the coefficient against the adjoint gradient.

    The adjoint differentiates the exact operator (derivatives of every entry), while an H-matrix
    forward model is not a smooth function of the geometry: ACA pivots can switch between x + h and
    x - h, which moves c by about the ACA tolerance, amplified 1/2h by the difference quotient (the
    FP64 oracle's H-matrix path shows the same, its dense path agrees with the adjoint to 1e-9).
    The check therefore uses an admissibility factor of 1e6, so that every leaf pair is a dense
    block and the forward operator is exact; the H-matrix gradient is checked against the oracle's
    adjoint in test_gradient_vs_oracle."""
    gpu, orc, R = small_diffbem(oracle_lib, "fp64", tol=1e-12, factor=1e6)
    gpu.set_band(1000.0)
    x = np.random.default_rng(7).uniform(0, 0.02, size=len(R.diff_pts))
    c, g = gpu.gradient(x)
    rng = np.random.default_rng(8)
    idx = rng.choice(len(x), size=8, replace=False)
    h = 1e-5
    for i in idx:
        e = np.zeros_like(x)
        e[i] = h
        fd = (gpu.value(x + e) - gpu.value(x - e)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-3 * max(1.0, np.max(np.abs(g)))
