"""Block (multi-right-hand-side) solves: ac3d_solve_multi against one-at-a-time solves of the same
H-matrix and against the oracle's golden pressures (normal incidence on the small relief)."""
import os

import numpy as np
import pytest

from acoustic_reliefs_gb300.acoustics3d import DiffBEM
from tests import cases

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _dirs(n, seed):
    """Seeded plane-wave directions in the lower hemisphere, the first one normal incidence."""
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d[:, 1] = -np.abs(d[:, 1]) - 0.5
    d[0] = [0.0, -1.0, 0.0]
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def _bem(c, precision, tol=None):
    bem = DiffBEM(c["leaf"], c["factor"], [c["freq"]], 1, c["aca_tol"], c["aca_tol"], tol or c["tol"],
                  precision=precision)
    bem.silent = True
    bem.set_mesh(c["Ps"], c["Es"])
    return bem


@pytest.mark.gpu
@pytest.mark.parametrize("nrhs", [3, 7, 16, 20])
def test_block_solve_matches_single_solves(gpu_lib, nrhs):
    """Mixed precision, solver tolerance 1e-9: every column of the block solve meets it and agrees
    with the single-right-hand-side solve of the same direction (same H-matrix, different Krylov
    paths) within 1e-6 relative L2."""
    c = cases.relief_small()
    dirs = _dirs(nrhs, 1)
    bem = _bem(c, "mixed", tol=1e-9)
    P = bem.pvals_multi(c["freq"], dirs, c["Ls"])
    st = bem.stats()
    assert P.shape == (nrhs, len(c["Ls"]))
    assert st["converged"] == 1 and st["rel_residual"] <= 1e-9 and st["solves"] == nrhs
    for i, d in enumerate(dirs):
        bem.set_incident("plane", d)
        y = bem.pvals(c["freq"], c["Ls"])
        assert cases.rel_l2(P[i], y) < 1e-6, i


@pytest.mark.gpu
def test_block_solve_vs_oracle_golden(gpu_lib):
    g = np.load(os.path.join(GOLDEN, "relief_small.npz"))
    c = cases.relief_small()
    bem = _bem(c, "mixed")
    P, X = bem.pvals_multi(c["freq"], _dirs(5, 2), c["Ls"], surface=True)
    assert cases.rel_l2(P[0], g["y_oracle"]) < 1e-4
    assert cases.rel_l2(X[0], g["x_oracle"]) < 1e-4


@pytest.mark.gpu
def test_block_solve_fp64_is_single_solves(gpu_lib):
    """FP64 storage runs the columns through the FP64 single-vector solver: bitwise equal."""
    c = cases.relief_small()
    dirs = _dirs(3, 3)
    bem = _bem(c, "fp64")
    P = bem.pvals_multi(c["freq"], dirs, c["Ls"])
    for i, d in enumerate(dirs):
        bem.set_incident("plane", d)
        assert np.array_equal(P[i], bem.pvals(c["freq"], c["Ls"]))


@pytest.mark.gpu
def test_block_solve_point_sources_and_repeatable(gpu_lib):
    c = cases.relief_small()
    srcs = np.array([[0.0, 5.0, 0.0], [1.0, 3.0, -0.5], [0.2, 10.0, 0.3], [-2.0, 4.0, 1.0]])
    bem = _bem(c, "mixed")
    P1 = bem.pvals_multi(c["freq"], srcs, c["Ls"], kind="point")
    P2 = bem.pvals_multi(c["freq"], srcs, c["Ls"], kind="point")
    assert np.array_equal(P1, P2)
    bem.set_incident("point", srcs[1])
    assert cases.rel_l2(P1[1], bem.pvals(c["freq"], c["Ls"])) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("nrhs", [6, 16])
def test_tensor_core_dot_pass_matches_cuda_cores(gpu_lib, nrhs):
    """The block dot pass on the tensor cores (tcgen05, TF32 split in three products, from the
    split segments) and on the FP32 CUDA cores solve to the same answers: both runs reach relative
    residual 1e-8 on the same H-matrix, so their pressures agree to about that level."""
    c = cases.relief_small()
    rng = np.random.default_rng(3)
    dirs = rng.normal(size=(nrhs, 3))
    dirs[:, 1] = -np.abs(dirs[:, 1]) - 0.5
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    out = {}
    for tc in (True, False):
        bem = DiffBEM(c["leaf"], c["factor"], [c["freq"]], 1, c["aca_tol"], c["aca_tol"], 1e-8, precision="mixed")
        bem.silent = True
        bem.set_krylov("gmres")
        bem.set_tensor_cores(tc)
        bem.set_mesh(c["Ps"], c["Es"])
        out[tc] = bem.pvals_multi(c["freq"], dirs, c["Ls"])
        st = bem.stats()
        assert st["converged"] == 1 and st["rel_residual"] <= 1e-8
    assert cases.rel_l2(out[True], out[False]) < 1e-6
