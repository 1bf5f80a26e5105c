"""Mixed-precision assembly in double-float arithmetic (the default, AC3D_ASSEMBLY_DF): near-field
entries, the admissible blocks' rows and columns and the ACA recursion (compute_ACA_block,
aca.cpp:38-82) evaluated to about 1e-13, everything stored in complex FP32. The low-rank blocks then have the FP64 path's
(and the FP64 oracle's) pivots and ranks, so the mixed operator is the FP64 operator rounded to
FP32 and the mixed pressures stay close to the FP64 path's. Tolerances: ranks equal except where two pivot candidates agree to rounding
(at most 0.1% of the blocks, none on these cases so far); pressures within 1e-5 relative L2 of
the FP64 path (the FP32 storage rounding, amplified by the conditioning)."""
import os

import numpy as np
import pytest

from acoustic_reliefs_gb300.acoustics3d import DiffBEM
from tests import cases

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
RANK_MISMATCH_FRAC = 1e-3
P_TOL_VS_FP64 = 1e-5


def solve(c, precision, assembly="df", freq=None):
    bem = DiffBEM(c["leaf"], c["factor"], [c["freq"]], 1, c["aca_tol"], c["aca_tol"], c["tol"],
                  precision=precision, incident=("plane", c["vec"]))
    bem.silent = True
    if precision == "mixed":
        bem.set_assembly(assembly)
    bem.set_mesh(c["Ps"], c["Es"])
    y = bem.pvals(freq or c["freq"], c["Ls"])
    return y, bem.ranks(), bem.stats()


def test_ranks_match_oracle(gpu_lib):
    """FP64 path and double-float mixed path against the FP64 oracle's per-block ranks (relief,
    5280 triangles, 2 kHz, leaf 32, factor 2, ACA 1e-4). The GPU does not store exactly-zero
    terms, so its ranks are the oracle's stored ranks (terms with u != 0 and v != 0)."""
    g = np.load(os.path.join(GOLDEN, "relief_small.npz"))
    c = cases.relief_small()
    _, r64, _ = solve(c, "fp64")
    _, rdf, _ = solve(c, "mixed", "df")
    assert len(r64) == len(g["ranks_stored"])
    for r in (r64, rdf):
        assert np.mean(r != g["ranks_stored"]) <= RANK_MISMATCH_FRAC
    assert np.mean(rdf != r64) <= RANK_MISMATCH_FRAC


@pytest.mark.parametrize("freq", [1000.0, 2000.0, 3500.0])
def test_mixed_df_close_to_fp64(gpu_lib, freq):
    """Both paths solve to relative residual 1e-9, so the difference is the FP32 storage of the
    double-float operator (with solves stopped at 1e-6, where each one stops moves the pressures
    by up to about cond(A) 1e-6, above this test's 1e-5)."""
    c = cases.relief_small(freq=freq)
    c["tol"] = 1e-9
    y64, r64, _ = solve(c, "fp64")
    ydf, rdf, st = solve(c, "mixed", "df")
    assert st["converged"] == 1 and st["rel_residual"] <= c["tol"]
    assert np.mean(rdf != r64) <= RANK_MISMATCH_FRAC
    assert cases.rel_l2(ydf, y64) < P_TOL_VS_FP64


def test_fp32_assembly_option(gpu_lib):
    """The FP32 assembly stays available and within the path's 1e-4 of the oracle."""
    g = np.load(os.path.join(GOLDEN, "relief_small.npz"))
    c = cases.relief_small()
    y, _, st = solve(c, "mixed", "fp32")
    assert st["converged"] == 1
    assert cases.rel_l2(y, g["y_oracle"]) < 1e-4


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_c2_vs_oracle(gpu_lib, precision):
    """The bench workload (20480 triangles, 2 kHz) against the committed FP64 oracle solve:
    pressures within 1e-4 relative L2, ranks equal to the oracle's stored ranks."""
    g = np.load(os.path.join(GOLDEN, "relief_c2.npz"))
    c = cases.relief_c2()
    bem = DiffBEM(c["leaf"], c["factor"], [c["freq"]], 1, c["aca_tol"], c["aca_tol"], c["tol"],
                  precision=precision, incident=("plane", c["vec"]))
    bem.silent = True
    bem.set_krylov("gmres")
    _, Es = bem.set_mesh(c["Ps"], c["Es"])
    assert np.array_equal(Es, g["Es_tree"])
    y = bem.pvals(c["freq"], c["Ls"])
    assert cases.rel_l2(y, g["y_oracle"]) < 1e-4
    assert np.mean(bem.ranks() != g["ranks_stored"]) <= RANK_MISMATCH_FRAC


def test_receiver_aca_mixed_close_to_fp64(gpu_lib):
    """The receiver ACA (compute_ACA_listener, aca.cpp:84-134) of the mixed path runs in double-float
    as well: with tolerance 1e-5, mixed and FP64 receiver pressures agree to the FP32 storage level."""
    c = cases.relief_small()
    out = {}
    for prec in ("fp64", "mixed"):
        bem = DiffBEM(c["leaf"], c["factor"], [c["freq"]], 1, 1e-5, 1e-5, 1e-8, precision=prec,
                      incident=("plane", c["vec"]), listener="aca")
        bem.silent = True
        bem.set_mesh(c["Ps"], c["Es"])
        out[prec] = bem.pvals(c["freq"], c["Ls"])
    assert cases.rel_l2(out["mixed"], out["fp64"]) < P_TOL_VS_FP64
