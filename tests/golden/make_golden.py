"""Writes the golden fixtures of tests/golden/ (run from the repository root).

sphere_c1.npz: the 1280-triangle icosphere case -- tree-ordered connectivity, receiver pressures
of the FP64 oracle with the reference's ACA receiver matrix (y_oracle) and with the exact receiver
matrix (y_oracle_dense), and the analytic Mie series at the same receivers.
relief_small.npz: the 5280-triangle relief case -- oracle receiver pressures (FP64, ACA 1e-4,
tol 1e-6) with the exact (y_oracle) and ACA (y_oracle_aca) receiver matrix, surface solution,
per-block ACA ranks (iterations, the reference's count) and stored ranks (terms with u != 0 and
v != 0), used by the GPU parity tests without re-running the oracle.
relief_c2.npz: the bench workload (0.6 m relief, 20480 triangles, 2 kHz, normal plane wave, 181
receivers on a 5 m semicircle, leaf 32, factor 2, ACA 1e-4, tol 1e-6) -- oracle pressures with the
exact receiver matrix and the stored ranks.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import mie  # noqa: E402
from tests import cases  # noqa: E402


def main():
    out = os.path.dirname(os.path.abspath(__file__))
    c = cases.sphere_c1()
    m = oracle.Mesh(c["Ps"], c["Es"], c["leaf"], c["factor"])
    k = oracle.wavenumber(c["freq"])
    y, x, info = oracle.solve_pressures(m, k, c["vec"], 1, c["Ls"], c["aca_tol"], c["aca_tol"], c["tol"])
    yd = oracle.mesh_dense_listener_apply(m, k, c["Ls"], x)
    th = np.arccos(np.clip(c["Ls"] @ c["vec"] / 5.0, -1, 1))
    np.savez_compressed(os.path.join(out, "sphere_c1.npz"), Es_tree=m.Es, y_oracle=y, y_oracle_dense=yd,
                        y_mie=mie.scattered_pressure(5.0, th, k, 0.5))
    c = cases.relief_small()
    m = oracle.Mesh(c["Ps"], c["Es"], c["leaf"], c["factor"])
    k = oracle.wavenumber(c["freq"])
    y, x, info = oracle.solve_pressures(m, k, c["vec"], 1, c["Ls"], c["aca_tol"], c["aca_tol"], c["tol"],
                                        listener="dense")
    ya = oracle.ListenerACA(m, k, c["Ls"], c["aca_tol"]).apply(x)
    H = oracle.HMat(m, k, c["aca_tol"])
    assert np.array_equal(H.ranks, info["ranks"])
    np.savez_compressed(os.path.join(out, "relief_small.npz"), Es_tree=m.Es, y_oracle=y, y_oracle_aca=ya,
                        x_oracle=x, ranks=info["ranks"], ranks_stored=H.stored_ranks(), iters=info["iters"])
    c = cases.relief_c2()
    m = oracle.Mesh(c["Ps"], c["Es"], c["leaf"], c["factor"])
    k = oracle.wavenumber(c["freq"])
    y, x, info = oracle.solve_pressures(m, k, c["vec"], 1, c["Ls"], c["aca_tol"], c["aca_tol"], c["tol"],
                                        listener="dense")
    H = oracle.HMat(m, k, c["aca_tol"])
    np.savez_compressed(os.path.join(out, "relief_c2.npz"), Es_tree=m.Es, y_oracle=y,
                        ranks_stored=H.stored_ranks(), iters=info["iters"])


if __name__ == "__main__":
    main()
