"""Writes tests/golden/ref_*.npz from the reference project's own mesh fixtures (run from the
repository root, where the reference checkout is readable; the GPU tests only read the .npz).

Meshes are parsed as the reference reader does (read_obj.cpp:8-65: "v x y z" records, triangle
"f a b c" records with 1-based indices) and stored as float64 / int32 arrays.

ref_spheres.npz -- test-data/spheres/sphere_s.obj (1984 triangles) and sphere_m.obj (8064), the
  reference's known-answer case (misc/analytic_sphere.py:32-60 calling sphere(), sphere.h:28-85):
  plane wave e^{-ikx}, 360 receivers on a 10 m circle in the xz plane, leaf 128, factor 1.5,
  ACA / receiver ACA / BiCGSTAB tolerances 1e-10; 2 kHz as the reference runs it, and 500 Hz and
  1 kHz on sphere_s (the reference's commented-out setting), where the discretisation error
  against the analytic series is small. Stored per case: the FP64 oracle's pressures and the Mie
  series at the same receivers with c = 344 (the C++ constant, constants.h:13) and c = 343 (the
  Python check's constant, analytic_sphere.py:11).
ref_relief_cat.npz -- submission/acoustic_reliefs/0.6/cat_0.6.obj (38686 triangles), a relief the
  reference pipeline produced, under the reference's own product call (acoustics_pipeline.py:11-17):
  DiffBEM(128, 1.5, [band], 3, 1e-5, 1e-5, 1e-5, src (0, 100, 0), 50, 5) -- point source, receiver
  ACA, the 1297-point hemisphere. Stored: the oracle's band_value(1000) (three frequencies of the
  1 kHz third-octave band) and pvals(1000) at the hemisphere, with the tree-ordered connectivity;
  and pvals(1000) with the solver tolerance 1e-10 (same ACA tolerances), the reference's answer
  without its solver's stopping error.
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import mie  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"


def read_obj(path):
    V, F = [], []
    with open(path) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "v":
                V.append([float(x) for x in t[1:4]])
            elif t[0] == "f":
                F.append([int(x.split("/")[0]) - 1 for x in t[1:4]])
    return np.array(V, np.float64), np.array(F, np.int32)


def sphere_case(Ps, Es, freq=2000.0, LL=360, lrad=10.0, tol=1e-10):
    th = np.arange(LL) / LL * 2 * np.pi
    Ls = np.stack([lrad * np.cos(th), np.zeros(LL), -lrad * np.sin(th)], 1)
    m = oracle.Mesh(Ps, Es, 128, 1.5)
    k = oracle.wavenumber(freq)
    y, _, info = oracle.solve_pressures(m, k, np.array([1.0, 0.0, 0.0]), 1, Ls, tol, tol, tol, listener="aca")
    mie344 = mie.scattered_pressure(lrad, th, 2 * np.pi * freq / 344.0, 1.0)
    mie343 = mie.scattered_pressure(lrad, th, 2 * np.pi * freq / 343.0, 1.0)
    return dict(Es_tree=m.Es, y_oracle=y, mie344=mie344, mie343=mie343, iters=info["iters"])


def main():
    out = os.path.dirname(os.path.abspath(__file__))
    spheres = {}
    for name, freqs in (("sphere_s", (500, 1000, 2000)), ("sphere_m", (2000,))):
        Ps, Es = read_obj(os.path.join(REF, "test-data", "spheres", name + ".obj"))
        spheres[name + "_Ps"] = Ps
        spheres[name + "_Es"] = Es
        for f in freqs:
            t = time.time()
            r = sphere_case(Ps, Es, float(f))
            print(f"{name} {f} Hz: {len(Es)} triangles, oracle {time.time() - t:.1f} s, {r['iters']} iterations",
                  flush=True)
            for k, v in r.items():
                spheres[f"{name}_{f}_{k}"] = v
    np.savez_compressed(os.path.join(out, "ref_spheres.npz"), **spheres)
    if "spheres" in sys.argv[2:]:
        return

    Ps, Es = read_obj(os.path.join(REF, "submission", "acoustic_reliefs", "0.6", "cat_0.6.obj"))
    t = time.time()
    bem = oracle.OracleDiffBEM(128, 1.5, [1000.0], 3, 1e-5, 1e-5, 1e-5, (0.0, 100.0, 0.0), 50, 5)
    _, Es_tree = bem.set_mesh(Ps, Es)
    c = bem.band_value(1000.0)
    y = bem.pvals(1000.0)
    print(f"cat_0.6: {len(Es)} triangles, coefficient {c:.6f}, oracle {time.time() - t:.1f} s", flush=True)
    tight = oracle.OracleDiffBEM(128, 1.5, [1000.0], 3, 1e-5, 1e-5, 1e-10, (0.0, 100.0, 0.0), 50, 5)
    tight.set_mesh(Ps, Es)
    y_tight = tight.pvals(1000.0)
    np.savez_compressed(os.path.join(out, "ref_relief_cat.npz"), Ps=Ps, Es=Es, Es_tree=Es_tree, coef_1000=c,
                        y_1000=y, y_1000_tol1e10=y_tight, Ls=bem.get_listeners())


if __name__ == "__main__":
    main()
