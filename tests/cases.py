"""Seeded synthetic cases shared by the tests (shapes and sizes of the reference workloads)."""
import math

import numpy as np

from acoustic_reliefs_gb300 import meshes


def sphere_c1():
    """Icosphere subdivision 3 (1280 triangles), r = 0.5, 500 Hz plane wave along -z,
    181 receivers on a 5 m circle in the xz plane; leaf 32, factor 2, ACA 1e-4, tol 1e-6."""
    Ps, Es = meshes.icosphere(3, 0.5)
    return dict(Ps=Ps, Es=Es, freq=500.0, kind=1, vec=np.array([0.0, 0.0, -1.0]), Ls=meshes.circle_xz(5.0, 181),
                leaf=32, factor=2.0, aca_tol=1e-4, tol=1e-6)


def relief_small(seed=0, nx=30, ny=7, subdiv=0, freq=2000.0):
    """0.6 m relief, 30 x 7 x 30 box (5280 triangles) with a seeded 64 x 64 smoothed heightmap,
    normal plane-wave incidence (-y), 181 receivers on a 5 m semicircle."""
    R = meshes.relief(0.6, 0.6, 0.05, nx, ny, nx, subdiv, meshes.smooth_heightmap(64, seed))
    return dict(Ps=R.Ps, Es=R.Es, relief=R, freq=freq, kind=1, vec=np.array([0.0, -1.0, 0.0]),
                Ls=meshes.semicircle(5.0, 181), leaf=32, factor=2.0, aca_tol=1e-4, tol=1e-6)


def relief_c2(seed=0):
    """The bench workload: 0.6 m relief with a seeded smoothed 64 x 64 heightmap, 20480 triangles,
    2 kHz, normal plane wave (-y), 181 receivers on a 5 m semicircle."""
    R = meshes.relief_20k(seed)
    return dict(Ps=R.Ps, Es=R.Es, relief=R, freq=2000.0, kind=1, vec=np.array([0.0, -1.0, 0.0]),
                Ls=meshes.semicircle(5.0, 181), leaf=32, factor=2.0, aca_tol=1e-4, tol=1e-6)


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))
