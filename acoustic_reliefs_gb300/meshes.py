"""Synthetic inputs for the BEM path: relief boxes, icospheres, heightmaps, receivers, OBJ I/O.

The relief generator restates the reference mesher (pyoptim/mesher.py:87-231: six unwelded
structured face grids, top face ``y = h``; optional 1->4 subdivision of the top triangles) and the
heightmap sampling of the optimiser (acoustics_opt.py:24-34 ``eval_uv``; pyoptim/diffmesh.py:248
``rect_points_to_uv``). gmsh is not needed.
"""
from __future__ import annotations

import math

import numpy as np


def box_grid(w: float, h: float, b: float, nx: int, ny: int, nz: int):
    """Structured box of triangles (generate_base_mesh, pyoptim/mesher.py:87-149).

    Each face is its own (nu+1) x (nv+1) vertex grid (faces do not share vertices); quads are
    split into two triangles. Returns (Ps (V,3) float64, Es (F,3) int64)."""
    verts: list[np.ndarray] = []
    faces: list[np.ndarray] = []
    nbase = 0

    def grid(start, u, v, nu, nv, sign):
        nonlocal nbase
        jj, ii = np.meshgrid(np.arange(nv + 1), np.arange(nu + 1), indexing="ij")
        pts = (np.asarray(start)[None, :] + ii.reshape(-1, 1) * np.asarray(u)[None, :]
               + jj.reshape(-1, 1) * np.asarray(v)[None, :])
        verts.append(pts)
        j, i = np.meshgrid(np.arange(nv), np.arange(nu), indexing="ij")
        a = (nbase + j * (nu + 1) + i).reshape(-1)
        bq, c = a + 1, a + (nu + 1)
        d = c + 1
        if sign > 0:
            tri = np.stack([np.stack([a, c, d], 1), np.stack([a, d, bq], 1)], 1)
        else:
            tri = np.stack([np.stack([a, d, c], 1), np.stack([a, bq, d], 1)], 1)
        faces.append(tri.reshape(-1, 3))
        nbase += (nu + 1) * (nv + 1)

    dx, dy, dz = w / nx, h / ny, b / nz
    grid((-w / 2, 0, -b / 2), (dx, 0, 0), (0, dy, 0), nx, ny, 1)
    grid((-w / 2, 0, b / 2), (dx, 0, 0), (0, dy, 0), nx, ny, -1)
    grid((-w / 2, h, -b / 2), (dx, 0, 0), (0, 0, dz), nx, nz, 1)
    grid((-w / 2, 0, -b / 2), (dx, 0, 0), (0, 0, dz), nx, nz, -1)
    grid((-w / 2, 0, -b / 2), (0, dy, 0), (0, 0, dz), ny, nz, 1)
    grid((w / 2, 0, -b / 2), (0, dy, 0), (0, 0, dz), ny, nz, -1)
    return np.concatenate(verts).astype(np.float64), np.concatenate(faces).astype(np.int64)


def subdivide(Ps, Es, faces, n_subdivisions: int = 1):
    """Midpoint 1->4 subdivision of the listed triangles (face_subdivision,
    pyoptim/mesher.py:153-231); neighbours that share a split edge are re-triangulated.
    Returns (Ps, Es, faces) with `faces` the indices of the subdivided children."""
    Ps = np.asarray(Ps, np.float64).copy()
    Es = np.asarray(Es, np.int64).copy()
    faces = list(faces)
    for _ in range(n_subdivisions):
        mid: dict[tuple[int, int], int] = {}
        for i1, i2, i3 in Es[faces]:
            for e in ((min(i1, i2), max(i1, i2)), (min(i2, i3), max(i2, i3)), (min(i1, i3), max(i1, i3))):
                mid.setdefault((int(e[0]), int(e[1])), -1)
        new = []
        for e in mid:
            mid[e] = len(Ps) + len(new)
            new.append((Ps[e[0]] + Ps[e[1]]) / 2)
        nP = np.vstack([Ps, np.array(new).reshape(-1, 3)])
        sub = np.zeros(len(Es), bool)
        sub[faces] = True
        nE: list[list[int]] = []
        nfaces: list[int] = []
        for s, (i1, i2, i3) in zip(sub, Es):
            i1, i2, i3 = int(i1), int(i2), int(i3)
            i4 = mid.get((min(i1, i2), max(i1, i2)), -1)
            i5 = mid.get((min(i2, i3), max(i2, i3)), -1)
            i6 = mid.get((min(i1, i3), max(i1, i3)), -1)
            if s:
                nfaces.extend(range(len(nE), len(nE) + 4))
            if i4 >= 0 and i5 < 0 and i6 < 0:
                nE += [[i4, i2, i3], [i1, i4, i3]]
            elif i5 >= 0 and i4 < 0 and i6 < 0:
                nE += [[i1, i2, i5], [i1, i5, i3]]
            elif i6 >= 0 and i4 < 0 and i5 < 0:
                nE += [[i1, i2, i6], [i2, i3, i6]]
            elif i4 < 0 and i5 >= 0 and i6 >= 0:
                nE += [[i1, i2, i6], [i2, i5, i6], [i5, i3, i6]]
            elif i5 < 0 and i4 >= 0 and i6 >= 0:
                nE += [[i1, i4, i6], [i2, i6, i4], [i2, i3, i6]]
            elif i6 < 0 and i4 >= 0 and i5 >= 0:
                nE += [[i1, i4, i3], [i3, i4, i5], [i4, i2, i5]]
            elif i4 >= 0 and i5 >= 0 and i6 >= 0:
                nE += [[i1, i4, i6], [i4, i2, i5], [i6, i5, i3], [i4, i5, i6]]
            else:
                nE += [[i1, i2, i3]]
        Ps, Es, faces = nP, np.array(nE, np.int64), nfaces
    return Ps, Es, faces


def rect_uv(points, x_min, x_max, z_min, z_max, uvmin=0.0001, uvmax=0.9999):
    """Top-face (x, z) -> texture uv (pyoptim/diffmesh.py:248-249)."""
    return np.column_stack([(points[:, 0] - x_min) / (x_max - x_min) * (uvmax - uvmin) + uvmin,
                            (points[:, 2] - z_min) / (z_max - z_min) * (uvmax - uvmin) + uvmin])


def bilinear_weights(shape, uvs):
    """Texel indices and weights of the bilinear lookup in ``eval_uv`` (acoustics_opt.py:24-34).
    Returns (rows (n,4), cols (n,4), weights (n,4))."""
    h, w = shape
    uf, ui = np.modf(uvs[:, 0] * w - 0.5)
    vf, vi = np.modf(uvs[:, 1] * h - 0.5)
    uf = np.where(uf < 0, 1 + uf, uf)
    vf = np.where(vf < 0, 1 + vf, vf)
    ui = np.maximum(ui.astype(int), 0)
    vi = np.maximum(vi.astype(int), 0)
    u1 = np.minimum(ui + 1, w - 1)
    v1 = np.minimum(vi + 1, h - 1)
    rows = np.stack([vi, vi, v1, v1], 1)
    cols = np.stack([ui, u1, ui, u1], 1)
    wts = np.stack([(1 - vf) * (1 - uf), (1 - vf) * uf, vf * (1 - uf), vf * uf], 1)
    return rows, cols, wts


def sample_heightmap(tex, uvs):
    """Bilinear heightmap lookup at uv points (eval_uv, acoustics_opt.py:24-34)."""
    rows, cols, wts = bilinear_weights(tex.shape, uvs)
    return np.sum(np.asarray(tex)[rows, cols] * wts, axis=1)


def scatter_to_heightmap(shape, uvs, grad):
    """Transpose of ``sample_heightmap`` (acoustics_opt.py:44-57): per-vertex gradient -> texels."""
    rows, cols, wts = bilinear_weights(shape, uvs)
    out = np.zeros(shape)
    np.add.at(out, (rows.reshape(-1), cols.reshape(-1)), (wts * np.asarray(grad)[:, None]).reshape(-1))
    return out


def smooth_heightmap(res: int, seed: int, amp: float = 0.1, sigma: float = 2.0) -> np.ndarray:
    """Seeded uniform [0, amp] heightmap smoothed by a Gaussian of `sigma` cells."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    return gaussian_filter(rng.uniform(0.0, amp, size=(res, res)), sigma=sigma)


class Relief:
    """A relief: box mesh, top-face ("differentiable") vertex ids and their texture uvs."""

    def __init__(self, Ps, Es, diff_pts, uvs):
        self.Ps, self.Es, self.diff_pts, self.uvs = Ps, Es, diff_pts, uvs

    @property
    def num_triangles(self) -> int:
        return len(self.Es)


def relief(w: float = 0.6, b: float = 0.6, h: float = 0.05, nx: int = 64, ny: int = 8, nz: int = 64,
           subdiv_top: int = 0, heightmap=None) -> Relief:
    """Relief box with optional heightmap displacement of the top face (y = h).

    Follows the optimiser's set-up (acoustics_opt.py:182-210): base grid, top vertices found by
    ``isclose(y, max y)``, optional top-face subdivision, uvs over the top face, heights added in y.
    Triangle count: 4 nx ny + 4 ny nz + 2 nx nz (1 + 4^subdiv_top)."""
    Ps, Es = box_grid(w, h, b, nx, ny, nz)
    top = np.where(np.isclose(Ps[:, 1], np.max(Ps[:, 1])))[0]
    if subdiv_top > 0:
        top_faces = np.where(np.all(np.isin(Es, top), axis=1))[0]
        Ps, Es, _ = subdivide(Ps, Es, top_faces, subdiv_top)
        top = np.where(np.isclose(Ps[:, 1], np.max(Ps[:, 1])))[0]
    mx, mn = Ps.max(0), Ps.min(0)
    uvs = rect_uv(Ps[top], mn[0], mx[0], mn[2], mx[2])
    if heightmap is not None:
        Ps = Ps.copy()
        Ps[top, 1] += sample_heightmap(heightmap, uvs)
    return Relief(Ps, Es, top, uvs)


def relief_device(w: float = 0.6, b: float = 0.6, h: float = 0.05, nx: int = 64, ny: int = 8, nz: int = 64,
                  subdiv_top: int = 0, device=None):
    """The base box, top-face subdivision and top uvs of ``relief`` generated by CUDA kernels
    (``ac3d_relief_dev``) into torch device tensors: (Ps (V,3) float64, Es (F,3) int32, top ids,
    uvs (n_top,2) float64), bitwise the host generator's. Heights are then the texture lookup at
    the uvs (``autograd.TexMap``)."""
    import ctypes

    import torch

    from . import _lib as _L
    L = _L.lib()
    V, F = ctypes.c_int(), ctypes.c_int()
    rc = L.ac3d_relief_sizes(int(nx), int(ny), int(nz), int(subdiv_top), ctypes.byref(V), ctypes.byref(F))
    if rc != _L.OK:
        raise _L.AC3DError(rc, "invalid relief parameters")
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    Ps = torch.empty((V.value, 3), dtype=torch.float64, device=dev)
    Es = torch.empty((F.value, 3), dtype=torch.int32, device=dev)
    top = torch.empty(V.value, dtype=torch.int32, device=dev)
    uvs = torch.empty((V.value, 2), dtype=torch.float64, device=dev)
    nt = ctypes.c_int()
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = L.ac3d_relief_dev(float(w), float(b), float(h), int(nx), int(ny), int(nz), int(subdiv_top),
                           ctypes.c_void_p(Ps.data_ptr()), ctypes.c_void_p(Es.data_ptr()),
                           ctypes.c_void_p(top.data_ptr()), ctypes.c_void_p(uvs.data_ptr()), ctypes.byref(nt),
                           ctypes.c_void_p(stream))
    if rc != _L.OK:
        raise _L.AC3DError(rc, "relief generation failed")
    return Ps, Es, top[:nt.value], uvs[:nt.value]


def icosphere(subdivisions: int = 3, radius: float = 1.0):
    """Geodesic sphere: icosahedron with `subdivisions` midpoint refinements (20 * 4^s
    triangles), vertices projected to the sphere, triangles wound outward."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
         (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    P = [np.array(v, float) / np.linalg.norm(v) for v in V]
    for _ in range(subdivisions):
        cache: dict[tuple[int, int], int] = {}

        def mid(i, j):
            key = (min(i, j), max(i, j))
            if key not in cache:
                m = P[i] + P[j]
                P.append(m / np.linalg.norm(m))
                cache[key] = len(P) - 1
            return cache[key]

        nF = []
        for a, b_, c in F:
            ab, bc, ca = mid(a, b_), mid(b_, c), mid(c, a)
            nF += [(a, ab, ca), (b_, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nF
    Ps = np.array(P) * radius
    Es = np.array(F, np.int64)
    # orient outward: (b - a) x (c - a) along the centroid direction
    a, b_, c = Ps[Es[:, 0]], Ps[Es[:, 1]], Ps[Es[:, 2]]
    flip = np.einsum("ij,ij->i", np.cross(b_ - a, c - a), a + b_ + c) < 0
    Es[flip] = Es[flip][:, [0, 2, 1]]
    return Ps, Es


def semicircle(radius: float = 5.0, n: int = 181, plane: str = "xy") -> np.ndarray:
    """n receivers on a half circle, angles 0..pi (misc/pressure_calcs.py:47-49 uses xy)."""
    th = np.linspace(0.0, math.pi, n)
    z = np.zeros_like(th)
    if plane == "xy":
        return np.column_stack([np.cos(th) * radius, np.sin(th) * radius, z])
    return np.column_stack([np.cos(th) * radius, z, np.sin(th) * radius])


def circle_xz(radius: float = 5.0, n: int = 181) -> np.ndarray:
    """n receivers on a full circle in the xz plane, angle 2 pi l / n (sphere.h:58-63)."""
    th = np.arange(n) / n * 2 * math.pi
    return np.column_stack([radius * np.cos(th), np.zeros(n), -radius * np.sin(th)])


def read_obj(path: str):
    """Triangle OBJ reader (read_obj.cpp:8-50), reading only ``v `` and ``f `` records (so
    ``vn``/``vt`` lines are skipped) and the vertex index of ``f a/b/c`` forms."""
    verts, faces = [], []
    with open(path) as f:
        for line in f:
            if line.startswith("v "):
                verts.append([float(t) for t in line.split()[1:4]])
            elif line.startswith("f "):
                idx = [int(t.split("/")[0]) - 1 for t in line.split()[1:]]
                if len(idx) != 3:
                    raise ValueError("only triangle faces are supported")
                faces.append(idx)
    return np.array(verts, np.float64), np.array(faces, np.int64)


def write_obj(path: str, Ps, Es) -> None:
    """write_obj (read_obj.cpp:52-63): full-precision vertices, 1-based faces."""
    with open(path, "w") as f:
        for p in np.asarray(Ps):
            f.write("v %.17g %.17g %.17g\n" % tuple(p))
        for e in np.asarray(Es):
            f.write("f %d %d %d\n" % tuple(int(i) + 1 for i in e))


def relief_20k(seed: int = 0) -> Relief:
    """The 0.6 m relief workload: 0.6 x 0.6 x 0.05 m box, top face a 64 x 64 grid displaced by a
    seeded 64 x 64 uniform [0, 0.1] m heightmap smoothed with sigma = 2 cells; 20480 triangles."""
    return relief(0.6, 0.6, 0.05, 64, 8, 64, 0, smooth_heightmap(64, seed))
