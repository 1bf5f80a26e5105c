"""FP64 CPU oracle for the acoustics3d BEM hot path (TEST INFRASTRUCTURE ONLY).

Python front end over ``oracle/_build/liboracle.so`` (built from ``oracle/oracle.cpp`` by
``oracle/Makefile``). Only ``tests/``, the smoke check and the CPU-baseline leg of ``bench.py``
import this package; the product never does.

Parity status: the reference library cannot be compiled (its Eigen submodule is empty), so the
restatement is pinned by the rigid-sphere Mie known answer (``oracle/mie.py``) and by its own
dense-versus-H-matrix cross-check. Agreement with the reference binary itself is unpinned.

``OracleDiffBEM`` mirrors the reference binding ``DiffBEM`` (acoustics3d_cpp/src/acoustics3d.cpp:
22-351) and driver ``bem3d::gradient`` (acoustics3d_cpp/src/adjoint.cpp:24-242).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

SPEED_OF_SOUND = 344.0  # constants.h:13
APPROX_ACA_MAX_K = 100  # constants.h:16
Q_ACA_MAX_K = 5000  # constants.h:17


def build() -> str:
    """Compile the oracle with its Makefile (g++ -O2 -fopenmp, no FP contraction)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
                os.path.join(_HERE, "oracle.cpp")):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        D = ctypes.c_double
        I = ctypes.c_int
        sig = {
            "orc_wavenumber": (D, [D]),
            "orc_num_threads": (I, []),
            "orc_set_threads": (None, [I]),
            "orc_mesh_new": (P, [P, I, P, I, I, D]),
            "orc_mesh_free": (None, [P]),
            "orc_mesh_tree_ok": (I, [P]),
            "orc_mesh_counts": (None, [P, P, P, P]),
            "orc_mesh_get": (None, [P, P, P, P, P]),
            "orc_mesh_nodes": (None, [P, P, P, P, P]),
            "orc_mesh_set_points": (None, [P, P]),
            "orc_mesh_geometry": (None, [P, P, P]),
            "orc_rhs": (None, [P, D, P, I, P]),
            "orc_entries": (None, [P, D, I, P, P, P]),
            "orc_dense_boundary": (None, [P, D, P]),
            "orc_dense_listener": (None, [P, D, P, I, P]),
            "orc_hmat_new": (P, [P, D, D]),
            "orc_hmat_free": (None, [P]),
            "orc_hmat_ranks": (None, [P, P]),
            "orc_hmat_block_factors": (None, [P, I, P, P]),
            "orc_hmat_matvec": (None, [P, P, P, I]),
            "orc_bicgstab": (I, [P, P, P, D, I, I, P]),
            "orc_listener_new": (P, [P, D, P, I, D]),
            "orc_listener_free": (None, [P]),
            "orc_listener_rank": (I, [P]),
            "orc_listener_apply": (None, [P, P, P, I]),
            "orc_compute_u": (D, [I, P, P]),
            "orc_der_A": (None, [P, D, P, I, I, P, P, P, P, P]),
            "orc_der_B": (None, [P, D, I, P, P, P, P, P]),
            "orc_der_C": (None, [P, D, P, I, I, P, P, P, P]),
            "orc_dM_dtarget_y": (None, [D, P, P, P]),
            "orc_dM_dsource_y": (None, [D, P, P, I, P]),
            "orc_entry_pt": (None, [D, P, P, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def wavenumber(freq: float) -> float:
    """freq_to_wavenumber (helpers.h:8): k = 2 pi f / 344."""
    return 2 * math.pi * freq / SPEED_OF_SOUND


def frequencies(freq_band: float, n_freqs: int) -> list[float]:
    """get_frequencies (helpers.cpp:67-83): n log-spaced points over +-1/6 octave."""
    if n_freqs == 1:
        return [float(freq_band)]
    bw = 2.0 ** (1.0 / 6.0)
    lo = math.log(freq_band / bw)
    hi = math.log(freq_band * bw)
    d = (hi - lo) / (n_freqs - 1.0)
    return [math.exp(lo + i * d) for i in range(n_freqs)]


def listener_hemisphere(radius: float, ds: float) -> np.ndarray:
    """compute_listener_pts + spherical_to_cartesian (helpers.cpp:34-65)."""
    el, az = [0.0], [0.0]
    e = ds
    while e < 91:
        a = 0.0
        while a < 360:
            el.append(e)
            az.append(a)
            a += ds
        e += ds
    th = np.array(el) * math.pi / 180.0
    ph = np.array(az) * math.pi / 180.0
    return np.column_stack([radius * np.sin(th) * np.cos(ph), radius * np.cos(th),
                            -radius * np.sin(th) * np.sin(ph)])


def compute_u(yt: np.ndarray) -> tuple[float, np.ndarray]:
    """compute_u (adjoint.cpp:388-397): diffusion coefficient c and dc/dyt."""
    yt = np.ascontiguousarray(yt, dtype=np.float64)
    u = np.zeros_like(yt)
    c = lib().orc_compute_u(len(yt), _p(yt), _p(u))
    return c, u


class Mesh:
    """Tree + block partition (DiffBEM::set_mesh, acoustics3d.cpp:36-67)."""

    def __init__(self, Ps, Es, leaf: int, factor: float):
        self.Ps = np.ascontiguousarray(Ps, dtype=np.float64)
        Es = np.ascontiguousarray(Es, dtype=np.int32)
        self.V = len(self.Ps)
        self.Ne = len(Es)
        self.h = lib().orc_mesh_new(_p(self.Ps), self.V, _p(Es), self.Ne, leaf, factor)
        nd, na, nn = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        lib().orc_mesh_counts(self.h, ctypes.byref(nd), ctypes.byref(na), ctypes.byref(nn))
        self.order = np.zeros(self.Ne, np.int32)
        self.Es = np.zeros((self.Ne, 3), np.int32)
        self.direct = np.zeros((nd.value, 4), np.int32)
        self.approx = np.zeros((na.value, 4), np.int32)
        lib().orc_mesh_get(self.h, _p(self.order), _p(self.Es), _p(self.direct), _p(self.approx))
        self.node_c = np.zeros((nn.value, 3))
        self.node_r = np.zeros(nn.value)
        self.node_range = np.zeros((nn.value, 2), np.int32)
        self.node_child = np.zeros((nn.value, 2), np.int32)
        lib().orc_mesh_nodes(self.h, _p(self.node_c), _p(self.node_r), _p(self.node_range),
                             _p(self.node_child))
        self.tree_ok = bool(lib().orc_mesh_tree_ok(self.h))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_mesh_free(self.h)
            self.h = None

    def set_points(self, Ps):
        self.Ps = np.ascontiguousarray(Ps, dtype=np.float64)
        lib().orc_mesh_set_points(self.h, _p(self.Ps))

    def geometry(self):
        C = np.zeros((self.Ne, 3))
        N = np.zeros((self.Ne, 3))
        lib().orc_mesh_geometry(self.h, _p(C), _p(N))
        return C, N

    def rhs(self, k: float, src, kind: int = 0) -> np.ndarray:
        """Incident field b: point source (kind 0) or plane wave along unit vector src (kind 1)."""
        s = np.ascontiguousarray(src, dtype=np.float64)
        out = np.zeros(self.Ne, np.complex128)
        lib().orc_rhs(self.h, k, _p(s), kind, _p(out))
        return out

    def entries(self, k, rows, cols):
        rows = np.ascontiguousarray(rows, np.int32)
        cols = np.ascontiguousarray(cols, np.int32)
        out = np.zeros(len(rows), np.complex128)
        lib().orc_entries(self.h, k, len(rows), _p(rows), _p(cols), _p(out))
        return out

    def dense_boundary(self, k: float) -> np.ndarray:
        out = np.zeros((self.Ne, self.Ne), np.complex128)
        lib().orc_dense_boundary(self.h, k, _p(out))
        return out

    def dense_listener(self, k: float, Ls) -> np.ndarray:
        Ls = np.ascontiguousarray(Ls, dtype=np.float64)
        out = np.zeros((len(Ls), self.Ne), np.complex128)
        lib().orc_dense_listener(self.h, k, _p(Ls), len(Ls), _p(out))
        return out


class HMat:
    """H-matrix of (K - I/2) at wavenumber k (HMatrix, hmatrix.h:27-139)."""

    def __init__(self, mesh: Mesh, k: float, aca_tol: float):
        self.mesh = mesh
        self.k = k
        self.h = lib().orc_hmat_new(mesh.h, k, aca_tol)
        self.ranks = np.zeros(len(mesh.approx), np.int32)
        lib().orc_hmat_ranks(self.h, _p(self.ranks))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_hmat_free(self.h)
            self.h = None

    def factors(self, b: int):
        rs, re, cs, ce = self.mesh.approx[b]
        m, n, r = re - rs, ce - cs, self.ranks[b]
        U = np.zeros(m * r, np.complex128)
        V = np.zeros(r * n, np.complex128)
        lib().orc_hmat_block_factors(self.h, b, _p(U), _p(V))
        return U.reshape(r, m).T, V.reshape(r, n)

    def stored_ranks(self) -> np.ndarray:
        """Per block, the ACA terms with u != 0 and v != 0. The reference keeps exactly-zero terms
        (they come from coplanar panels, aca.cpp:56-60) in its rank count; they add nothing to any
        product, and the GPU path does not store them."""
        out = np.zeros(len(self.ranks), np.int32)
        for b in range(len(self.ranks)):
            if self.ranks[b] == 0:
                continue
            U, V = self.factors(b)
            out[b] = int(np.sum(np.any(U != 0, axis=0) & np.any(V != 0, axis=1)))
        return out

    def matvec(self, x, transposed=False) -> np.ndarray:
        x = _c(x)
        y = np.zeros_like(x)
        lib().orc_hmat_matvec(self.h, _p(x), _p(y), int(transposed))
        return y

    def solve(self, b, tol: float, maxit: int | None = None, transposed=False):
        b = _c(b)
        x = np.zeros_like(b)
        err = ctypes.c_double()
        it = lib().orc_bicgstab(self.h, _p(b), _p(x), tol, maxit or 2 * len(b), int(transposed),
                                ctypes.byref(err))
        return x, it, err.value


class ListenerACA:
    """Listener matrix Q ~ U V by ACA (compute_ACA_listener, aca.cpp:84-134)."""

    def __init__(self, mesh: Mesh, k: float, Ls, tol: float):
        Ls = np.ascontiguousarray(Ls, dtype=np.float64)
        self.L = len(Ls)
        self.Ne = mesh.Ne
        self.h = lib().orc_listener_new(mesh.h, k, _p(Ls), self.L, tol)
        self.rank = lib().orc_listener_rank(self.h)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_listener_free(self.h)
            self.h = None

    def apply(self, x):
        x = _c(x)
        y = np.zeros(self.L, np.complex128)
        lib().orc_listener_apply(self.h, _p(x), _p(y), 0)
        return y

    def apply_t(self, v):
        v = _c(v)
        y = np.zeros(self.Ne, np.complex128)
        lib().orc_listener_apply(self.h, _p(v), _p(y), 1)
        return y


def mesh_dense_listener_apply(mesh: Mesh, k: float, Ls, x) -> np.ndarray:
    """y = Q x with the exact receiver matrix (compute_listener_matrix, integrate.cpp:46-57)."""
    return mesh.dense_listener(k, Ls) @ np.asarray(x)


def incidence(Es: np.ndarray, diff_pts) -> tuple[dict, np.ndarray, np.ndarray]:
    """set_diff_points (acoustics3d.cpp:69-101) as CSR (offsets, (element, corner) pairs)."""
    Hs = {}
    for i in diff_pts:
        Hs[int(i)] = len(Hs)
    lists = [[] for _ in range(len(Hs))]
    for j in range(len(Es)):
        for o in range(3):
            h = Hs.get(int(Es[j, o]))
            if h is not None:
                lists[h].append((j, o))
    off = np.zeros(len(Hs) + 1, np.int32)
    for h, l in enumerate(lists):
        off[h + 1] = off[h] + len(l)
    pairs = np.array([p for l in lists for p in l], np.int32).reshape(-1, 2)
    return Hs, off, np.ascontiguousarray(pairs)


def der_A(mesh, k, Ls, off, pairs, vf, x):
    Ls = np.ascontiguousarray(Ls, dtype=np.float64)
    out = np.zeros(len(off) - 1)
    vf, x = _c(vf), _c(x)
    lib().orc_der_A(mesh.h, k, _p(Ls), len(Ls), len(off) - 1, _p(off), _p(pairs), _p(vf), _p(x), _p(out))
    return out


def der_B(mesh, k, off, pairs, lmb, x):
    out = np.zeros(len(off) - 1)
    lmb, x = _c(lmb), _c(x)
    lib().orc_der_B(mesh.h, k, len(off) - 1, _p(off), _p(pairs), _p(lmb), _p(x), _p(out))
    return out


def der_C(mesh, k, src, kind, off, pairs, lmb):
    s = np.ascontiguousarray(src, dtype=np.float64)
    out = np.zeros(len(off) - 1)
    lmb = _c(lmb)
    lib().orc_der_C(mesh.h, k, _p(s), kind, len(off) - 1, _p(off), _p(pairs), _p(lmb), _p(out))
    return out


def entry_pt(k, p, tri):
    p = np.ascontiguousarray(p, np.float64)
    q = np.ascontiguousarray(tri, np.float64).reshape(9)
    out = np.zeros(2)
    lib().orc_entry_pt(k, _p(p), _p(q), _p(out))
    return complex(out[0], out[1])


def dM_dtarget_y(k, p, tri):
    p = np.ascontiguousarray(p, np.float64)
    q = np.ascontiguousarray(tri, np.float64).reshape(9)
    out = np.zeros(2)
    lib().orc_dM_dtarget_y(k, _p(p), _p(q), _p(out))
    return complex(out[0], out[1])


def dM_dsource_y(k, p, tri, o):
    p = np.ascontiguousarray(p, np.float64)
    q = np.ascontiguousarray(tri, np.float64).reshape(9)
    out = np.zeros(2)
    lib().orc_dM_dsource_y(k, _p(p), _p(q), o, _p(out))
    return complex(out[0], out[1])


def solve_pressures(mesh: Mesh, k: float, src, kind: int, Ls, aca_tol: float, q_tol: float,
                    solver_tol: float, listener: str = "aca", maxit: int | None = None):
    """One forward solve (DiffBEM::pvals, acoustics3d.cpp:240-280): assemble, BiCGSTAB on -b,
    listener product. Returns (y, x, info)."""
    H = HMat(mesh, k, aca_tol)
    b = mesh.rhs(k, src, kind)
    x, it, err = H.solve(-b, solver_tol, maxit)
    if listener == "aca":
        Q = ListenerACA(mesh, k, Ls, q_tol)
        y = Q.apply(x)
        qrank = Q.rank
    else:
        y = mesh.dense_listener(k, Ls) @ x
        qrank = -1
    return y, x, {"iters": it, "err": err, "ranks": H.ranks, "qrank": qrank}


class OracleDiffBEM:
    """FP64 restatement of the reference ``DiffBEM`` (acoustics3d.cpp:22-351)."""

    def __init__(self, cluster_size=64, radius_factor=1.5, freq_bands=(1000,), n_freqs=1,
                 approx_ACA_tol=1e-3, Q_ACA_tol=1e-3, solver_tol=1e-3, src_pt=(0, 100, 0),
                 listener_radius=50, listener_ds=5, recompute_matrices=False):
        self.cluster_size = int(cluster_size)
        self.radius_factor = float(radius_factor)
        self.freq_bands = [float(f) for f in freq_bands]
        self.n_freqs = int(n_freqs)
        self.aca_tol = float(approx_ACA_tol)
        self.q_tol = float(Q_ACA_tol)
        self.solver_tol = float(solver_tol)
        self.src = np.asarray(src_pt, dtype=np.float64).reshape(3)
        self.src_kind = 0
        self.Ls = listener_hemisphere(listener_radius, listener_ds)
        self.recompute = bool(recompute_matrices)
        self.use_actual = False
        self.silent = True
        self.mesh = None
        self.Hs = {}
        self.off = np.zeros(1, np.int32)
        self.pairs = np.zeros((0, 2), np.int32)

    def set_mesh(self, Ps, Es):
        self.mesh = Mesh(Ps, Es, self.cluster_size, self.radius_factor)
        self.Ps0 = self.mesh.Ps.copy()
        return self.Ps0.copy(), self.mesh.Es.astype(np.int64)

    def set_diff_points(self, diff_pts):
        self.Hs, self.off, self.pairs = incidence(self.mesh.Es, diff_pts)

    def precompute(self, Ps, Es, diff_pts):
        out = self.set_mesh(Ps, Es)
        self.set_diff_points(diff_pts)
        return out

    def _points(self, x):
        Ps = self.Ps0.copy()
        if x is not None:
            for v, h in self.Hs.items():
                Ps[v, 1] = x[h] + self.Ps0[v, 1]
        return Ps

    def _band(self, freq_band, forward_only, x=None):
        """bem3d::gradient (adjoint.cpp:24-242) for one band."""
        self.mesh.set_points(self._points(x))
        Ls = self.Ls
        LL = len(Ls)
        HH = len(self.off) - 1
        freqs = frequencies(freq_band, self.n_freqs)
        yt = np.zeros(LL)
        xs, ys, saved = [], [], []
        for f in freqs:
            k = wavenumber(f)
            b = self.mesh.rhs(k, self.src, self.src_kind)
            if self.use_actual:
                M = self.mesh.dense_boundary(k)
                xv = np.linalg.solve(M, -b)
                Q = self.mesh.dense_listener(k, Ls)
                y = Q @ xv
                saved.append((M, Q))
            else:
                H = HMat(self.mesh, k, self.aca_tol)
                xv, _, _ = H.solve(-b, self.solver_tol)
                Q = ListenerACA(self.mesh, k, Ls, self.q_tol)
                y = Q.apply(xv)
                saved.append((H, Q))
            yt += np.abs(y)
            xs.append(xv)
            ys.append(y)
        c, u = compute_u(yt)
        if forward_only:
            return c, None
        dcdh = np.zeros(HH)
        for ff, f in enumerate(freqs):
            k = wavenumber(f)
            xv, y = xs[ff], ys[ff]
            vf = u * np.conj(y) / np.abs(y)
            A, Q = saved[ff]
            if self.use_actual:
                adj_b = Q.T @ vf
                lmb = np.linalg.solve(A.T, adj_b)
            else:
                adj_b = Q.apply_t(vf)
                lmb, _, _ = A.solve(adj_b, self.solver_tol, transposed=True)
            dA = der_A(self.mesh, k, Ls, self.off, self.pairs, vf, xv)
            dB = der_B(self.mesh, k, self.off, self.pairs, lmb, xv)
            dC = der_C(self.mesh, k, self.src, self.src_kind, self.off, self.pairs, lmb)
            dcdh += dA - dB + dC
        return c, dcdh

    def value(self, x=None):
        return sum(self._band(fb, True, x)[0] for fb in self.freq_bands) / len(self.freq_bands)

    def band_value(self, freq_band):
        return self._band(freq_band, True)[0]

    def values(self):
        return [self._band(fb, True)[0] for fb in self.freq_bands]

    def gradient(self, x):
        c = 0.0
        g = np.zeros(len(self.off) - 1)
        for fb in self.freq_bands:
            cb, gb = self._band(fb, False, x)
            c += cb
            g += gb
        return c, g

    def pvals(self, frequency, listeners=None):
        Ls = self.Ls if listeners is None else np.asarray(listeners, np.float64)
        self.mesh.set_points(self.Ps0)
        y, _, _ = solve_pressures(self.mesh, wavenumber(frequency), self.src, self.src_kind, Ls,
                                  self.aca_tol, self.q_tol, self.solver_tol)
        return y

    def surface_vals(self, frequency):
        self.mesh.set_points(self.Ps0)
        k = wavenumber(frequency)
        H = HMat(self.mesh, k, self.aca_tol)
        x, _, _ = H.solve(-self.mesh.rhs(k, self.src, self.src_kind), self.solver_tol)
        return x

    def get_listeners(self):
        return self.Ls.copy()

    def set_band(self, freq_band):
        self.freq_bands = [float(freq_band)]
