"""Drop-in replacement of the reference Python module ``acoustics3d`` (``DiffBEM`` and ``sphere``).

Same constructor signature and defaults (acoustics3d_cpp/src/acoustics3d.cpp:355-357), same
method names, argument meaning and return types (acoustics3d.cpp:358-382). Where the reference
printed to stderr and returned a sentinel, these raise ``AC3DError``. Keyword-only extensions:
``precision`` ("mixed" = complex FP32 H-matrix with FP64 refinement, "fp64"), ``incident``
(``("point", xyz)`` default at ``src_pt``, or ``("plane", direction)``).

The work runs on the GPU through ``libac3d.so`` (include/ac3d.h); there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib as _L
from ._lib import AC3DError

__all__ = ["DiffBEM", "sphere", "read_obj", "write_obj", "AC3DError"]

_PREC = {"mixed": _L.PREC_MIXED, "fp32": _L.PREC_MIXED, "fp64": _L.PREC_FP64}
_KRYLOV = {"bicgstab": 0, "gmres": 1}


def _f64(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def _cplx(buf: np.ndarray) -> np.ndarray:
    return buf.view(np.complex128).copy()


class DiffBEM:
    """GPU BEM value / gradient of the diffusion coefficient of a mesh (reference ``DiffBEM``)."""

    def __init__(self, cluster_size=64, radius_factor=1.5, freq_bands=(1000,), n_freqs=1, approx_ACA_tol=1e-3,
                 Q_ACA_tol=1e-3, solver_tol=1e-3, src_pt=(0.0, 100.0, 0.0), listener_radius=50, listener_ds=5,
                 recompute_matrices=False, *, precision: str = "mixed", incident=None, listener: str = "dense",
                 device: int | None = None):
        L = _L.lib()
        if device is not None:
            rc = L.ac3d_select_device(int(device))
            if rc != _L.OK:
                raise AC3DError(rc, f"cannot select CUDA device {device}")
        bands = _f64(list(freq_bands))
        src = _f64(src_pt, (3,))
        h = ctypes.c_void_p()
        rc = L.ac3d_create(ctypes.byref(h), int(cluster_size), float(radius_factor), _L.ptr(bands), len(bands),
                           int(n_freqs), float(approx_ACA_tol), float(Q_ACA_tol), float(solver_tol), _L.ptr(src),
                           float(listener_radius), float(listener_ds), int(bool(recompute_matrices)))
        if rc != _L.OK:
            raise AC3DError(rc, "invalid DiffBEM parameters or no CUDA device")
        self._h = h
        self._bands = list(bands)
        self.silent = False
        self._use_actual = False
        self._Hs: dict[int, int] = {}
        self._Ps = None
        self._Es = None
        self._diff_set = False
        self.set_precision(precision)
        self.set_listener_mode(listener)
        if incident is not None:
            self.set_incident(*incident)

    # -- lifecycle ----------------------------------------------------------------------------
    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _L.lib().ac3d_destroy(h)
            except Exception:
                pass
            self._h = None

    def _check(self, rc):
        _L.check(self._h, rc)

    @property
    def use_actual(self) -> bool:
        """acoustics3d.h:49: coefficient and gradient calls on the exact (all-dense, FP64) operator."""
        return self._use_actual

    @use_actual.setter
    def use_actual(self, on) -> None:
        self._check(_L.lib().ac3d_set_actual(self._h, int(bool(on))))
        self._use_actual = bool(on)

    # -- extensions -----------------------------------------------------------------------------
    def set_precision(self, precision: str) -> None:
        self._check(_L.lib().ac3d_set_precision(self._h, _PREC[precision]))
        self.precision = precision

    def set_assembly(self, mode: str = "df") -> None:
        """Arithmetic of the mixed-precision assembly: "df" (default) evaluates the near field, the
        admissible blocks' rows and columns and runs ACA in double-float arithmetic, so the low-rank
        blocks have the FP64 path's pivots and ranks and every stored entry differs from the FP64
        path's only by its FP32 rounding; "fp32" evaluates in FP32."""
        self._check(_L.lib().ac3d_set_assembly(self._h, {"df": _L.ASSEMBLY_DF, "fp32": _L.ASSEMBLY_FP32}[mode]))
        self.assembly = mode

    def set_tensor_cores(self, on: bool = True) -> None:
        """Block matvecs (pvals_multi, gradient_multi) form their dot pass on the tensor cores
        (default) or on the FP32 CUDA cores."""
        self._check(_L.lib().ac3d_set_tensor_cores(self._h, int(bool(on))))

    def set_listener_mode(self, mode: str) -> None:
        """"dense": receiver matrix evaluated exactly on the fly (default); "aca": partially pivoted
        ACA with Q_ACA_tol, as the reference (aca.cpp:84-134)."""
        m = {"dense": _L.LISTENER_DENSE, "aca": _L.LISTENER_ACA}[mode]
        self._check(_L.lib().ac3d_set_listener_mode(self._h, m))
        self.listener = mode

    def set_incident(self, kind: str, vec) -> None:
        k = {"point": _L.INCIDENT_POINT, "plane": _L.INCIDENT_PLANE}[kind]
        self._check(_L.lib().ac3d_set_incident(self._h, k, _L.ptr(_f64(vec, (3,)))))

    def set_solver(self, max_iterations: int = 0, inner_tol: float = 1e-6, max_outer: int = 10) -> None:
        self._check(_L.lib().ac3d_set_solver(self._h, int(max_iterations), float(inner_tol), int(max_outer)))

    def set_krylov(self, method: str = "gmres", restart: int = 300) -> None:
        """Krylov method of the single right-hand-side solves: "bicgstab" (the reference's solver,
        the default) or "gmres" (one matvec per iteration; cycles of at most `restart` iterations
        inside the refinement loop, which checks the same relative residual)."""
        self._check(_L.lib().ac3d_set_krylov(self._h, _KRYLOV[method], int(restart)))

    def set_listeners(self, listeners) -> None:
        Ls = _f64(listeners).reshape(-1, 3)
        self._check(_L.lib().ac3d_set_listeners(self._h, _L.ptr(Ls), len(Ls)))

    def matvec_timing(self, iters: int = 50, transposed: bool = False):
        """(ms per H-matvec, algorithmic bytes per matvec) on the H-matrix of the last solve."""
        ms = ctypes.c_double()
        nb = ctypes.c_longlong()
        self._check(_L.lib().ac3d_matvec_timing(self._h, int(iters), int(transposed), ctypes.byref(ms),
                                                ctypes.byref(nb)))
        return ms.value, nb.value

    def block_matvec_timing(self, nrb: int = 16, iters: int = 20, transposed: bool = False):
        """(ms per block matvec of nrb right-hand sides, algorithmic bytes) on the last H-matrix."""
        ms = ctypes.c_double()
        nb = ctypes.c_longlong()
        self._check(_L.lib().ac3d_block_matvec_timing(self._h, int(nrb), int(iters), int(transposed),
                                                      ctypes.byref(ms), ctypes.byref(nb)))
        return ms.value, nb.value

    def ranks(self) -> np.ndarray:
        """ACA ranks of the admissible blocks (partition order) of the last solve's H-matrix."""
        n = self.stats()["n_approx"]
        r = np.zeros(max(n, 1), dtype=np.int32)
        self._check(_L.lib().ac3d_get_ranks(self._h, _L.ptr(r), int(n)))
        return r[:n]

    def stats(self) -> dict:
        s = _L.Stats()
        self._check(_L.lib().ac3d_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    # -- reference API --------------------------------------------------------------------------
    def set_mesh(self, Ps, Es):
        """acoustics3d.cpp:36-67: returns (Ps, Es permuted into cluster-tree order)."""
        Ps = _f64(Ps).reshape(-1, 3)
        Es = _i32(Es).reshape(-1, 3)
        out = np.zeros_like(Es)
        self._check(_L.lib().ac3d_set_mesh(self._h, _L.ptr(Ps), len(Ps), _L.ptr(Es), len(Es), _L.ptr(out)))
        self._Ps, self._Es = Ps.copy(), out
        self._diff_set = False
        if not self.silent:
            print(f"{len(Ps)} vertices, {len(Es)} elements")
        return Ps.copy(), out.copy()

    def set_diff_points(self, diff_pts) -> None:
        """acoustics3d.cpp:69-101."""
        d = _i32(list(diff_pts))
        self._check(_L.lib().ac3d_set_diff_points(self._h, _L.ptr(d), len(d)))
        self._Hs = {}
        for i in d:
            self._Hs[int(i)] = len(self._Hs)
        self._diff_set = True

    def precompute(self, Ps, Es, diff_pts):
        """acoustics3d.cpp:103-107."""
        out = self.set_mesh(Ps, Es)
        self.set_diff_points(diff_pts)
        return out

    def value(self, x=None) -> float:
        """acoustics3d.cpp:109-160: band-mean diffusion coefficient (optionally at heights x)."""
        c = ctypes.c_double()
        xx = None if x is None else _f64(x)
        self._check(_L.lib().ac3d_value(self._h, _L.ptr(xx), ctypes.byref(c)))
        return c.value

    def band_value(self, freq_band) -> float:
        """acoustics3d.cpp:162-176."""
        c = ctypes.c_double()
        self._check(_L.lib().ac3d_band_value(self._h, float(freq_band), ctypes.byref(c)))
        return c.value

    def values(self) -> list:
        """acoustics3d.cpp:178-197."""
        out = np.zeros(len(self._bands))
        self._check(_L.lib().ac3d_values(self._h, _L.ptr(out)))
        return [float(v) for v in out]

    def gradient(self, x):
        """acoustics3d.cpp:199-234: (c, dc/dx), both summed over bands."""
        xx = _f64(x)
        g = np.zeros(len(xx))
        c = ctypes.c_double()
        self._check(_L.lib().ac3d_gradient(self._h, _L.ptr(xx), ctypes.byref(c), _L.ptr(g)))
        return c.value, g

    def gradient_multi(self, x, frequencies, directions):
        """Multi-incidence objective (an extension): loss = 1 - mean over frequencies x plane-wave
        directions of the single-frequency diffusion coefficient at the receivers (set_listeners),
        with the heights x. Returns (loss, d loss / dx, coefficients (nf, nd))."""
        xx = _f64(x)
        fr = _f64(frequencies).reshape(-1)
        dr = _f64(directions).reshape(-1, 3)
        g = np.zeros(len(xx))
        cf = np.zeros((len(fr), len(dr)))
        loss = ctypes.c_double()
        self._check(_L.lib().ac3d_gradient_multi(self._h, _L.ptr(xx), _L.ptr(fr), len(fr), _L.ptr(dr), len(dr),
                                                 ctypes.byref(loss), _L.ptr(g), _L.ptr(cf)))
        return loss.value, g, cf

    def value_dev(self, x_ptr: int | None, c_ptr: int, stream: int = 0) -> None:
        """value(x) with x (HH float64, or None for the stored heights) and c (one float64) in device
        memory, ordered on the CUDA stream handle `stream`; c is the band mean."""
        self._check(_L.lib().ac3d_value_dev(self._h, ctypes.c_void_p(x_ptr or 0), ctypes.c_void_p(c_ptr),
                                            ctypes.c_void_p(stream)))

    def gradient_dev(self, x_ptr: int, c_ptr: int, grad_ptr: int, stream: int = 0) -> None:
        """gradient(x) with x, c and grad (HH float64) in device memory; c and grad band-summed."""
        self._check(_L.lib().ac3d_gradient_dev(self._h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(c_ptr),
                                               ctypes.c_void_p(grad_ptr), ctypes.c_void_p(stream)))

    @property
    def n_bands(self) -> int:
        return len(self._bands)

    def pvals_dev(self, frequency, out_ptr: int, listeners_ptr: int | None = None, n_listeners: int = 0,
                  stream: int = 0) -> None:
        """Pressures into device memory (out_ptr: L complex128), receivers optionally in device
        memory (listeners_ptr: L x 3 float64), ordered on the CUDA stream handle `stream`."""
        self._check(_L.lib().ac3d_pressures_dev(self._h, float(frequency), ctypes.c_void_p(listeners_ptr or 0),
                                                int(n_listeners), ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream)))

    def set_points(self, Ps) -> None:
        """Replace all vertex positions (same topology, partition kept)."""
        P = _f64(Ps).reshape(-1, 3)
        self._check(_L.lib().ac3d_set_points(self._h, _L.ptr(P)))
        self._Ps = P.copy()

    def pvals(self, frequency, listeners=None) -> np.ndarray:
        """acoustics3d.cpp:236-280: complex pressures at the receivers."""
        if listeners is None:
            n = ctypes.c_int()
            self._check(_L.lib().ac3d_num_listeners(self._h, ctypes.byref(n)))
            out = np.zeros(2 * n.value)
            self._check(_L.lib().ac3d_pressures(self._h, float(frequency), None, 0, _L.ptr(out)))
        else:
            Ls = _f64(listeners).reshape(-1, 3)
            out = np.zeros(2 * len(Ls))
            self._check(_L.lib().ac3d_pressures(self._h, float(frequency), _L.ptr(Ls), len(Ls), _L.ptr(out)))
        return _cplx(out)

    def pvals_multi(self, frequency, vecs, listeners=None, kind: str = "plane", surface: bool = False):
        """Pressures for several incident fields at one frequency, solved as one block against one
        H-matrix (ac3d_solve_multi). vecs: (nrhs, 3) plane-wave directions or point-source
        positions. Returns (nrhs, L) complex128, and the (nrhs, Ne) surface solutions if `surface`."""
        V = _f64(vecs).reshape(-1, 3)
        k = {"point": _L.INCIDENT_POINT, "plane": _L.INCIDENT_PLANE}[kind]
        if listeners is None:
            n = ctypes.c_int()
            self._check(_L.lib().ac3d_num_listeners(self._h, ctypes.byref(n)))
            Ls, nL = None, n.value
        else:
            Ls = _f64(listeners).reshape(-1, 3)
            nL = len(Ls)
        out = np.zeros((len(V), 2 * nL))
        ne = 0 if self._Es is None else len(self._Es)
        xs = np.zeros((len(V), 2 * max(ne, 1))) if surface else None
        self._check(_L.lib().ac3d_solve_multi(self._h, float(frequency), k, _L.ptr(V), len(V), _L.ptr(Ls),
                                              0 if Ls is None else nL, _L.ptr(out), _L.ptr(xs)))
        p = out.view(np.complex128).copy()
        if surface:
            return p, xs[:, :2 * ne].copy().view(np.complex128)
        return p

    def surface_vals(self, frequency) -> np.ndarray:
        """acoustics3d.cpp:282-315: the surface solution in tree order."""
        n = 0 if self._Es is None else len(self._Es)
        out = np.zeros(2 * max(n, 1))
        self._check(_L.lib().ac3d_surface_values(self._h, float(frequency), _L.ptr(out)))
        return _cplx(out[:2 * n])

    def get_listeners(self) -> np.ndarray:
        n = ctypes.c_int()
        self._check(_L.lib().ac3d_num_listeners(self._h, ctypes.byref(n)))
        out = np.zeros((n.value, 3))
        self._check(_L.lib().ac3d_get_listeners(self._h, _L.ptr(out)))
        return out

    def get_mesh(self, x=None):
        """acoustics3d.cpp:321-342."""
        if self._Ps is None:
            print("Warning! No mesh set. Behavior might not be as expected.")
            return np.zeros((0, 3)), np.zeros((0, 3), np.int32)
        Ps = self._Ps.copy()
        if x is not None:
            if not self._diff_set:
                print("Warning! No diff points set. Behavior might not be as expected.")
            for v, h in self._Hs.items():
                Ps[v, 1] = x[h] + self._Ps[v, 1]
        return Ps, self._Es.copy()

    def get_Hs(self) -> dict:
        return dict(self._Hs)

    def set_band(self, freq_band) -> None:
        """acoustics3d.cpp:348-351."""
        self._check(_L.lib().ac3d_set_band(self._h, float(freq_band)))
        self._bands = [float(freq_band)]

    def set_bands(self, freq_bands) -> None:
        b = _f64(list(freq_bands))
        self._check(_L.lib().ac3d_set_bands(self._h, _L.ptr(b), len(b)))
        self._bands = list(b)


def read_obj(path: str):
    """read_obj (read_obj.cpp:8-50) in the C++ library: (Ps (V, 3) float64, Es (Ne, 3) int32,
    0-based). Reads "v" and triangle "f" records, including "f a/b/c" forms and negative indices;
    skips "vn", "vt" and other records."""
    L = _L.lib()
    V, Ne = ctypes.c_int(), ctypes.c_int()
    p = os.fsencode(path)
    rc = L.ac3d_read_obj(p, None, 0, None, 0, ctypes.byref(V), ctypes.byref(Ne))
    if rc == _L.OK:
        Ps = np.zeros((V.value, 3))
        Es = np.zeros((Ne.value, 3), np.int32)
        rc = L.ac3d_read_obj(p, _L.ptr(Ps), V.value, _L.ptr(Es), Ne.value, ctypes.byref(V), ctypes.byref(Ne))
    if rc != _L.OK:
        raise AC3DError(rc, L.ac3d_obj_last_error().decode())
    return Ps, Es


def write_obj(path: str, Ps, Es) -> None:
    """write_obj (read_obj.cpp:52-63) in the C++ library: full-precision vertices, 1-based faces."""
    P = _f64(Ps).reshape(-1, 3)
    E = _i32(Es).reshape(-1, 3)
    L = _L.lib()
    rc = L.ac3d_write_obj(os.fsencode(path), _L.ptr(P), len(P), _L.ptr(E), len(E))
    if rc != _L.OK:
        raise AC3DError(rc, L.ac3d_obj_last_error().decode())


def sphere(sphere_mesh, freq, LL=100, lrad=10, actual=False, *, precision: str = "fp64") -> np.ndarray:
    """sphere.h:28-85: scattered pressure of a plane wave e^{-ikx} on a mesh read from an OBJ path
    (or given as an (Ps, Es) tuple), at LL receivers on a circle of radius lrad in the xz plane.
    actual=True solves the exact operator (every leaf pair a dense FP64 block, BiCGSTAB to 1e-12)
    where the reference uses a dense QR solve."""
    if isinstance(sphere_mesh, (tuple, list)):
        Ps, Es = sphere_mesh
    else:
        Ps, Es = read_obj(sphere_mesh)  # sphere.h:30
    Ps = _f64(Ps).reshape(-1, 3)
    Es = _i32(Es).reshape(-1, 3)
    out = np.zeros(2 * int(LL))
    rc = _L.lib().ac3d_sphere(_L.ptr(Ps), len(Ps), _L.ptr(Es), len(Es), float(freq), int(LL), float(lrad),
                              _PREC[precision], int(bool(actual)), _L.ptr(out))
    if rc != _L.OK:
        raise AC3DError(rc, "sphere evaluation failed")
    return _cplx(out)
