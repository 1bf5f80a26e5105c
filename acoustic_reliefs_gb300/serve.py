"""Request server: many forward solves (meshes x frequencies x incident fields) on one GPU.

Python side of ``ac3d_server_*`` (include/ac3d.h). Meshes are registered once and stay on the
device; each submitted request (mesh, frequency, incident field, receivers) is queued, admitted
when a slot is free and its estimated device footprint fits in the byte budget, and solved on its
slot's own CUDA stream, overlapping with the other running requests. The reference has no server:
it evaluates one frequency after another inside DiffBEM (adjoint.cpp:46-104); a request here is
one iteration of that loop (assemble, solve, receivers; acoustics3d.cpp:236-280 ``pvals``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as _L
from ._lib import AC3DError

__all__ = ["Server", "admit_next"]

_PREC = {"mixed": _L.PREC_MIXED, "fp64": _L.PREC_FP64}
_STATE = {_L.REQ_QUEUED: "queued", _L.REQ_RUNNING: "running", _L.REQ_DONE: "done", _L.REQ_FAILED: "failed"}


def admit_next(footprints, bypassed, budget: int, in_use: int, n_running: int) -> int:
    """The server's admission rule (``ac3d_admit_next``): index of the queued request to start next,
    or -1."""
    fp = np.ascontiguousarray(footprints, dtype=np.int64)
    by = np.ascontiguousarray(bypassed, dtype=np.int32)
    return int(_L.lib().ac3d_admit_next(_L.ptr(fp), _L.ptr(by), len(fp), int(budget), int(in_use), int(n_running)))


class Server:
    def __init__(self, slots: int = 4, precision: str = "mixed", hbm_budget: int = 0, device: int | None = None,
                 krylov: str = "bicgstab", restart: int = 300, assembly: str = "df"):
        L = _L.lib()
        if device is not None:
            rc = L.ac3d_select_device(int(device))
            if rc != _L.OK:
                raise AC3DError(rc, f"cannot select CUDA device {device}")
        h = ctypes.c_void_p()
        rc = L.ac3d_server_create(ctypes.byref(h), int(slots), _PREC[precision], int(hbm_budget))
        if rc != _L.OK:
            raise AC3DError(rc, "cannot create the server (no CUDA device or invalid arguments)")
        self._h = h
        self._check(L.ac3d_server_set_krylov(h, {"bicgstab": 0, "gmres": 1}[krylov], int(restart)))
        self._check(L.ac3d_server_set_assembly(h, {"df": _L.ASSEMBLY_DF, "fp32": _L.ASSEMBLY_FP32}[assembly]))
        self.precision = precision
        self.slots = slots
        self._nL: dict[int, int] = {}

    def _check(self, rc):
        if rc != _L.OK:
            raise AC3DError(rc, _L.lib().ac3d_server_last_error(self._h).decode() or "invalid argument")

    def add_mesh(self, Ps, Es, cluster_size=32, radius_factor=2.0, aca_tol=1e-4, solver_tol=1e-6):
        """Registers a mesh; returns (mesh_id, Es in tree order), the order results refer to."""
        Ps = np.ascontiguousarray(Ps, dtype=np.float64).reshape(-1, 3)
        Es = np.ascontiguousarray(Es, dtype=np.int32).reshape(-1, 3)
        Eo = np.zeros_like(Es)
        mid = ctypes.c_int()
        self._check(_L.lib().ac3d_server_add_mesh(self._h, _L.ptr(Ps), len(Ps), _L.ptr(Es), len(Es),
                                                  int(cluster_size), float(radius_factor), float(aca_tol),
                                                  float(solver_tol), _L.ptr(Eo), ctypes.byref(mid)))
        return mid.value, Eo

    def submit(self, mesh_id: int, frequency: float, listeners, incident=("plane", (0.0, -1.0, 0.0))) -> int:
        kind = {"point": _L.INCIDENT_POINT, "plane": _L.INCIDENT_PLANE}[incident[0]]
        v = np.ascontiguousarray(incident[1], dtype=np.float64).reshape(3)
        Ls = np.ascontiguousarray(listeners, dtype=np.float64).reshape(-1, 3)
        req = ctypes.c_longlong()
        self._check(_L.lib().ac3d_server_submit(self._h, int(mesh_id), float(frequency), kind, _L.ptr(v),
                                                _L.ptr(Ls), len(Ls), ctypes.byref(req)))
        self._nL[req.value] = len(Ls)
        return req.value

    def poll(self, request: int) -> str:
        st = ctypes.c_int()
        self._check(_L.lib().ac3d_server_poll(self._h, ctypes.c_longlong(request), ctypes.byref(st)))
        return _STATE[st.value]

    def wait(self, request: int):
        """Blocks until the request finishes; returns (pressures (L,) complex128, info dict)."""
        n = self._nL.pop(request, 0)
        out = np.zeros(2 * max(n, 1))
        info = _L.RequestInfo()
        rc = _L.lib().ac3d_server_wait(self._h, ctypes.c_longlong(request), _L.ptr(out), ctypes.byref(info))
        self._check(rc)
        return out[:2 * n].view(np.complex128).copy(), info.as_dict()

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h:
            _L.lib().ac3d_server_destroy(h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
