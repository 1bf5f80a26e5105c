"""ctypes binding of ``lib/libac3d.so`` (the C-ABI declared in ``include/ac3d.h``).

The library is required: there is no CPU fallback. If it has not been built, every call raises
``RuntimeError`` naming the build step.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libac3d.so")

OK, ERR_ARG, ERR_STATE, ERR_INTERNAL, ERR_RESOURCE, ERR_CUDA, ERR_NOT_CONVERGED = range(7)
PREC_MIXED, PREC_FP64 = 0, 1
INCIDENT_POINT, INCIDENT_PLANE = 0, 1
LISTENER_DENSE, LISTENER_ACA = 0, 1
ASSEMBLY_DF, ASSEMBLY_FP32 = 0, 1

# Exported symbols and their signatures (restype, argtypes); kept in step with include/ac3d.h.
_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
SIGNATURES = {
    "ac3d_version": (ctypes.c_char_p, []),
    "ac3d_create": (_I, [ctypes.POINTER(_P), _I, _D, _P, _I, _I, _D, _D, _D, _P, _D, _D, _I]),
    "ac3d_destroy": (None, [_P]),
    "ac3d_select_device": (_I, [_I]),
    "ac3d_last_error": (ctypes.c_char_p, [_P]),
    "ac3d_set_precision": (_I, [_P, _I]),
    "ac3d_set_incident": (_I, [_P, _I, _P]),
    "ac3d_set_listener_mode": (_I, [_P, _I]),
    "ac3d_set_solver": (_I, [_P, _I, _D, _I]),
    "ac3d_set_krylov": (_I, [_P, _I, _I]),
    "ac3d_set_assembly": (_I, [_P, _I]),
    "ac3d_set_tensor_cores": (_I, [_P, _I]),
    "ac3d_get_ranks": (_I, [_P, _P, _I]),
    "ac3d_gradient_multi": (_I, [_P, _P, _P, _I, _P, _I, _P, _P, _P]),
    "ac3d_block_matvec_timing": (_I, [_P, _I, _I, _I, _P, _P]),
    "ac3d_relief_sizes": (_I, [_I, _I, _I, _I, _P, _P]),
    "ac3d_relief_dev": (_I, [_D, _D, _D, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P]),
    "ac3d_set_listeners": (_I, [_P, _P, _I]),
    "ac3d_set_mesh": (_I, [_P, _P, _I, _P, _I, _P]),
    "ac3d_set_diff_points": (_I, [_P, _P, _I]),
    "ac3d_set_band": (_I, [_P, _D]),
    "ac3d_set_bands": (_I, [_P, _P, _I]),
    "ac3d_num_listeners": (_I, [_P, ctypes.POINTER(_I)]),
    "ac3d_get_listeners": (_I, [_P, _P]),
    "ac3d_set_points": (_I, [_P, _P]),
    "ac3d_pressures": (_I, [_P, _D, _P, _I, _P]),
    "ac3d_pressures_dev": (_I, [_P, _D, _P, _I, _P, _P]),
    "ac3d_surface_values": (_I, [_P, _D, _P]),
    "ac3d_solve_multi": (_I, [_P, _D, _I, _P, _I, _P, _I, _P, _P]),
    "ac3d_band_value": (_I, [_P, _D, _P]),
    "ac3d_values": (_I, [_P, _P]),
    "ac3d_value": (_I, [_P, _P, _P]),
    "ac3d_gradient": (_I, [_P, _P, _P, _P]),
    "ac3d_value_dev": (_I, [_P, _P, _P, _P]),
    "ac3d_gradient_dev": (_I, [_P, _P, _P, _P, _P]),
    "ac3d_sphere": (_I, [_P, _I, _P, _I, _D, _I, _D, _I, _I, _P]),
    "ac3d_set_actual": (_I, [_P, _I]),
    "ac3d_read_obj": (_I, [ctypes.c_char_p, _P, _I, _P, _I, _P, _P]),
    "ac3d_write_obj": (_I, [ctypes.c_char_p, _P, _I, _P, _I]),
    "ac3d_obj_last_error": (ctypes.c_char_p, []),
    "ac3d_kernel_launches": (ctypes.c_longlong, []),
    "ac3d_texmap_create": (_I, [_P, _P, _I, _I, _I]),
    "ac3d_texmap_destroy": (None, [_P]),
    "ac3d_texmap_sample_dev": (_I, [_P, _P, _P, _P]),
    "ac3d_texmap_scatter_dev": (_I, [_P, _P, _P, _P]),
    "ac3d_get_stats": (_I, [_P, _P]),
    "ac3d_matvec_timing": (_I, [_P, _I, _I, _P, _P]),
    "ac3d_far_field_noalloc": (_I, [_P, _I, _P, _I, _P, _D, _P, _I, _P, _P]),
    "ac3d_partition_build": (_I, [_P, _I, _P, _I, _I, _D, ctypes.POINTER(_P)]),
    "ac3d_partition_counts": (_I, [_P, _P, _P, _P, _P]),
    "ac3d_partition_get": (_I, [_P, _P, _P, _P, _P]),
    "ac3d_partition_free": (None, [_P]),
    "ac3d_server_create": (_I, [ctypes.POINTER(_P), _I, _I, ctypes.c_longlong]),
    "ac3d_server_destroy": (None, [_P]),
    "ac3d_server_set_krylov": (_I, [_P, _I, _I]),
    "ac3d_server_set_assembly": (_I, [_P, _I]),
    "ac3d_server_last_error": (ctypes.c_char_p, [_P]),
    "ac3d_server_add_mesh": (_I, [_P, _P, _I, _P, _I, _I, _D, _D, _D, _P, ctypes.POINTER(_I)]),
    "ac3d_server_submit": (_I, [_P, _I, _D, _I, _P, _P, _I, ctypes.POINTER(ctypes.c_longlong)]),
    "ac3d_server_poll": (_I, [_P, ctypes.c_longlong, ctypes.POINTER(_I)]),
    "ac3d_server_wait": (_I, [_P, ctypes.c_longlong, _P, _P]),
    "ac3d_admit_next": (_I, [_P, _P, _I, ctypes.c_longlong, ctypes.c_longlong, _I]),
    "ac3d_tensor_selftest": (_I, [_P, _P, _I, _P]),
}


class Stats(ctypes.Structure):
    """Mirror of ``ac3d_stats``."""
    _fields_ = [("n_elements", _I), ("n_direct", _I), ("n_approx", _I), ("n_leaves", _I),
                ("near_entries", ctypes.c_longlong), ("lr_entries", ctypes.c_longlong),
                ("mean_rank", _D), ("max_rank", _I), ("hmat_bytes", ctypes.c_longlong),
                ("solves", _I), ("iterations", _I), ("outer_steps", _I), ("matvecs", _I),
                ("rel_residual", _D), ("converged", _I),
                ("ms_assemble", _D), ("ms_solve", _D), ("ms_listener", _D), ("ms_adjoint", _D),
                ("ms_total", _D), ("kernel_launches", ctypes.c_longlong),
                ("aca_entries_evaluated", ctypes.c_longlong), ("ms_graph", _D)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class RequestInfo(ctypes.Structure):
    """Mirror of ``ac3d_request_info``."""
    _fields_ = [("status", _I), ("slot", _I), ("queue_ms", _D), ("run_ms", _D), ("latency_ms", _D),
                ("footprint_bytes", ctypes.c_longlong), ("hmat_bytes", ctypes.c_longlong),
                ("lr_entries", ctypes.c_longlong), ("near_entries", ctypes.c_longlong),
                ("iterations", _I), ("outer_steps", _I), ("rel_residual", _D),
                ("ms_assemble", _D), ("ms_solve", _D), ("ms_listener", _D), ("ms_graph", _D),
                ("aca_entries_evaluated", ctypes.c_longlong)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = range(4)
SERVE_MAX_BYPASS = 8


class AC3DError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[ac3d error {code}] {msg}")
        self.code = code


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
                               "or `python acoustic_reliefs_gb300/build.py`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(ctx, rc: int) -> None:
    if rc != OK:
        msg = lib().ac3d_last_error(ctx).decode() if ctx else "invalid argument"
        raise AC3DError(rc, msg or "invalid argument")


def ptr(a) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)
