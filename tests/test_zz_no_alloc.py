"""GPU: the allocation-free far-field entry point against the allocating solver path.

ac3d_far_field_noalloc exists for callers that must not allocate device memory when they ask for
a result (a real-time audio callback, a frame loop, a host whose allocator owns the device
memory). It keeps its scratch in a fixed array reserved on the device, shared by every call. This
test computes a surface solution with the regular API, evaluates the receivers three times in a
row through the new entry point, and compares the results with ac3d_pressures, which runs the
same FP64 product with allocated scratch: equal to 1e-12 (only the summation order differs), and
bitwise equal from call to call (the sums have a fixed order). Device free memory is the same
after the second and third calls as after the first. Collected last so that a failure here does
not stop the other GPU tests of a -x run."""
import ctypes
import math

import numpy as np
import pytest

from acoustic_reliefs_gb300 import _lib as L
from acoustic_reliefs_gb300.acoustics3d import DiffBEM
from tests import cases

pytestmark = pytest.mark.gpu
TOL_VS_PRESSURES = 1e-12


def test_far_field_noalloc_matches_pressures(gpu_lib):
    torch = pytest.importorskip("torch")
    c = cases.relief_small()
    freq = c["freq"]
    assert L.lib().ac3d_select_device(0) == L.OK  # the library runtime's device (torch's is separate)
    bem = DiffBEM(c["leaf"], c["factor"], [freq], 1, c["aca_tol"], c["aca_tol"], c["tol"], precision="fp64",
                  incident=("plane", c["vec"]), listener="dense", device=0)
    bem.silent = True
    Ps, Es_tree = bem.set_mesh(c["Ps"], c["Es"])
    x = bem.surface_vals(freq)                   # solution in tree order
    y_ref = bem.pvals(freq, c["Ls"])             # same solve + the allocating far-field product

    dev = torch.device("cuda", 0)
    Ps_d = torch.tensor(Ps, dtype=torch.float64, device=dev)
    Es_d = torch.tensor(Es_tree, dtype=torch.int32, device=dev)
    x_d = torch.tensor(np.ascontiguousarray(x).view(np.float64), dtype=torch.float64, device=dev)
    Ls_d = torch.tensor(c["Ls"], dtype=torch.float64, device=dev)
    ys = [torch.zeros(2 * len(c["Ls"]), dtype=torch.float64, device=dev) for _ in range(3)]
    k = 2 * math.pi * freq / 344.0
    stream = torch.cuda.current_stream(dev)
    free = []
    for y_d in ys:
        rc = L.lib().ac3d_far_field_noalloc(ctypes.c_void_p(Ps_d.data_ptr()), len(Ps),
                                            ctypes.c_void_p(Es_d.data_ptr()), len(Es_tree),
                                            ctypes.c_void_p(x_d.data_ptr()), k, ctypes.c_void_p(Ls_d.data_ptr()),
                                            len(c["Ls"]), ctypes.c_void_p(y_d.data_ptr()),
                                            ctypes.c_void_p(stream.cuda_stream))
        assert rc == L.OK
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info(dev)[0])
    results = [y.cpu().numpy().view(np.complex128).copy() for y in ys]
    for y in results:
        assert cases.rel_l2(y, y_ref) < TOL_VS_PRESSURES
    assert np.array_equal(results[0], results[1]) and np.array_equal(results[1], results[2])
    assert free[1] == free[0] and free[2] == free[0]


def test_far_field_noalloc_rejects_oversize(gpu_lib):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    Ps_d = torch.zeros(9, dtype=torch.float64, device=dev)
    Es_d = torch.tensor([0, 1, 2], dtype=torch.int32, device=dev)
    x_d = torch.zeros(2, dtype=torch.float64, device=dev)
    L_big = 70000
    Ls_d = torch.zeros(3 * L_big, dtype=torch.float64, device=dev)
    y_d = torch.zeros(2 * L_big, dtype=torch.float64, device=dev)
    rc = L.lib().ac3d_far_field_noalloc(ctypes.c_void_p(Ps_d.data_ptr()), 3, ctypes.c_void_p(Es_d.data_ptr()), 1,
                                        ctypes.c_void_p(x_d.data_ptr()), 1.0, ctypes.c_void_p(Ls_d.data_ptr()), L_big,
                                        ctypes.c_void_p(y_d.data_ptr()), ctypes.c_void_p(0))
    assert rc == L.ERR_RESOURCE
