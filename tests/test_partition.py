"""CPU: the product's cluster tree / block partition is bit-identical to the oracle's."""
import ctypes

import numpy as np
import pytest

from acoustic_reliefs_gb300 import _lib as L
from acoustic_reliefs_gb300 import meshes
from tests import cases


def product_partition(Ps, Es, leaf, factor):
    lib = L.lib()
    Ps = np.ascontiguousarray(Ps, np.float64)
    Es = np.ascontiguousarray(Es, np.int32)
    h = ctypes.c_void_p()
    assert lib.ac3d_partition_build(L.ptr(Ps), len(Ps), L.ptr(Es), len(Es), leaf, factor, ctypes.byref(h)) == 0
    nd, na, nl, ok = (ctypes.c_int() for _ in range(4))
    lib.ac3d_partition_counts(h, ctypes.byref(nd), ctypes.byref(na), ctypes.byref(nl), ctypes.byref(ok))
    order = np.zeros(len(Es), np.int32)
    direct = np.zeros((nd.value, 4), np.int32)
    approx = np.zeros((na.value, 4), np.int32)
    leaves = np.zeros(nl.value + 1, np.int32)
    lib.ac3d_partition_get(h, L.ptr(order), L.ptr(direct), L.ptr(approx), L.ptr(leaves))
    lib.ac3d_partition_free(h)
    return order, direct, approx, leaves, bool(ok.value)


@pytest.mark.parametrize("case", ["sphere", "relief", "relief_sub", "relief_leaf128"])
def test_partition_bit_exact(oracle_lib, case):
    if case == "sphere":
        c = cases.sphere_c1()
        Ps, Es, leaf, factor = c["Ps"], c["Es"], 32, 2.0
    elif case == "relief":
        c = cases.relief_small()
        Ps, Es, leaf, factor = c["Ps"], c["Es"], 32, 2.0
    elif case == "relief_sub":
        R = meshes.relief(0.6, 0.6, 0.05, 20, 4, 20, 1, meshes.smooth_heightmap(32, 4))
        Ps, Es, leaf, factor = R.Ps, R.Es, 64, 1.5
    else:
        c = cases.relief_small()
        Ps, Es, leaf, factor = c["Ps"], c["Es"], 128, 1.5
    order, direct, approx, leaves, ok = product_partition(Ps, Es, leaf, factor)
    m = oracle_lib.Mesh(Ps, Es, leaf, factor)
    assert ok and m.tree_ok
    assert np.array_equal(order, m.order)
    assert np.array_equal(direct, m.direct)
    assert np.array_equal(approx, m.approx)
    # leaves tile [0, Ne) and near blocks are leaf x leaf
    assert leaves[0] == 0 and leaves[-1] == len(Es) and np.all(np.diff(leaves) > 0)
    assert np.all(np.diff(leaves) <= leaf)
    ls = set(leaves[:-1].tolist())
    assert all(d[0] in ls and d[2] in ls for d in direct)


def test_partition_covers_matrix_once():
    """Every (row, column) pair lies in exactly one block."""
    Ps, Es = meshes.icosphere(2, 1.0)
    order, direct, approx, leaves, ok = product_partition(Ps, Es, 16, 1.5)
    n = len(Es)
    cover = np.zeros((n, n), np.int32)
    for rs, re, cs, ce in np.vstack([direct, approx]):
        cover[rs:re, cs:ce] += 1
    assert np.all(cover == 1)


def test_partition_rejects_bad_indices():
    Ps, Es = meshes.icosphere(1, 1.0)
    Es = Es.copy()
    Es[3, 1] = len(Ps) + 5
    h = ctypes.c_void_p()
    lib = L.lib()
    Ps = np.ascontiguousarray(Ps, np.float64)
    Es = np.ascontiguousarray(Es, np.int32)
    assert lib.ac3d_partition_build(L.ptr(Ps), len(Ps), L.ptr(Es), len(Es), 16, 1.5, ctypes.byref(h)) == L.ERR_ARG
