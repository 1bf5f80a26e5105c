"""Tensor-core (tcgen05) product of the block matvec, checked against an FP64 product."""
import numpy as np
import pytest

from acoustic_reliefs_gb300 import _lib as L


@pytest.mark.gpu
@pytest.mark.parametrize("K", [8, 32, 64])
def test_tcgen05_tf32_split_product(gpu_lib, K):
    """D = A B^T with TF32 operands split in three products: FP32-level accuracy (error per entry
    within 1e-5 of the entry's scale sum |a||b|, against FP64)."""
    rng = np.random.default_rng(K)
    A = rng.normal(size=(128, K)).astype(np.float32)
    B = rng.normal(size=(32, K)).astype(np.float32)
    D = np.zeros((128, 32), np.float32)
    rc = L.lib().ac3d_tensor_selftest(L.ptr(A), L.ptr(B), K, L.ptr(D))
    assert rc == L.OK
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T
    assert np.max(np.abs(D - ref) / scale) < 1e-5
