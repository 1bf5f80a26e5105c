"""GPU: the relief generator on the device (ac3d_relief_dev: generate_base_mesh + face_subdivision,
pyoptim/mesher.py:87-231) is bitwise the host generator (meshes.relief, the NumPy restatement the
tests and the bench use) for subdiv_top 0 to 3: vertices, triangles, top vertex ids and uvs."""
import numpy as np
import pytest

from acoustic_reliefs_gb300 import meshes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,subdiv", [((0.6, 0.6, 0.05, 30, 7, 30), 0), ((0.6, 0.6, 0.05, 30, 7, 30), 1),
                                         ((0.6, 0.6, 0.05, 30, 7, 30), 2), ((0.6, 0.6, 0.05, 30, 7, 30), 3),
                                         ((0.9, 0.9, 0.05, 48, 7, 48), 2), ((0.6, 0.6, 0.05, 64, 8, 64), 0)])
def test_relief_device_bitwise(gpu_lib, dims, subdiv):
    torch = pytest.importorskip("torch")
    w, b, h, nx, ny, nz = dims
    R = meshes.relief(w, b, h, nx, ny, nz, subdiv)
    Ps, Es, top, uvs = meshes.relief_device(w, b, h, nx, ny, nz, subdiv, device="cuda:0")
    torch.cuda.synchronize()
    assert np.array_equal(Ps.cpu().numpy(), R.Ps)
    assert np.array_equal(Es.cpu().numpy().astype(np.int64), R.Es)
    assert np.array_equal(top.cpu().numpy(), R.diff_pts)
    assert np.array_equal(uvs.cpu().numpy(), R.uvs)
