"""CPU: the C++ OBJ reader and writer (read_obj.cpp:8-63) through the C-ABI, against the NumPy
reader in ``meshes`` and hand-written files with the records the reference reader rejects."""
import numpy as np
import pytest

from acoustic_reliefs_gb300 import meshes
from acoustic_reliefs_gb300.acoustics3d import AC3DError, read_obj, write_obj


def test_round_trip_is_exact(tmp_path):
    Ps, Es = meshes.icosphere(2, 0.5)
    Ps = Ps * np.pi  # digits that a short format would lose
    p = str(tmp_path / "s.obj")
    write_obj(p, Ps, Es)
    P2, E2 = read_obj(p)
    assert np.array_equal(P2, Ps) and np.array_equal(E2, Es)
    P3, E3 = meshes.read_obj(p)
    assert np.array_equal(P3, Ps) and np.array_equal(E3, Es)


def test_normals_texcoords_slashes_negative_indices(tmp_path):
    p = tmp_path / "m.obj"
    p.write_text("# comment\nmtllib a.mtl\no box\n"
                 "v 0 0 0\nv 1 0 0 1.0\nv 0 1 0\nvn 0 0 1\nvt 0.5 0.5\nv 1 1 0\n"
                 "g side\nusemtl m\ns off\n"
                 "f 1/1/1 2/1/1 3/1/1\n"
                 "f 2//1 4//1 3//1  # trailing comment\n"
                 "f -3 -1 -2\n")
    Ps, Es = read_obj(str(p))
    assert Ps.shape == (4, 3) and np.array_equal(Ps[3], [1.0, 1.0, 0.0])
    assert Es.tolist() == [[0, 1, 2], [1, 3, 2], [1, 3, 2]]


@pytest.mark.parametrize("body,msg", [("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nf 1 2 4 3\n", "triangles"),
                                      ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 5\n", "out of range"),
                                      ("v 0 0\nf 1 2 3\n", "vertex"),
                                      ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2\n", "triangles")])
def test_malformed_files_raise(tmp_path, body, msg):
    p = tmp_path / "bad.obj"
    p.write_text(body)
    with pytest.raises(AC3DError) as e:
        read_obj(str(p))
    assert msg in str(e.value)


def test_missing_file_raises(tmp_path):
    with pytest.raises(AC3DError):
        read_obj(str(tmp_path / "none.obj"))
