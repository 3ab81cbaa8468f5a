"""HDF5 subset and input.dat deck (euler3d.cpp:84-117, :243-312; io.h:28-205). CPU only."""
import ctypes as C

import numpy as np
import pytest

import mgcfd
from mgcfd import _lib


def test_mesh_round_trip_through_files(tmp_path):
    mesh = mgcfd.HostMesh.generate(7, 3, 12)
    mesh.write(str(tmp_path), "grid_")
    back = mgcfd.HostMesh.load("input.dat", str(tmp_path))
    assert back.num_levels == 3
    for a, b in zip(mesh.levels(), back.levels()):
        for f in ("coords", "edge_to_nodes", "bnd_to_node", "bnd_group", "edge_weights", "bnd_weights"):
            np.testing.assert_array_equal(getattr(a, f), getattr(b, f))
        if a.node_to_mg is None:
            assert b.node_to_mg is None
        else:
            np.testing.assert_array_equal(a.node_to_mg, b.node_to_mg)


def test_base_array_index_one_is_the_default(tmp_path):
    """euler3d.cpp:92: maps are 1-based unless input.dat says otherwise."""
    mesh = mgcfd.HostMesh.generate(5, 2, 1)
    mesh.write(str(tmp_path), "m_")
    deck = (tmp_path / "input.dat").read_text().replace("base_array_index=0\n", "")
    (tmp_path / "input.dat").write_text(deck)
    with pytest.raises(_lib.MgcfdError, match="out of range"):
        mgcfd.HostMesh.load("input.dat", str(tmp_path))  # 0-based ids read as 1-based: id -1


def test_write_read_f64_dataset_with_attributes(tmp_path):
    lib = _lib.load()
    a = np.arange(35, dtype=np.float64).reshape(7, 5) / 3.0
    p = str(tmp_path / "x.h5").encode()
    _lib.check(lib.mgcfd_h5_write_f64(p, b"p_variables_result_L0", a.ctypes.data_as(_lib.c_double_p), 7, 5))
    np.testing.assert_array_equal(mgcfd.h5_read(tmp_path / "x.h5", "p_variables_result_L0"), a)
    dims = (C.c_int64 * 2)()
    rank = C.c_int()
    _lib.check(lib.mgcfd_h5_dataset_shape(p, b"p_variables_result_L0", dims, C.byref(rank)))
    assert (rank.value, dims[0], dims[1]) == (2, 7, 5)
    assert lib.mgcfd_h5_read_f64(p, b"missing", a.ctypes.data_as(_lib.c_double_p), 35) == _lib.ERR_IO


def test_legacy_files_span_several_symbol_table_nodes(tmp_path):
    """13 datasets per level file need two symbol-table nodes under the group B-tree."""
    mesh = mgcfd.HostMesh.generate(6, 2, 3)
    mesh.write(str(tmp_path), "m_", legacy_datasets=True)
    modern = mgcfd.HostMesh.load("input.dat", str(tmp_path))
    legacy = mgcfd.HostMesh.load("input.dat", str(tmp_path), legacy=True)
    for a, b in zip(modern.levels(), legacy.levels()):
        np.testing.assert_array_equal(a.coords, b.coords)
        np.testing.assert_array_equal(a.edge_to_nodes, b.edge_to_nodes)
        assert b.volumes is not None and (b.volumes > 0).all()
        assert np.abs(np.linalg.norm(b.edge_weights, axis=1) - np.linalg.norm(a.edge_weights, axis=1)).max() > 0


def test_truncated_and_foreign_files_are_rejected(tmp_path):
    lib = _lib.load()
    a = np.ones((4, 3))
    p = tmp_path / "t.h5"
    _lib.check(lib.mgcfd_h5_write_f64(str(p).encode(), b"d", a.ctypes.data_as(_lib.c_double_p), 4, 3))
    raw = p.read_bytes()
    p.write_bytes(raw[: len(raw) - 40])
    out = np.empty(12)
    assert lib.mgcfd_h5_read_f64(str(p).encode(), b"d", out.ctypes.data_as(_lib.c_double_p), 12) == _lib.ERR_IO
    (tmp_path / "n.h5").write_bytes(b"not hdf5 at all")
    assert lib.mgcfd_h5_read_f64(str(tmp_path / "n.h5").encode(), b"d", out.ctypes.data_as(_lib.c_double_p),
                                 12) == _lib.ERR_IO


@pytest.mark.parametrize("text,msg", [
    ("num_levels=1\nmesh_name=fvcorr\n[levels]\n0=a.h5\n", "size not present"),
    ("size=1\nmesh_name=fvcorr\n[levels]\n0=a.h5\n", "Need to know number of levels"),
    ("size=1\nnum_levels=1\nmesh_name=foo\n[levels]\n0=a.h5\n", "Unknown mesh_name"),
    ("size=1\nnum_levels=1\n[levels]\n0=a.h5\n", "mesh name not present"),
    ("size=1\nnum_levels=1\nmesh_name=rotor37\n", "mesh filenames not present"),
    ("size=1\nnum_levels=2\nmesh_name=m6wing\n[levels]\n0=a.h5\n", "EOF"),
])
def test_input_deck_errors(tmp_path, text, msg):
    (tmp_path / "input.dat").write_text(text)
    with pytest.raises(_lib.MgcfdError, match=msg):
        mgcfd.HostMesh.load("input.dat", str(tmp_path))


def test_input_deck_comments_and_missing_level_file(tmp_path):
    (tmp_path / "input.dat").write_text("# comment\nsize=8\nnum_levels=1\nmesh_name=la_cascade\n[levels]\n0=nope.h5\n")
    with pytest.raises(_lib.MgcfdError, match="cannot open"):
        mgcfd.HostMesh.load("input.dat", str(tmp_path))
