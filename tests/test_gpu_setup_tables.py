"""Tables built on the GPU (device_setup.cu) equal the host reference
implementation (setup.cpp) exactly: permutations, edge order and
orientation, CSR offsets and lists, boundary rows, multigrid maps, and the
volumes and weights (both follow the reference's sequential order).  Only the
1/vol and cube root of the volume are computed on the device in both paths."""
import ctypes as C

import numpy as np
import pytest

import mgcfd
from mgcfd import _lib

pytestmark = pytest.mark.gpu

TABLES = {0: ("PERM", np.int32), 1: ("EDGES", np.int32), 2: ("WEIGHTS", np.float64), 3: ("VOLUMES", np.float64),
          4: ("INV_VOL", np.float64), 5: ("CBRT_VOL", np.float64), 6: ("BIDX", np.int32), 7: ("BDATA", np.float64),
          8: ("N2MG", np.int32), 9: ("DVEC", np.float64), 10: ("CH_OFF", np.int32), 11: ("CH_LIST", np.int32),
          12: ("A_OFF", np.int32), 13: ("B_OFF", np.int32), 14: ("B_LIST", np.int32), 15: ("WEIGHTS32", np.float32)}


def table(solver, level, t):
    lib = _lib.load()
    n = C.c_int64()
    _lib.check(lib.mgcfd_solver_table(solver._h, level, t, None, 0, C.byref(n)))
    dt = TABLES[t][1]
    out = np.empty(n.value // np.dtype(dt).itemsize, dtype=dt)
    if n.value:
        _lib.check(lib.mgcfd_solver_table(solver._h, level, t, out.ctypes.data, n.value, C.byref(n)))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n,nl,renumber", [(11, 3, "spatial"), (16, 4, "spatial"), (9, 2, "none"), (24, 3, "spatial")])
def test_device_tables_equal_host_tables(n, nl, renumber, precision):
    """Mixed precision computes the per-edge geometry in FP32, on the device and
    on the host alike: its weights and volumes must agree bit for bit too."""
    mesh = mgcfd.HostMesh.generate(n, nl, 300 + n)
    dev = mgcfd.Solver(mesh, 0.8, 3.0, increment="gather", renumber=renumber, precision=precision)
    host = mgcfd.Solver(mesh, 0.8, 3.0, increment="gather", renumber=renumber, host_setup=True, precision=precision)
    for l in range(nl):
        for t, (name, _) in TABLES.items():
            a, b = table(dev, l, t), table(host, l, t)
            assert a.shape == b.shape, (l, name)
            np.testing.assert_array_equal(a, b, err_msg=f"level {l} table {name}")


def test_device_setup_rejects_out_of_range_maps():
    mesh = mgcfd.HostMesh.generate(8, 2, 1)
    levels = mesh.levels()
    bad = [mgcfd.Level(**{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in L.__dict__.items()
                          if k != "owner"}) for L in levels]
    bad[0].edge_to_nodes[5, 1] = bad[0].nnodes + 7
    with pytest.raises(_lib.MgcfdError, match="out of range"):
        mgcfd.Solver(bad, 0.5, 3.0)
    bad[0].edge_to_nodes[5, 1] = 0
    bad[0].node_to_mg[3] = -2
    with pytest.raises(_lib.MgcfdError, match="out of range"):
        mgcfd.Solver(bad, 0.5, 3.0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_legacy_mesh_on_device(tmp_path, precision):
    import oracle as O
    from parity import MIXED_TOL, STATE_TOL, per_variable_errors, state_error
    mesh = mgcfd.HostMesh.generate(10, 3, 8)
    mesh.write(str(tmp_path), "m_", legacy_datasets=True)
    legacy = mgcfd.HostMesh.load("input.dat", str(tmp_path), legacy=True)
    ref = O.OracleRun(legacy.levels())
    assert ref.run(0.6, 2.0, 3)[0] == 0
    s = mgcfd.Solver(legacy, 0.6, 2.0, precision=precision)
    s.run(3)
    assert s.synchronize() == 0
    for l in range(3):
        got, want = s.fetch(l), ref.get(l, O.Q_VARIABLES)
        if precision == "fp64":
            assert state_error(got, want) <= STATE_TOL
        else:  # volumes as read, FP64-damped weights rounded to FP32 (legacy datasets)
            mx, l2 = per_variable_errors(got, want)
            assert mx.max() <= MIXED_TOL and l2.max() <= MIXED_TOL, (l, mx, l2)
    host = mgcfd.Solver(legacy, 0.6, 2.0, precision=precision, host_setup=True, increment="gather")
    dev = mgcfd.Solver(legacy, 0.6, 2.0, precision=precision, increment="gather")
    for l in range(3):
        for t in (3, 15 if precision == "mixed" else 2):  # volumes, weights
            np.testing.assert_array_equal(table(dev, l, t), table(host, l, t))


@pytest.mark.parametrize("renumber", ["spatial", "none"])
def test_batch_tables_are_shifted_single_mesh_tables(renumber):
    """A batch is prepared as one set of concatenated levels; mesh m's tables
    must equal those of mesh m prepared alone, shifted by its node, edge and
    boundary-row offsets."""
    nl = 3
    meshes = [mgcfd.HostMesh.generate(n, nl, 40 + n) for n in (9, 12, 7, 10)]
    machs, aoas = [0.5, 0.8, 0.65, 0.7], [1.0, 3.0, 0.0, 5.5]
    batch = mgcfd.Batch(meshes, machs, aoas, increment="gather", renumber=renumber)
    singles = [mgcfd.Solver(m, a, b, increment="gather", renumber=renumber) for m, a, b in zip(meshes, machs, aoas)]
    for l in range(nl):
        nn = [m.level(l).nnodes for m in meshes]
        ne = [m.level(l).nedges for m in meshes]
        noff = np.concatenate([[0], np.cumsum(nn)])
        eoff = np.concatenate([[0], np.cumsum(ne)])
        nc = [m.level(l + 1).nnodes for m in meshes] if l + 1 < nl else None
        coff = np.concatenate([[0], np.cumsum(nc)]) if nc else None
        fine_off = np.concatenate([[0], np.cumsum([m.level(l - 1).nnodes for m in meshes])]) if l > 0 else None
        rows = [int((table(s, l, 6) >= 0).sum()) for s in singles]
        roff = np.concatenate([[0], np.cumsum(rows)])
        for t, (name, _) in TABLES.items():
            parts = [table(s, l, t) for s in singles]
            if name in ("PERM", "EDGES"):
                parts = [p + noff[m] for m, p in enumerate(parts)]
            elif name == "BIDX":
                parts = [np.where(p >= 0, p + roff[m], p) for m, p in enumerate(parts)]
            elif name == "N2MG" and coff is not None:
                parts = [p + coff[m] for m, p in enumerate(parts)]
            elif name in ("CH_OFF",) and fine_off is not None:
                parts = [p[:-1] + fine_off[m] for m, p in enumerate(parts)] + [np.array([fine_off[-1]], np.int32)]
            elif name == "CH_LIST" and fine_off is not None:
                parts = [p + fine_off[m] for m, p in enumerate(parts)]
            elif name in ("A_OFF", "B_OFF"):
                parts = [p[:-1] + eoff[m] for m, p in enumerate(parts)] + [np.array([eoff[-1]], np.int32)]
            elif name == "B_LIST":
                parts = [p + eoff[m] for m, p in enumerate(parts)]
            parts = [p for p in parts if p.size]
            want = np.concatenate(parts) if parts else np.empty(0, TABLES[t][1])
            got = table(batch, l, t)
            assert got.shape == want.shape, (l, name)
            np.testing.assert_array_equal(got, want.astype(got.dtype), err_msg=f"level {l} table {name}")
    for s in singles:
        s.close()
    batch.close()
