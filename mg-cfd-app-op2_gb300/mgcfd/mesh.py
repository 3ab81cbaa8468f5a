"""Host meshes: synthetic lattices or input.dat + HDF5 decks (euler3d.cpp:243-336)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib


@dataclass
class Level:
    """One multigrid level as numpy arrays in file order (0-based maps)."""
    coords: np.ndarray         # [N,3] f64
    edge_to_nodes: np.ndarray  # [E,2] i32
    bnd_to_node: np.ndarray    # [B]   i32
    bnd_group: np.ndarray      # [B]   i32
    edge_weights: np.ndarray   # [E,3] f64
    bnd_weights: np.ndarray    # [B,3] f64
    node_to_mg: np.ndarray | None  # [N] i32 into the next level
    n_axis: int = 0
    volumes: np.ndarray | None = None  # [N] legacy-mode volumes ("areas"), else computed
    owner: object = field(default=None, repr=False, compare=False)  # keeps zero-copy views' memory alive

    @property
    def nnodes(self) -> int:
        return int(self.coords.shape[0])

    @property
    def nedges(self) -> int:
        return int(self.edge_to_nodes.shape[0])

    @property
    def nbnd(self) -> int:
        return int(self.bnd_to_node.shape[0])


def _view(ptr, shape, dtype):
    n = int(np.prod(shape))
    if n == 0:
        return np.zeros(shape, dtype=dtype)
    ctype = C.c_double if dtype == np.float64 else C.c_int32
    buf = (ctype * n).from_address(C.cast(ptr, C.c_void_p).value)
    return np.frombuffer(buf, dtype=dtype).reshape(shape)


RENUMBER_METHODS = {"none": 0, "spatial": 1, "rcm": 2}


def renumber_nodes(method: str, coords: np.ndarray, edge_to_nodes: np.ndarray | None = None) -> np.ndarray:
    """perm[new] = old for one node set (mgcfd_renumber_nodes)."""
    lib = _lib.load()
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    e2n = np.ascontiguousarray(edge_to_nodes if edge_to_nodes is not None else np.zeros((0, 2)), dtype=np.int32)
    perm = np.empty(len(coords), dtype=np.int32)
    _lib.check(lib.mgcfd_renumber_nodes(RENUMBER_METHODS[method], len(coords), coords.ctypes.data_as(_lib.c_double_p),
                                        len(e2n), e2n.ctypes.data_as(_lib.c_int32_p),
                                        perm.ctypes.data_as(_lib.c_int32_p)))
    return perm


class HostMesh:
    """Owner of a native mgcfd_host_mesh; level arrays are zero-copy views."""

    _next_serial = 1

    def __init__(self, handle):
        self._h = handle
        self._lib = _lib.load()
        # Process-unique identity, used as the server's resident-mesh key.
        self.serial = HostMesh._next_serial
        HostMesh._next_serial += 1

    @classmethod
    def generate(cls, n: int, nlevels: int, seed: int) -> "HostMesh":
        lib = _lib.load()
        h = C.c_void_p()
        _lib.check(lib.mgcfd_host_mesh_generate(n, nlevels, seed, C.byref(h)))
        return cls(h)

    @classmethod
    def load(cls, input_file: str, input_dir: str | None = None, legacy: bool = False) -> "HostMesh":
        lib = _lib.load()
        h = C.c_void_p()
        _lib.check(lib.mgcfd_host_mesh_load(input_file.encode(), (input_dir or "").encode(), int(legacy),
                                            C.byref(h)))
        return cls(h)

    @classmethod
    def from_levels(cls, levels) -> "HostMesh":
        """A host mesh copied from a list of Level arrays (mgcfd_host_mesh_from_views)."""
        lib = _lib.load()
        views = level_views_from_arrays(levels)
        h = C.c_void_p()
        _lib.check(lib.mgcfd_host_mesh_from_views(len(levels), views, C.byref(h)))
        return cls(h)

    def write(self, directory: str, prefix: str = "mesh_", legacy_datasets: bool = False) -> None:
        _lib.check(self._lib.mgcfd_host_mesh_write(self._h, str(directory).encode(), prefix.encode(),
                                                   int(legacy_datasets)))

    def renumber(self, method: str = "spatial") -> "HostMesh":
        """A relabelled copy of the mesh (mgcfd_host_mesh_renumber): nodes in
        Morton ("spatial") or reverse Cuthill-McKee ("rcm") order on every level."""
        h = C.c_void_p()
        _lib.check(self._lib.mgcfd_host_mesh_renumber(self._h, RENUMBER_METHODS[method], C.byref(h)))
        return HostMesh(h)

    @property
    def num_levels(self) -> int:
        return self._lib.mgcfd_host_mesh_num_levels(self._h)

    def level_view(self, l: int) -> _lib.LevelView:
        v = _lib.LevelView()
        _lib.check(self._lib.mgcfd_host_mesh_level(self._h, l, C.byref(v)))
        return v

    def level_views(self):
        arr = (_lib.LevelView * self.num_levels)()
        for l in range(self.num_levels):
            arr[l] = self.level_view(l)
        return arr

    def level(self, l: int) -> Level:
        v = self.level_view(l)
        n2mg = _view(v.node_to_mg, (v.nnodes,), np.int32) if v.node_to_mg else None
        vols = _view(v.volumes, (v.nnodes,), np.float64) if v.volumes else None
        return Level(coords=_view(v.coords, (v.nnodes, 3), np.float64),
                     edge_to_nodes=_view(v.edge_to_nodes, (v.nedges, 2), np.int32),
                     bnd_to_node=_view(v.bnd_to_node, (v.nbnd,), np.int32),
                     bnd_group=_view(v.bnd_group, (v.nbnd,), np.int32),
                     edge_weights=_view(v.edge_weights, (v.nedges, 3), np.float64),
                     bnd_weights=_view(v.bnd_weights, (v.nbnd, 3), np.float64),
                     node_to_mg=n2mg, n_axis=v.n_axis, volumes=vols, owner=self)

    def levels(self):
        return [self.level(l) for l in range(self.num_levels)]

    def close(self):
        if self._h:
            self._lib.mgcfd_host_mesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def level_views_from_arrays(levels):
    """Build a LevelView array over numpy Level objects (caller keeps them alive)."""
    arr = (_lib.LevelView * len(levels))()
    for i, L in enumerate(levels):
        v = arr[i]
        v.nnodes, v.nedges, v.nbnd, v.n_axis = L.nnodes, L.nedges, L.nbnd, L.n_axis
        v.coords = L.coords.ctypes.data_as(_lib.c_double_p)
        v.edge_to_nodes = L.edge_to_nodes.ctypes.data_as(_lib.c_int32_p)
        v.bnd_to_node = L.bnd_to_node.ctypes.data_as(_lib.c_int32_p)
        v.bnd_group = L.bnd_group.ctypes.data_as(_lib.c_int32_p)
        v.edge_weights = L.edge_weights.ctypes.data_as(_lib.c_double_p)
        v.bnd_weights = L.bnd_weights.ctypes.data_as(_lib.c_double_p)
        v.node_to_mg = L.node_to_mg.ctypes.data_as(_lib.c_int32_p) if L.node_to_mg is not None else None
        v.volumes = L.volumes.ctypes.data_as(_lib.c_double_p) if L.volumes is not None else None
    return arr


def h5_read(path: str, name: str) -> np.ndarray:
    lib = _lib.load()
    dims = (C.c_int64 * 2)()
    rank = C.c_int()
    _lib.check(lib.mgcfd_h5_dataset_shape(str(path).encode(), name.encode(), dims, C.byref(rank)))
    shape = (dims[0],) if rank.value < 2 else (dims[0], dims[1])
    out = np.empty(shape, dtype=np.float64)
    _lib.check(lib.mgcfd_h5_read_f64(str(path).encode(), name.encode(), out.ctypes.data_as(_lib.c_double_p),
                                     out.size))
    return out


def freestream(mach: float, aoa_deg: float) -> _lib.Freestream:
    lib = _lib.load()
    ff = _lib.Freestream()
    _lib.check(lib.mgcfd_freestream_init(mach, aoa_deg, C.byref(ff)))
    return ff
