"""Synthetic jittered-lattice meshes: sizes, ids, maps and determinism (CPU)."""
import numpy as np
import pytest

import mgcfd


@pytest.mark.parametrize("n,nl", [(6, 3), (9, 3), (13, 2), (24, 4)])
def test_structure(n, nl):
    mesh = mgcfd.HostMesh.generate(n, nl, 31)
    levels = mesh.levels()
    m = n
    for l, L in enumerate(levels):
        assert L.n_axis == m
        assert L.nnodes == m ** 3
        assert L.nedges == 3 * m * m * (m - 1)
        # one boundary entry per (node, face): 6 faces of m^2 nodes
        assert L.nbnd == 6 * m * m
        assert np.array_equal(np.sort(L.edge_to_nodes.reshape(-1)) >= 0, np.ones(2 * L.nedges, bool))
        assert L.edge_to_nodes.max() < L.nnodes
        assert (L.edge_to_nodes[:, 0] != L.edge_to_nodes[:, 1]).all()
        # every node has degree 3..6 on a lattice
        deg = np.bincount(L.edge_to_nodes.reshape(-1), minlength=L.nnodes)
        assert deg.min() == 3 and deg.max() == (6 if m > 2 else 3)
        # groups: 0 on z = 0 (one face), 3 elsewhere
        assert set(np.unique(L.bnd_group)) == {0, 3}
        assert (L.bnd_group == 0).sum() == m * m
        # weights: |w| = h_l^2 for edges and boundary entries
        h = (1.0 / (n - 1)) * 2 ** l
        np.testing.assert_allclose(np.linalg.norm(L.edge_weights, axis=1), h * h, rtol=1e-12)
        np.testing.assert_allclose(np.linalg.norm(L.bnd_weights, axis=1), h * h, rtol=1e-12)
        # wall normals point out of the domain at z = 0
        wall = L.bnd_group == 0
        assert np.all(L.bnd_weights[wall, 2] < 0)
        assert np.allclose(L.coords[L.bnd_to_node[wall], 2], 0.0)
        if l + 1 < nl:
            c = L.node_to_mg
            assert c.min() >= 0 and c.max() < levels[l + 1].nnodes
            assert np.bincount(c, minlength=levels[l + 1].nnodes).min() >= 1  # every coarse node has a child
        m = (m + 1) // 2


def test_coarse_nodes_reuse_fine_coordinates():
    mesh = mgcfd.HostMesh.generate(10, 2, 3)
    F, Cl = mesh.level(0), mesh.level(1)
    fine = {tuple(x) for x in F.coords}
    assert all(tuple(x) in fine for x in Cl.coords)


def test_jitter_only_in_interior():
    n = 12
    L = mgcfd.HostMesh.generate(n, 1, 9).level(0)
    h = 1.0 / (n - 1)
    on_lattice = np.all(np.abs(L.coords / h - np.round(L.coords / h)) < 1e-9, axis=1)
    boundary = np.any((L.coords < 1e-12) | (L.coords > 1 - 1e-12), axis=1)
    assert on_lattice[boundary].all()
    assert (~on_lattice[~boundary]).mean() > 0.99
    assert np.abs(L.coords / h - np.round(L.coords / h)).max() <= 0.2 + 1e-9


def test_deterministic_and_seed_dependent():
    a = mgcfd.HostMesh.generate(9, 2, 5).level(0)
    b = mgcfd.HostMesh.generate(9, 2, 5).level(0)
    c = mgcfd.HostMesh.generate(9, 2, 6).level(0)
    assert np.array_equal(a.coords, b.coords) and np.array_equal(a.edge_to_nodes, b.edge_to_nodes)
    assert not np.array_equal(a.edge_to_nodes, c.edge_to_nodes)


def test_invalid_sizes_are_rejected():
    with pytest.raises(mgcfd._lib.MgcfdError):
        mgcfd.HostMesh.generate(1, 1, 0)
    with pytest.raises(mgcfd._lib.MgcfdError):
        mgcfd.HostMesh.generate(4, 4, 0)  # 4 -> 2 -> 1 node per axis
