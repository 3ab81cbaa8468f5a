"""Seeded irregular multigrid meshes for the tests (not lattices).

Every level has random node positions and three random edges per node, plus
parallel edges (the same pair twice) and reversed copies; about a tenth of the
nodes carry one or two boundary entries whose groups cover 0..9 (0-2 wall,
3-7 far field, 8-9 ignored by compute_bnd_node_flux_kernel, flux.h:14-39);
the fine-to-coarse map leaves about a tenth of the coarse nodes without
children (mg.h:29-64 keeps their state)."""
import numpy as np

import mgcfd


def irregular_levels(n0=1500, nlevels=3, seed=0):
    rng = np.random.default_rng(seed)
    ns = [n0]
    for _ in range(1, nlevels):
        ns.append(max(12, ns[-1] // 4))
    levels = []
    for l, n in enumerate(ns):
        coords = rng.random((n, 3))
        a = np.repeat(np.arange(n), 3)
        b = rng.integers(0, n, len(a))
        b = np.where(b == a, (b + 1) % n, b)
        e = np.stack([a, b], 1)
        e = np.concatenate([e, e[rng.choice(len(e), len(e) // 20)], e[rng.choice(len(e), len(e) // 20)][:, ::-1]])
        e = e[rng.permutation(len(e))]
        h = n ** (-1.0 / 3.0)
        d = coords[e[:, 1]] - coords[e[:, 0]]
        w = h * h * d / np.linalg.norm(d, axis=1, keepdims=True) * rng.uniform(0.5, 1.5, (len(e), 1))
        bn = rng.choice(n, max(1, n // 10), replace=False)
        bn = np.concatenate([bn, bn[: len(bn) // 3]])
        bn = bn[rng.permutation(len(bn))]
        grp = rng.integers(0, 10, len(bn))
        bw = rng.normal(size=(len(bn), 3)) * h * h
        n2mg = None
        if l + 1 < len(ns):
            used = rng.choice(ns[l + 1], max(1, (ns[l + 1] * 9) // 10), replace=False)
            n2mg = used[rng.integers(0, len(used), n)].astype(np.int32)
        levels.append(mgcfd.Level(coords=np.ascontiguousarray(coords), edge_to_nodes=e.astype(np.int32),
                                  bnd_to_node=bn.astype(np.int32), bnd_group=grp.astype(np.int32),
                                  edge_weights=np.ascontiguousarray(w), bnd_weights=np.ascontiguousarray(bw),
                                  node_to_mg=n2mg))
    return levels
