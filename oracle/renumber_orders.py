"""Oracle for mesh renumbering (test infrastructure only; never shipped).

The reference's renumbering (-n, op_renumber(p_edge_to_nodes[0]) at
euler3d.cpp:377) runs Scotch inside OP2-Common.  Neither is vendored in the
reference tree (OP2-Common is an un-vendored build dependency; the Scotch
version is whatever OP2 was linked against), so its exact order cannot be
reproduced and is not the target.  What the reference fixes is the contract:
renumbering is a relabelling of the node set, and the solution it produces is
the same solution, permuted, up to the rounding of the changed loop order.
The tests pin that contract against the reference binary itself
(tests/test_renumber.py).

This file restates, independently of the C++ product, the two orders the
product offers, so that the integer work is checked bit for bit:

  * morton_order: coordinates quantised to 21 bits per axis inside the
    bounding box, bits interleaved x-lowest (key = ..z1y1x1z0y0x0), nodes
    sorted by key, ties in input order;
  * rcm_order: reverse Cuthill-McKee; each connected component (taken in
    order of its lowest node id) starts from the node returned by two
    breadth-first sweeps (farthest node, lowest degree among the farthest),
    neighbours are visited by ascending (degree, id), and the whole
    sequence is reversed.
"""
from __future__ import annotations

from collections import deque

import numpy as np

Q_MAX = 2097151.0  # 2^21 - 1


def _spread3(q: np.ndarray) -> np.ndarray:
    out = np.zeros_like(q, dtype=np.uint64)
    for bit in range(21):
        out |= ((q >> np.uint64(bit)) & np.uint64(1)) << np.uint64(3 * bit)
    return out


def morton_order(coords: np.ndarray) -> np.ndarray:
    xyz = np.asarray(coords, dtype=np.float64).reshape(-1, 3)
    lo = xyz.min(axis=0)
    hi = xyz.max(axis=0)
    span = hi - lo
    with np.errstate(divide="ignore", invalid="ignore"):
        scale = np.where((hi > lo) & np.isfinite(span), Q_MAX / np.where(span > 0, span, 1.0), 0.0)
    t = (xyz - lo) * scale
    t = np.where(t > 0.0, t, 0.0)  # also maps NaN to 0
    t = np.minimum(t, Q_MAX)
    q = t.astype(np.uint64)
    key = (_spread3(q[:, 2]) << np.uint64(2)) | (_spread3(q[:, 1]) << np.uint64(1)) | _spread3(q[:, 0])
    return np.argsort(key, kind="stable").astype(np.int32)


def rcm_order(nnodes: int, edge_to_nodes: np.ndarray) -> np.ndarray:
    e2n = np.asarray(edge_to_nodes, dtype=np.int64).reshape(-1, 2)
    deg = np.zeros(nnodes, dtype=np.int64)
    np.add.at(deg, e2n[:, 0], 1)
    np.add.at(deg, e2n[:, 1], 1)
    adj = [[] for _ in range(nnodes)]
    for a, b in e2n.tolist():
        adj[a].append(b)
        adj[b].append(a)
    for u in range(nnodes):
        adj[u].sort(key=lambda v: (deg[v], v))

    def farthest(s):
        level = {s: 0}
        q = deque([s])
        last = s
        while q:
            u = q.popleft()
            if level[u] > level[last] or (level[u] == level[last] and deg[u] < deg[last]):
                last = u
            for v in adj[u]:
                if v not in level:
                    level[v] = level[u] + 1
                    q.append(v)
        return last

    seen = np.zeros(nnodes, dtype=bool)
    order = []
    for s0 in range(nnodes):
        if seen[s0]:
            continue
        s = farthest(farthest(s0))
        seen[s] = True
        q = deque([s])
        while q:
            u = q.popleft()
            order.append(u)
            for v in adj[u]:
                if not seen[v]:
                    seen[v] = True
                    q.append(v)
    return np.array(order[::-1], dtype=np.int32)


def relabel(level: dict, perm: np.ndarray, perm_next: np.ndarray | None) -> dict:
    """The relabelled level for perm (perm[new] = old) and the next coarser
    level's perm (None on the coarsest level)."""
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm), dtype=perm.dtype)
    e = inv[level["edge_to_nodes"]]
    eorder = np.lexsort((e.max(axis=1), e.min(axis=1)))  # stable: primary min, then max
    border = np.argsort(inv[level["bnd_to_node"]], kind="stable")
    out = {"coords": level["coords"][perm], "edge_to_nodes": e[eorder],
           "edge_weights": level["edge_weights"][eorder], "bnd_to_node": inv[level["bnd_to_node"]][border],
           "bnd_group": level["bnd_group"][border], "bnd_weights": level["bnd_weights"][border]}
    if perm_next is not None and level.get("node_to_mg") is not None:
        inv_next = np.empty_like(perm_next)
        inv_next[perm_next] = np.arange(len(perm_next), dtype=perm_next.dtype)
        out["node_to_mg"] = inv_next[level["node_to_mg"][perm]]
    return out
