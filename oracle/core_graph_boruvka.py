"""Restatement of the reference's core-graph Boruvka -- TEST INFRASTRUCTURE ONLY.

Only the tests use this module, as the checker of the GPU core-graph forest;
the product library never imports it.  It follows core_graph.py:198
boruvka_mst on a CoreGraph whose rows are sorted by weight:

* select_components (:104): points in index order; a point's candidate is
  the first entry of its row (entries inside its own component have been
  removed); a component keeps the first point's candidate with the strictly
  smallest weight; components are kept in order of first insertion.
* merge_components (:126): the candidates in that order, each added when its
  ends are still in different components (union by rank).
* update_graph_components (:143): rows drop the entries that now point into
  their own component, keeping order.

Returns ``(n_components, point_components, edges float64[m, 3])`` like the
reference (component ids are the union-find roots).
"""
import numpy as np


def _find(parent, x):
    while parent[x] != x:
        parent[x] = parent[parent[x]]
        x = parent[x]
    return x


def boruvka_mst(weights, indices, indptr):
    n = len(indptr) - 1
    w = np.array(weights, dtype=np.float32)
    idx = np.array(indices, dtype=np.int64)
    parent = np.arange(n)
    rank = np.zeros(n, np.int64)
    comp = np.arange(n)
    n_components = n
    out = []
    while n_components > 1:
        best = {}
        for p in range(n):
            s = indptr[p]
            if s == len(idx) or idx[s] == -1:
                continue
            c = comp[p]
            if c not in best or w[s] < best[c][2]:
                best[c] = (p, int(idx[s]), float(w[s]))
        new = []
        for a, b, d in best.values():
            ra, rb = _find(parent, a), _find(parent, b)
            if ra != rb:
                new.append((float(a), float(b), d))
                if rank[ra] < rank[rb]:
                    parent[ra] = rb
                elif rank[ra] > rank[rb]:
                    parent[rb] = ra
                else:
                    parent[rb] = ra
                    rank[ra] += 1
        if not new:
            break
        out += new
        comp = np.array([_find(parent, i) for i in range(n)])
        for p in range(n):
            s, e = indptr[p], indptr[p + 1]
            row_i, row_w = idx[s:e], w[s:e]
            keep = (row_i != -1)
            keep[keep] = comp[row_i[keep]] != comp[p]
            k = int(keep.sum())
            idx[s:s + k], w[s:s + k] = row_i[keep], row_w[keep]
            idx[s + k:e], w[s + k:e] = -1, np.inf
        n_components -= len(new)
    return n_components, comp, np.array(out, dtype=np.float64).reshape(-1, 3)
