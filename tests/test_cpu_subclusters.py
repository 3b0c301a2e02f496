"""Host side of sub-cluster / branch detection: the core graph of a cluster
(core_graph.py:19 knn_mst_union + :47 flatten_to_csr) against the
reference's own graph stored in the fixtures."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = ["sc_branches_flares", "sc_branches_flares_leaf", "sc_lens_x_propagate"]


@pytest.mark.parametrize("name", CASES)
def test_core_graph_matches_reference(name):
    from fast_hdbscan_gb300.core_graph import core_graph_to_edge_list, knn_mst_union

    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    ours = knn_mst_union(g["cg_neighbors"], g["cg_core"], g["cg_mst"], g["cg_lens"])
    assert np.array_equal(ours.indptr, g["cg_indptr"])
    n = len(ours.indptr) - 1
    rows = np.repeat(np.arange(n), np.diff(g["cg_indptr"]))
    ref = sorted(zip(rows.tolist(), g["cg_indices"].tolist(), g["cg_weights"].tolist(),
                     g["cg_distances"].tolist()))
    mine = sorted(map(tuple, core_graph_to_edge_list(ours).tolist()))
    mine = [(int(a), int(b), float(c), float(d)) for a, b, c, d in mine]
    assert mine == [(int(a), int(b), float(c), float(d)) for a, b, c, d in ref]
    # rows sorted by weight
    for i in range(n):
        w = ours.weights[ours.indptr[i]:ours.indptr[i + 1]]
        assert np.all(np.diff(w) >= 0)


def test_branch_threshold_and_label_merge():
    """branches.py:14 and sub_clusters.py:98 on a hand-made two-cluster case."""
    from fast_hdbscan_gb300.branches import apply_branch_threshold
    from fast_hdbscan_gb300.sub_clusters import update_labels

    pts = [np.array([0, 1, 2, 3]), np.array([4, 5, 6])]
    sub = [np.array([0, 1, 2, -1]), np.array([0, 0, 0])]
    probs = [np.ones(4, np.float32), np.full(3, 0.5, np.float32)]
    lens = [np.arange(4, dtype=np.float32), np.arange(3, dtype=np.float32)]
    cp = np.full(7, 0.8, np.float32)
    labels, p, sl, sp, lv = update_labels(cp, sub, probs, lens, pts, 7)
    assert labels.tolist() == [1, 2, 3, 0, 4, 4, 4]
    assert np.allclose(p, [0.9, 0.9, 0.9, 0.9, 0.65, 0.65, 0.65])
    apply_branch_threshold(labels, sl, p, cp, pts, [np.zeros((3, 4)), np.zeros((2, 4))])
    # three branches in the first cluster stay; one in the second merges to one label
    assert labels.tolist() == [1, 2, 3, 0, 4, 4, 4]
    assert np.allclose(p[4:], 0.8)


CG_CASES = ["cg_float_400", "cg_int_400", "cg_neg_300", "cg_sparse_300", "cg_disconnected_300"]


@pytest.mark.parametrize("name", CG_CASES)
def test_core_graph_and_oracle_forest_match_reference(name):
    """The host core graph and the restated Boruvka (the checker of the GPU
    forest) against the reference's own graph and forest (core_graph.py:198),
    including empty rows, integer lens (ties) and a disconnected graph."""
    from fast_hdbscan_gb300.core_graph import knn_mst_union
    from oracle import core_graph_boruvka as CB

    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    ours = knn_mst_union(g["nb"], g["core"], g["mst"], g["lens"])
    np.testing.assert_array_equal(ours.indptr, g["indptr"])
    np.testing.assert_array_equal(ours.indices, g["indices"])
    np.testing.assert_array_equal(ours.weights, g["weights"])
    np.testing.assert_array_equal(ours.distances, g["distances"])
    nc, comp, edges = CB.boruvka_mst(g["weights"], g["indices"], g["indptr"])
    assert nc == int(g["n_components"])
    np.testing.assert_array_equal(edges, g["edges"])
    np.testing.assert_array_equal(comp, g["components"])


def test_root_labels_follow_union_by_rank():
    """A disconnected core graph's component labels: the reference's union-by-
    rank roots (disjoint_set.py:30) numbered in root order, from the forest's
    edges in order -- the same roots the restated Boruvka keeps."""
    from fast_hdbscan_gb300.core_graph import _root_labels
    from oracle import core_graph_boruvka as CB

    g = np.load(os.path.join(GOLDEN, "cg_disconnected_300.npz"))
    labels = _root_labels(len(g["indptr"]) - 1, g["edges"])
    np.testing.assert_array_equal(labels, np.unique(g["components"], return_inverse=True)[1])
    _, comp, _ = CB.boruvka_mst(g["weights"], g["indices"], g["indptr"])
    np.testing.assert_array_equal(comp, g["components"])


def reference_noise_dicts(graph, sub_labels):
    """sub_clusters.py:134-142 restated as the test's checker: the per-point
    dict of neighbours (insertion order, last value wins) of every noise
    point."""
    n = len(sub_labels)
    und = [dict() for _ in range(n)]
    for idx in range(n):
        for i in range(graph.indptr[idx], graph.indptr[idx + 1]):
            nb = int(graph.indices[i])
            w = 1.0 / float(graph.weights[i])
            if sub_labels[nb] == -1:
                und[nb][idx] = w
            if sub_labels[idx] == -1:
                und[idx][nb] = w
    return und


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_noise_adjacency_in_dict_order(seed):
    """The propagation's host layout lists every noise point's neighbours in
    the reference's dict order with the dict's values."""
    from fast_hdbscan_gb300.core_graph import CoreGraph
    from fast_hdbscan_gb300.sub_clusters import _noise_adjacency

    rng = np.random.default_rng(seed)
    n = 60
    rows = [sorted(rng.choice(n, rng.integers(0, 6), replace=False).tolist()) for _ in range(n)]
    if seed == 3:  # repeated pairs in both directions
        rows = [r + r[:1] for r in rows]
    ws = [rng.integers(1, 5, len(r)).astype(np.float32).tolist() for r in rows]
    indptr = np.cumsum([0] + [len(r) for r in rows]).astype(np.int32)
    g = CoreGraph(np.array(sum(ws, []), np.float32), np.zeros(indptr[-1], np.float32),
                  np.array(sum(rows, []), np.int32), indptr)
    sub = rng.integers(-1, 3, n)
    pts, counts, other, w = _noise_adjacency(g, sub, 100)
    want = reference_noise_dicts(g, sub)
    np.testing.assert_array_equal(pts - 100, np.nonzero(sub == -1)[0])
    at = 0
    for p, c in zip(pts - 100, counts):
        got = list(zip((other[at:at + c] - 100).tolist(), w[at:at + c].tolist()))
        assert got == list(want[p].items())
        at += c


def _cycle_rule_forest(weights, indices, indptr):
    """The GPU forest's round, restated in Python: candidates by (weight,
    point) per component, the functional graph of candidates, each cycle's
    largest-order edge dropped, the rest emitted in order (coregraph.cu)."""
    n = len(indptr) - 1
    w, idx = np.asarray(weights, np.float32), np.asarray(indices)
    comp, ptr = np.arange(n), np.array(indptr[:-1])
    own = np.array([next((r for r in range(p, n) if indptr[r + 1] > indptr[r]), -1)
                    for p in range(n)])
    out, first = [], True
    while True:
        if not first:
            for p in range(n):
                while ptr[p] < indptr[p + 1] and comp[idx[ptr[p]]] == comp[p]:
                    ptr[p] += 1
        first = False
        best, pos = {}, {}
        for p in range(n):
            r = own[p]
            if r < 0 or ptr[r] >= indptr[r + 1]:
                continue
            c, key = comp[p], (w[ptr[r]], p)
            if c not in best or key < best[c]:
                best[c] = key
            pos[c] = min(pos.get(c, n), p)
        succ = {c: comp[idx[ptr[own[p]]]] for c, (_, p) in best.items()}
        drop, seen = set(), {}
        for c in best:
            path, x = [], c
            while x in succ and x not in seen:
                seen[x] = c
                path.append(x)
                x = succ[x]
            if x in succ and seen.get(x) == c:
                cyc = path[path.index(x):]
                drop.add(max(cyc, key=lambda v: pos[v]))
        keep = sorted((c for c in best if c not in drop), key=lambda c: pos[c])
        if not keep:
            break
        par = {}

        def find(x):
            while par.get(x, x) != x:
                x = par[x]
            return x

        for c in keep:
            p = best[c][1]
            e = ptr[own[p]]
            out.append((float(p), float(idx[e]), float(w[e])))
            a, b = find(c), find(comp[idx[e]])
            par[max(a, b)] = min(a, b)
        comp = np.array([find(comp[p]) for p in range(n)])
    return np.array(out, dtype=np.float64).reshape(-1, 3)


@pytest.mark.parametrize("name", CG_CASES)
def test_cycle_rule_equals_sequential_merge(name):
    """Dropping each candidate cycle's largest-order edge (the GPU round) gives
    the reference's sequential union-find merge edge for edge."""
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    ours = _cycle_rule_forest(g["weights"], g["indices"], g["indptr"])
    np.testing.assert_array_equal(ours, g["edges"])


@pytest.mark.parametrize("seed", range(4))
def test_cluster_layout_equals_per_cluster_slices(seed):
    """cluster_layout (torch passes; CPU tensors here) cuts every cluster's
    points, in-cluster kNN ids and in-cluster MST edges exactly as slicing one
    cluster at a time does (sub_clusters.py:16-61)."""
    from fast_hdbscan_gb300.sub_clusters import cluster_layout

    rng = np.random.default_rng(seed)
    n, k, ncl = 3000, 7, 9
    labels = rng.integers(-1, ncl, size=n)
    nbrs = rng.integers(-1, n, size=(n, k)).astype(np.int32)
    parent = np.array([rng.integers(0, i) for i in range(1, n)])
    mst = np.stack([np.arange(1, n), parent, rng.random(n - 1)], axis=1)[rng.permutation(n - 1)]
    points, bounds, nb_local, mst_local, mst_bounds = cluster_layout(labels, ncl, nbrs, mst,
                                                                      device="cpu")
    for c in range(ncl):
        pts = np.nonzero(labels == c)[0]
        np.testing.assert_array_equal(points[bounds[c]:bounds[c + 1]], pts)
        local = {p: i for i, p in enumerate(pts)}
        want = np.array([[local.get(q, -1) if q >= 0 else -1 for q in row] for row in nbrs[pts]],
                        dtype=np.int32).reshape(-1, k)
        np.testing.assert_array_equal(nb_local[bounds[c]:bounds[c + 1]], want)
        rows = [(local[a], local[b], w) for a, b, w in mst
                if labels[int(a)] == c and labels[int(b)] == c]
        got = mst_local[mst_bounds[c]:mst_bounds[c + 1]]
        np.testing.assert_array_equal(got, np.array(rows, dtype=np.float64).reshape(-1, 3))
    assert nb_local.dtype == np.int32 and mst_local.dtype == np.float64
