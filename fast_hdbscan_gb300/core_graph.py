"""Core graphs of clusters for sub-cluster and branch detection
(core_graph.py of the reference).

A cluster's core graph joins each point to its in-cluster kNN neighbours and
to its in-cluster MST children; an edge's weight is the larger lens value of
its two ends and its distance the larger core distance (MST edges keep their
MST distance).  The graph is laid out on the host (a few numpy passes over
n * k entries, as cheap as the lens itself); its spanning forest
(``fhg_core_graph_mst``: the reference's Boruvka, including its choices
among the many equal lens weights, which shape the cluster hierarchy) and
the hierarchy's tree passes (``clusters_from_spanning_tree``) run on the GPU.

Rows are ordered by weight with ties in insertion order (the kNN children in
neighbour order, then the MST children): the order of the reference's sort
for rows of up to 15 entries, where its quicksort is an insertion sort.
"""
import ctypes
from collections import namedtuple

import numpy as np

from . import _native
from .cluster_trees import empty_condensed_tree

CoreGraph = namedtuple("CoreGraph", ["weights", "distances", "indices", "indptr"])


def knn_mst_union(neighbors, core_distances, min_spanning_tree, lens_values):
    """core_graph.py:19 knn_mst_union + :47 flatten_to_csr + :70 sort_by_lens:
    the core graph as CSR rows sorted by weight (ties keep insertion order:
    the kNN children in neighbour order, then the MST children)."""
    n = len(core_distances)
    lens = np.asarray(lens_values)
    core = np.asarray(core_distances)
    nb = np.asarray(neighbors).reshape(n, -1)
    k = nb.shape[1]
    valid = nb >= 0
    # a child enters a row once (the reference's per-row dict keeps the first)
    if k > 1:
        srt = np.sort(nb, axis=1)
        if np.any((srt[:, 1:] == srt[:, :-1]) & (srt[:, 1:] >= 0)):
            for j in range(1, k):
                valid[:, j] &= ~np.any(nb[:, :j] == nb[:, j:j + 1], axis=1)
    rows_k, jk = np.nonzero(valid)  # row-major: each row's children in neighbour order
    cols_k = nb[rows_k, jk].astype(np.int64)
    w_k = np.maximum(lens[rows_k], lens[cols_k])
    d_k = np.maximum(core[rows_k], core[cols_k])
    mst = np.asarray(min_spanning_tree, dtype=np.float64).reshape(-1, 3)
    rows_m = mst[:, 0].astype(np.int64)
    cols_m = mst[:, 1].astype(np.int64)
    new = ~np.any(nb[rows_m] == cols_m[:, None], axis=1) if k > 0 else np.ones(len(rows_m), bool)
    keys_m = rows_m * n + cols_m
    if len(np.unique(keys_m)) != len(keys_m):  # repeated MST pairs: the first counts
        _, first = np.unique(keys_m, return_index=True)
        once = np.zeros(len(keys_m), bool)
        once[first] = True
        new &= once
    rows_m, cols_m, d_m = rows_m[new], cols_m[new], mst[new, 2]
    w_m = np.maximum(lens[rows_m], lens[cols_m])
    rows = np.concatenate([rows_k, rows_m])
    cols = np.concatenate([cols_k, cols_m])
    weights = np.concatenate([w_k, w_m]).astype(np.float32)
    distances = np.concatenate([d_k, d_m]).astype(np.float32)
    order = np.lexsort((weights, rows))  # by row, then weight, stable
    indptr = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(np.bincount(rows, minlength=n), out=indptr[1:])
    return CoreGraph(weights[order], distances[order], cols[order].astype(np.int32), indptr)


def _root_labels(n, edges):
    """The reference's component labels for a disconnected core graph: the
    union-by-rank roots (disjoint_set.py:30, edges merged in forest order),
    numbered in increasing root order (core_graph.py:251)."""
    parent = np.arange(n)
    rank = np.zeros(n, np.int64)

    def find(x):
        while parent[x] != x:
            x = parent[x]
        return x

    for a, b in edges[:, :2].astype(np.int64):
        x, y = find(a), find(b)
        if x == y:
            continue
        if rank[x] < rank[y]:
            x, y = y, x
        parent[y] = x
        if rank[x] == rank[y]:
            rank[x] += 1
    roots = np.array([find(i) for i in range(n)])
    return np.unique(roots, return_inverse=True)[1].astype(np.int64)


def core_graph_spanning_tree(neighbors, core_distances, min_spanning_tree, lens):
    """core_graph.py:234: ``(n_components, component_labels, lensed_mst,
    graph)`` -- the core graph's spanning forest on its lens weights, built on
    the GPU with the reference's Boruvka choices (``fhg_core_graph_mst``)."""
    torch = _native._torch()
    graph = knn_mst_union(neighbors, core_distances, min_spanning_tree, lens)
    n = len(graph.indptr) - 1
    if np.any(np.isnan(graph.weights)):
        raise ValueError("lens values must not be NaN")
    if n <= 1:
        return n, np.zeros(n, np.int64), np.zeros((0, 3)), graph
    V = _native.vptr
    d_indptr = torch.from_numpy(np.ascontiguousarray(graph.indptr, np.int32)).cuda()
    d_indices = torch.from_numpy(np.ascontiguousarray(graph.indices, np.int32)).cuda()
    d_weights = torch.from_numpy(np.ascontiguousarray(graph.weights, np.float32)).cuda()
    edges = torch.empty((n - 1, 3), dtype=torch.float64, device="cuda")
    m = ctypes.c_int64(0)
    _native.check(_native.load().fhg_core_graph_mst(V(d_indptr), V(d_indices), V(d_weights),
                                                    None, n, V(edges), ctypes.byref(m),
                                                    _native.stream_ptr()))
    forest = edges[: m.value].cpu().numpy()
    nc = n - int(m.value)
    if nc <= 1:
        return 1, np.zeros(n, np.int64), forest, graph
    return nc, _root_labels(n, forest), forest, graph


def core_graph_forests(graphs):
    """Spanning forests of several core graphs in one GPU launch (their rows
    as disjoint blocks of one CSR): ``[(n_components, component_labels,
    forest), ...]``, each as ``core_graph_spanning_tree`` returns it."""
    torch = _native._torch()
    sizes = np.array([len(g.indptr) - 1 for g in graphs], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    n = int(offs[-1])
    if n <= 1:
        return [(int(sz), np.zeros(int(sz), np.int64), np.zeros((0, 3))) for sz in sizes]
    nnz = np.concatenate([[0], np.cumsum([g.indptr[-1] for g in graphs])])
    indptr = np.concatenate([g.indptr[:-1].astype(np.int64) + nnz[i]
                             for i, g in enumerate(graphs)] + [[nnz[-1]]]).astype(np.int32)
    indices = np.concatenate([g.indices.astype(np.int64) + offs[i]
                              for i, g in enumerate(graphs)]).astype(np.int32)
    weights = np.concatenate([g.weights for g in graphs]).astype(np.float32)
    if np.any(np.isnan(weights)):
        raise ValueError("lens values must not be NaN")
    seg_end = np.repeat(offs[1:], sizes).astype(np.int32)
    V = _native.vptr
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    d_indptr, d_indices, d_weights, d_seg = T(indptr), T(indices), T(weights), T(seg_end)
    edges = torch.empty((n - 1, 3), dtype=torch.float64, device="cuda")
    m = ctypes.c_int64(0)
    _native.check(_native.load().fhg_core_graph_mst(V(d_indptr), V(d_indices), V(d_weights),
                                                    V(d_seg), n, V(edges), ctypes.byref(m),
                                                    _native.stream_ptr()))
    all_edges = edges[: m.value].cpu().numpy()
    owner = np.searchsorted(offs, all_edges[:, 0].astype(np.int64), side="right") - 1
    order = np.argsort(owner, kind="stable")
    bounds = np.searchsorted(owner[order], np.arange(len(graphs) + 1))
    out = []
    for i, sz in enumerate(sizes):
        f = all_edges[order[bounds[i]:bounds[i + 1]]].copy()
        f[:, :2] -= offs[i]
        nc = int(sz) - len(f)
        comp = np.zeros(int(sz), np.int64) if nc <= 1 else _root_labels(int(sz), f)
        out.append((max(nc, 1) if sz > 0 else 0, comp, f))
    return out


def core_graphs_and_forests(inputs):
    """Core graphs and spanning forests of many clusters on the GPU: ``inputs``
    is a list of ``(neighbors, core_distances, min_spanning_tree, lens)`` in
    in-cluster ids.  Returns ``[(graph, n_components, component_labels,
    forest), ...]`` as knn_mst_union and core_graph_spanning_tree give them."""
    sizes = np.array([len(c) for _, c, _, _ in inputs], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    P = int(offs[-1])
    k = max([np.asarray(nb).reshape(len(c), -1).shape[1] if len(c) else 0
             for nb, c, _, _ in inputs] + [0])
    nb_block = np.full((P, k), -1, dtype=np.int32)
    for i, (nb, c, _, _) in enumerate(inputs):
        if len(c):
            a = np.asarray(nb).reshape(len(c), -1)
            nb_block[offs[i]:offs[i + 1], :a.shape[1]] = a
    lens_block = np.concatenate([np.asarray(l, np.float64) for _, _, _, l in inputs] + [[]])
    core_block = np.concatenate([np.asarray(c, np.float32) for _, c, _, _ in inputs] + [[]])
    msts = [np.asarray(m, np.float64).reshape(-1, 3) for _, _, m, _ in inputs]
    mst_bounds = np.concatenate([[0], np.cumsum([len(m) for m in msts])])
    mst_local = np.concatenate(msts + [np.zeros((0, 3))])
    return core_graphs_and_forests_block(sizes, nb_block, lens_block, core_block, mst_local,
                                         mst_bounds)


def core_graphs_and_forests_block(sizes, nb_block, lens_block, core_block, mst_local,
                                  mst_bounds):
    """Core graphs and spanning forests of many clusters laid out back to back
    (cluster c's rows are the next sizes[c] rows of the blocks): nb_block
    (rows x k in-cluster neighbour ids, -1 for none), lens_block (float64),
    core_block, and the in-cluster MST edges mst_local[mst_bounds[c]:
    mst_bounds[c+1]] (in-cluster ids, distance).  The graphs are laid out as
    one block CSR (``fhg_core_graphs``) and their forests built in one launch
    (``fhg_core_graph_mst``).  Returns ``[(graph, n_components,
    component_labels, forest), ...]``."""
    torch = _native._torch()
    sizes = np.asarray(sizes, dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    P = int(offs[-1])
    n_cl = len(sizes)
    nb_block = np.asarray(nb_block, dtype=np.int32).reshape(P, -1)
    k = nb_block.shape[1]
    lens_block = np.asarray(lens_block, dtype=np.float64)
    if np.any(np.isnan(lens_block)):
        raise ValueError("lens values must not be NaN")
    mst_local = np.asarray(mst_local, dtype=np.float64).reshape(-1, 3)
    mst_bounds = np.asarray(mst_bounds, dtype=np.int64)
    # parent rows as block rows; children stay in-cluster ids
    m_owner = np.repeat(np.arange(n_cl), np.diff(mst_bounds))
    mparent = (mst_local[:, 0].astype(np.int64) + offs[:-1][m_owner]).astype(np.int32)
    mchild = mst_local[:, 1].astype(np.int32)
    mdist = mst_local[:, 2]
    M = len(mparent)
    if P == 0:
        return [(CoreGraph(np.zeros(0, np.float32), np.zeros(0, np.float32),
                           np.zeros(0, np.int32), np.zeros(1, np.int32)), 0,
                 np.zeros(0, np.int64), np.zeros((0, 3))) for _ in range(n_cl)]
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    V = _native.vptr
    cap = P * k + M
    d = dict(nb=T(nb_block), lens=T(lens_block), core=T(np.asarray(core_block, np.float32)),
             bs=T(np.repeat(offs[:-1], sizes).astype(np.int32)),
             be=T(np.repeat(offs[1:], sizes).astype(np.int32)),
             mp=T(mparent), mc=T(mchild), md=T(np.ascontiguousarray(mdist)))
    indptr = torch.empty(P + 1, dtype=torch.int32, device="cuda")
    il = torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
    ib = torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
    w = torch.empty(max(cap, 1), dtype=torch.float32, device="cuda")
    dist = torch.empty(max(cap, 1), dtype=torch.float32, device="cuda")
    seg = torch.empty(P, dtype=torch.int32, device="cuda")
    nnz = ctypes.c_int64(0)
    lib = _native.load()
    s = _native.stream_ptr()
    _native.check(lib.fhg_core_graphs(P, k, V(d["nb"]), V(d["lens"]), V(d["core"]), V(d["bs"]),
                                      V(d["be"]), M, V(d["mp"]) if M else None,
                                      V(d["mc"]) if M else None, V(d["md"]) if M else None,
                                      V(indptr), V(il), V(ib), V(w), V(dist), V(seg),
                                      ctypes.byref(nnz), s))
    edges = torch.empty((max(P - 1, 1), 3), dtype=torch.float64, device="cuda")
    m = ctypes.c_int64(0)
    _native.check(lib.fhg_core_graph_mst(V(indptr), V(ib), V(w), V(seg), P, V(edges),
                                         ctypes.byref(m), s))
    z = int(nnz.value)
    h_indptr = indptr.cpu().numpy()
    h_il, h_w, h_d = il[:z].cpu().numpy(), w[:z].cpu().numpy(), dist[:z].cpu().numpy()
    all_edges = edges[: m.value].cpu().numpy()
    owner = np.searchsorted(offs, all_edges[:, 0].astype(np.int64), side="right") - 1
    order = np.argsort(owner, kind="stable")
    bounds = np.searchsorted(owner[order], np.arange(n_cl + 1))
    out_graphs = []
    for i, sz in enumerate(sizes):
        a, b = int(h_indptr[offs[i]]), int(h_indptr[offs[i + 1]])
        g = CoreGraph(h_w[a:b].copy(), h_d[a:b].copy(), h_il[a:b].copy(),
                      (h_indptr[offs[i]:offs[i + 1] + 1] - a).astype(np.int32))
        f = all_edges[order[bounds[i]:bounds[i + 1]]].copy()
        f[:, :2] -= offs[i]
        nc = int(sz) - len(f)
        comp = np.zeros(int(sz), np.int64) if nc <= 1 else _root_labels(int(sz), f)
        out_graphs.append((g, max(nc, 1) if sz > 0 else 0, comp, f))
    return out_graphs


def _clusters_of_forest(num_components, component_labels, lensed_mst, graph, **kwargs):
    from .hdbscan import clusters_from_spanning_tree

    if num_components > 1:
        return (component_labels, np.ones(len(component_labels), dtype=np.float32),
                np.empty((0, 4)), empty_condensed_tree(), lensed_mst, graph)
    return (*clusters_from_spanning_tree(lensed_mst, **kwargs), graph)


def core_graph_clusters(lens, neighbors, core_distances, min_spanning_tree, **kwargs):
    """core_graph.py:244: the cluster hierarchy of the lens-weighted core
    graph's spanning tree, or its components when it is disconnected."""
    num_components, component_labels, lensed_mst, graph = core_graph_spanning_tree(
        neighbors, core_distances, min_spanning_tree, lens)
    return _clusters_of_forest(num_components, component_labels, lensed_mst, graph, **kwargs)


def core_graph_to_rec_array(graph):
    """core_graph.py:253."""
    result = np.empty(graph.indptr[-1], dtype=[("parent", np.int32), ("child", np.int32),
                                               ("weight", np.float32),
                                               ("distance", np.float32)])
    result["parent"] = np.repeat(np.arange(len(graph.indptr) - 1), np.diff(graph.indptr))
    result["child"] = graph.indices
    result["weight"] = graph.weights
    result["distance"] = graph.distances
    return result


def core_graph_to_edge_list(graph):
    """core_graph.py:270."""
    result = np.empty((graph.indptr[-1], 4), dtype=np.float64)
    result[:, 0] = np.repeat(np.arange(len(graph.indptr) - 1), np.diff(graph.indptr))
    result[:, 1] = graph.indices
    result[:, 2] = graph.weights
    result[:, 3] = graph.distances
    return result
