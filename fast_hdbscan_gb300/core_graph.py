"""Core graphs of clusters for sub-cluster and branch detection
(core_graph.py of the reference).

A cluster's core graph joins each point to its in-cluster kNN neighbours and
to its in-cluster MST children; an edge's weight is the larger lens value of
its two ends and its distance the larger core distance (MST edges keep their
MST distance).  The graph is laid out on the host (a few numpy passes over
n * k entries, as cheap as the lens itself); its minimum spanning forest --
Kruskal's, with +inf bridges -- and the cluster hierarchy of that forest run
on the GPU (``fhg_precomputed_mst`` with min_samples 1, then the tree passes
of ``clusters_from_spanning_tree``).

The reference builds the forest with a Boruvka pass whose equal-weight
choices follow numba's unstable argsort; lens weights tie wherever an edge's
larger lens belongs to a shared end, so the forest's equal-weight edges may
differ while its weights, and the single-linkage merge heights, are the
same.
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
    nb = np.asarray(neighbors)
    k = nb.shape[1] if nb.ndim == 2 else 0
    rows_k = np.repeat(np.arange(n, dtype=np.int64), k)
    cols_k = nb.reshape(-1).astype(np.int64)
    valid = cols_k >= 0
    rows_k, cols_k = rows_k[valid], cols_k[valid]
    w_k = np.maximum(lens[rows_k], lens[cols_k])
    d_k = np.maximum(core[rows_k], core[cols_k])
    mst = np.asarray(min_spanning_tree, dtype=np.float64).reshape(-1, 3)
    rows_m = mst[:, 0].astype(np.int64)
    cols_m = mst[:, 1].astype(np.int64)
    new = ~np.isin(rows_m * n + cols_m, rows_k * n + cols_k)
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


def core_graph_spanning_tree(neighbors, core_distances, min_spanning_tree, lens):
    """core_graph.py:234: ``(n_components, component_labels, lensed_mst,
    graph)`` -- the minimum spanning forest of the core graph on its lens
    weights (component labels number the components by their smallest
    point)."""
    torch = _native._torch()
    graph = knn_mst_union(neighbors, core_distances, min_spanning_tree, lens)
    n = len(graph.indptr) - 1
    if n == 0:
        return 0, np.zeros(0, np.int64), np.zeros((0, 3)), graph
    w = graph.weights.astype(np.float64)
    if np.any(np.isnan(w)):
        raise ValueError("lens values must not be NaN")
    # the GPU forest orders non-negative float64 weights; a constant shift
    # (exact in float64 for float32 weights of similar magnitude) keeps their
    # order, and the forest's weights are recomputed from the lens below
    shift = -float(w.min()) if len(w) and w.min() < 0 else 0.0
    rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(graph.indptr))
    d_rows = torch.from_numpy(rows).cuda()
    d_cols = torch.from_numpy(np.ascontiguousarray(graph.indices)).cuda()
    d_w = torch.from_numpy(w + shift).cuda()
    edges = torch.empty((max(n - 1, 0), 3), dtype=torch.float64, device="cuda")
    nbrs = torch.empty((n, 1), dtype=torch.int32, device="cuda")
    core = torch.empty((n,), dtype=torch.float64, device="cuda")
    ncomp = ctypes.c_int64(0)
    V = _native.vptr
    _native.check(_native.load().fhg_precomputed_mst(
        V(d_rows), V(d_cols), V(d_w), int(d_w.numel()), n, 1, 1, V(edges), V(nbrs), V(core),
        ctypes.byref(ncomp), _native.stream_ptr()))
    nc = int(ncomp.value)
    # Kruskal's forest first, then the nc - 1 bridges between its components
    forest = edges.cpu().numpy()[: n - nc].copy()
    a, b = forest[:, 0].astype(np.int64), forest[:, 1].astype(np.int64)
    lv = np.asarray(lens)
    forest[:, 2] = np.maximum(lv[a], lv[b]).astype(np.float32).astype(np.float64)
    if nc <= 1:
        return 1, np.zeros(n, np.int64), forest, graph
    # the forest's components, numbered by their smallest point
    import scipy.sparse
    from scipy.sparse.csgraph import connected_components

    adj = scipy.sparse.coo_matrix((np.ones(len(forest)), (a, b)), shape=(n, n))
    _, comp = connected_components(adj, directed=False)
    return nc, comp.astype(np.int64), forest, graph


def core_graph_clusters(lens, neighbors, core_distances, min_spanning_tree, **kwargs):
    """core_graph.py:244: the cluster hierarchy of the lens-weighted core
    graph's spanning tree, or its components when it is disconnected."""
    from .hdbscan import clusters_from_spanning_tree

    num_components, component_labels, lensed_mst, graph = core_graph_spanning_tree(
        neighbors, core_distances, min_spanning_tree, lens)
    if num_components > 1:
        return (component_labels, np.ones(len(component_labels), dtype=np.float32),
                np.empty((0, 4)), empty_condensed_tree(), lensed_mst, graph)
    return (*clusters_from_spanning_tree(lensed_mst, **kwargs), graph)


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
