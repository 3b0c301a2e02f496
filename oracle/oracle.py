"""numpy front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the benchmark's CPU-baseline
leg use this module, as the checker; the product library never imports it.
Function names and return conventions follow the reference modules they
restate (fast_hdbscan/hdbscan.py, boruvka.py, numba_kdtree.py,
cluster_trees.py).  ``mode=0`` reproduces the reference's tie behaviour,
``mode=1`` the canonical total-order tie-breaking the GPU engine implements.
"""
import ctypes
import os
from collections import namedtuple

import numpy as np

from . import build as _build

CondensedTree = namedtuple("CondensedTree", ["parent", "child", "lambda_val", "child_size"])

_lib = None
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_INT = ctypes.c_int
_D = ctypes.c_double


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        L.orc_build_kdtree.restype = _P
        L.orc_build_kdtree.argtypes = [_P, _I64, _I64, _I64]
        L.orc_free_kdtree.argtypes = [_P]
        L.orc_kdtree_n_nodes.restype = _I64
        L.orc_kdtree_n_nodes.argtypes = [_P]
        L.orc_kdtree_arrays.argtypes = [_P] * 6
        L.orc_tree_query.argtypes = [_P, _I64, _INT, _INT, _P, _P]
        L.orc_parallel_boruvka.restype = _I64
        L.orc_parallel_boruvka.argtypes = [_P, _I64, _INT, _INT, _P, _I64, _P, _P, _P, _P]
        L.orc_sort_mst.argtypes = [_P, _I64, _P]
        L.orc_mst_to_linkage_tree.argtypes = [_P, _I64, _P]
        L.orc_mst_to_linkage_tree_w.argtypes = [_P, _I64, _P, _P]
        L.orc_condense_tree.restype = _I64
        L.orc_condense_tree.argtypes = [_P, _I64, _I64, _D, _P, _P, _P, _P, _P]
        L.orc_simplify_hierarchy.restype = _I64
        L.orc_simplify_hierarchy.argtypes = [_P, _P, _P, _P, _I64, _D]
        L.orc_extract_eom_clusters.restype = _I64
        L.orc_extract_eom_clusters.argtypes = [_P, _P, _P, _P, _I64, _D, _INT, _P]
        L.orc_cluster_tree_leaves.restype = _I64
        L.orc_cluster_tree_leaves.argtypes = [_P, _P, _P, _I64, _I64, _P]
        L.orc_cluster_epsilon_search.restype = _I64
        L.orc_cluster_epsilon_search.argtypes = [_P, _P, _P, _P, _I64, _P, _I64, _D, _P]
        L.orc_get_cluster_label_vector.restype = _INT
        L.orc_get_cluster_label_vector.argtypes = [_P, _P, _P, _I64, _P, _I64, _D, _I64, _P]
        L.orc_get_point_membership_strength_vector.argtypes = [
            _P, _P, _P, _P, _I64, _P, _I64, _P, _I64, _P]
        L.orc_get_cluster_labelling_at_cut.argtypes = [_P, _I64, _D, _I64, _P]
        L.orc_precomputed_kruskal.restype = _I64
        L.orc_precomputed_kruskal.argtypes = [_P, _P, _P, _I64, _I64, _I64, _P, _P, _P]
        L.orc_kruskal_knn.restype = _I64
        L.orc_kruskal_knn.argtypes = [_P, _P, _I64, _I64, _I64, _P, _P, _P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class KDTree:
    """numba_kdtree.py:478 build_kdtree restated (leaf_size 40)."""

    def __init__(self, X, leaf_size=40):
        self.data = np.ascontiguousarray(X, dtype=np.float32)
        if self.data.ndim == 1:
            self.data = self.data.reshape(-1, 1)
        n, d = self.data.shape
        self._h = lib().orc_build_kdtree(_p(self.data), n, d, leaf_size)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_free_kdtree(self._h)
            self._h = None

    def arrays(self):
        n, d = self.data.shape
        nn = lib().orc_kdtree_n_nodes(self._h)
        ia = np.empty(n, np.int64)
        s = np.empty(nn, np.int64)
        e = np.empty(nn, np.int64)
        lf = np.empty(nn, np.uint8)
        nb = np.empty((2, nn, d), np.float32)
        lib().orc_kdtree_arrays(self._h, _p(ia), _p(s), _p(e), _p(lf), _p(nb))
        return dict(idx_array=ia, idx_start=s, idx_end=e, is_leaf=lf.astype(bool),
                    node_bounds=nb)


def build_kdtree(X, leaf_size=40):
    return KDTree(X, leaf_size)


def tree_query(tree, k, mode=0, nthreads=1):
    """numba_kdtree.py:765 parallel_tree_query(tree, tree.data, k, output_rdist=True)."""
    n = tree.data.shape[0]
    rd = np.empty((n, k), np.float32)
    ix = np.empty((n, k), np.int32)
    lib().orc_tree_query(tree._h, k, mode, nthreads, _p(rd), _p(ix))
    return rd, ix


def weighted_knn_k(sample_weights, min_samples):
    """boruvka.py:561-563: k = int(2 * min_samples / mean(sample_weights)).  The
    mean is taken in float64 (the reference accumulates float32; the two agree
    unless 2 * min_samples / mean falls within rounding of an integer)."""
    w = np.asarray(sample_weights, np.float32)
    mean = float(np.sum(w, dtype=np.float64)) / w.shape[0]
    return int(2 * (min_samples / mean))


def parallel_boruvka(tree, min_samples=10, mode=0, nthreads=1, sample_weights=None):
    """boruvka.py:542 parallel_boruvka -> (edges, neighbors, core, rounds)."""
    n = tree.data.shape[0]
    w = None
    if sample_weights is not None and len(sample_weights) > 1:
        w = np.ascontiguousarray(sample_weights, np.float32)
        k = weighted_knn_k(w, min_samples)
    else:
        k = min_samples + 1 if min_samples > 1 else 2
    edges = np.zeros((max(n - 1, 0), 3), np.float64)
    nbrs = np.empty((n, max(k - 1, 0)), np.int32)
    core = np.empty(n, np.float32)
    rounds = np.zeros(1, np.int64)
    m = lib().orc_parallel_boruvka(tree._h, min_samples, mode, nthreads, _p(w), k, _p(edges),
                                   _p(nbrs), _p(core), _p(rounds))
    return edges[:m], nbrs, core, int(rounds[0])


def kruskal_query_k(min_samples, knn_k, sample_weights=None):
    """kruskal.py:981-1007: the kNN query size of _kruskal_mst_knn (the point
    itself included)."""
    if sample_weights is not None:
        mean_sw = float(np.mean(np.asarray(sample_weights, np.float32)))
        return max(knn_k, int(2 * min_samples / mean_sw)) + 1
    if min_samples > 1:
        return max(knn_k, min_samples) + 1
    return knn_k + 1


def kruskal_knn(tree, min_samples, knn_k, mode=0, nthreads=1, sample_weights=None):
    """kruskal.py:950 _kruskal_mst_knn (no cannot-link constraints) ->
    (mst_edges float64[n-1, 3], neighbors int32, core_distances float64)."""
    n = tree.data.shape[0]
    w = None if sample_weights is None else np.ascontiguousarray(sample_weights, np.float32)
    kq = kruskal_query_k(min_samples, knn_k, w)
    rd, ix = tree_query(tree, kq, mode, nthreads)
    edges = np.zeros((max(n - 1, 0), 3), np.float64)
    core = np.empty(n, np.float64)
    m = lib().orc_kruskal_knn(_p(rd), _p(ix), n, kq, min_samples, _p(w), _p(edges), _p(core))
    if w is not None:
        nbrs = ix[:, 1:]
    elif min_samples > 1:
        nbrs = ix[:, 1:min_samples + 1]
    else:
        nbrs = ix[:, 1:2]
    return edges[:m], np.ascontiguousarray(nbrs), core


def precomputed_kruskal(X, min_samples):
    """precomputed.py:479 compute_mst_from_precomputed_sparse_kruskal (no
    cannot-link constraints) on a scipy sparse matrix -> (mst_edges,
    neighbors, core_distances)."""
    coo = X.tocoo()
    n = X.shape[0]
    rows = np.ascontiguousarray(coo.row, np.int32)
    cols = np.ascontiguousarray(coo.col, np.int32)
    data = np.ascontiguousarray(coo.data, np.float64)
    k = max(1, int(min_samples))
    edges = np.zeros((max(n - 1, 0), 3), np.float64)
    nbrs = np.empty((n, k), np.int32)
    core = np.empty(n, np.float64)
    m = lib().orc_precomputed_kruskal(_p(rows), _p(cols), _p(data), len(data), n, min_samples,
                                      _p(edges), _p(nbrs), _p(core))
    return edges[:m], nbrs, core


def sort_mst(mst):
    """hdbscan.py:511 np.lexsort((dst, src, weight))."""
    mst = np.ascontiguousarray(mst, np.float64)
    out = np.empty_like(mst)
    lib().orc_sort_mst(_p(mst), mst.shape[0], _p(out))
    return out


def mst_to_linkage_tree(sorted_mst, sample_weights=None):
    """cluster_trees.py:65 (and :98 mst_to_linkage_tree_w_sample_weights)."""
    sorted_mst = np.ascontiguousarray(sorted_mst, np.float64)
    out = np.empty((sorted_mst.shape[0], 4), np.float64)
    if sample_weights is None:
        lib().orc_mst_to_linkage_tree(_p(sorted_mst), sorted_mst.shape[0], _p(out))
    else:
        w = np.ascontiguousarray(sample_weights, np.float32)
        lib().orc_mst_to_linkage_tree_w(_p(sorted_mst), sorted_mst.shape[0], _p(w), _p(out))
    return out


def condense_tree(hierarchy, min_cluster_size=10, max_cluster_size=np.inf, sample_weights=None):
    h = np.ascontiguousarray(hierarchy, np.float64)
    m = h.shape[0]
    cap = max(2 * m, 1)
    p = np.empty(cap, np.int64)
    c = np.empty(cap, np.int64)
    lam = np.empty(cap, np.float32)
    sz = np.empty(cap, np.float32)
    w = None if sample_weights is None else np.ascontiguousarray(sample_weights, np.float32)
    rows = lib().orc_condense_tree(_p(h), m, int(min_cluster_size), float(max_cluster_size),
                                   _p(w), _p(p), _p(c), _p(lam), _p(sz))
    return CondensedTree(p[:rows].copy(), c[:rows].copy(), lam[:rows].copy(), sz[:rows].copy())


def simplify_hierarchy(ct, threshold):
    p, c = ct.parent.copy(), ct.child.copy()
    lam, sz = ct.lambda_val.copy(), ct.child_size.copy()
    rows = lib().orc_simplify_hierarchy(_p(p), _p(c), _p(lam), _p(sz), p.shape[0],
                                        float(threshold))
    return CondensedTree(p[:rows].copy(), c[:rows].copy(), lam[:rows].copy(), sz[:rows].copy())


def _ct(ct):
    return (np.ascontiguousarray(ct.parent, np.int64), np.ascontiguousarray(ct.child, np.int64),
            np.ascontiguousarray(ct.lambda_val, np.float32),
            np.ascontiguousarray(ct.child_size, np.float32))


def extract_eom_clusters(ct, max_cluster_size=np.inf, allow_single_cluster=False):
    p, c, lam, sz = _ct(ct)
    sel = np.empty(max(p.shape[0], 1), np.int64)
    k = lib().orc_extract_eom_clusters(_p(p), _p(c), _p(lam), _p(sz), p.shape[0],
                                       float(max_cluster_size), int(allow_single_cluster),
                                       _p(sel))
    return sel[:k].copy()


def cluster_tree_leaves(ct, n_points):
    p, c, lam, sz = _ct(ct)
    sel = np.empty(max(p.shape[0], 1), np.int64)
    k = lib().orc_cluster_tree_leaves(_p(p), _p(c), _p(sz), p.shape[0], n_points, _p(sel))
    return sel[:k].copy()


def cluster_epsilon_search(ct, clusters, min_epsilon):
    p, c, lam, sz = _ct(ct)
    cl = np.ascontiguousarray(clusters, np.int64)
    out = np.empty(max(cl.shape[0], 1), np.int64)
    k = lib().orc_cluster_epsilon_search(_p(p), _p(c), _p(lam), _p(sz), p.shape[0], _p(cl),
                                         cl.shape[0], float(min_epsilon), _p(out))
    return out[:k].copy()


def get_cluster_label_vector(ct, clusters, epsilon, n_samples):
    p, c, lam, sz = _ct(ct)
    cl = np.ascontiguousarray(clusters, np.int64)
    out = np.empty(n_samples, np.int64)
    rc = lib().orc_get_cluster_label_vector(_p(p), _p(c), _p(lam), p.shape[0], _p(cl),
                                            cl.shape[0], float(epsilon), n_samples, _p(out))
    if rc != 0:
        raise KeyError("a point resolved to a cluster that was not selected")
    return out


def get_point_membership_strength_vector(ct, clusters, labels):
    p, c, lam, sz = _ct(ct)
    cl = np.ascontiguousarray(clusters, np.int64)
    lab = np.ascontiguousarray(labels, np.int64)
    out = np.empty(lab.shape[0], np.float32)
    lib().orc_get_point_membership_strength_vector(_p(p), _p(c), _p(lam), _p(sz), p.shape[0],
                                                   _p(cl), cl.shape[0], _p(lab), lab.shape[0],
                                                   _p(out))
    return out


def get_cluster_labelling_at_cut(linkage, cut, min_cluster_size):
    lk = np.ascontiguousarray(linkage, np.float64)
    out = np.empty(lk.shape[0] + 1, np.int64)
    lib().orc_get_cluster_labelling_at_cut(_p(lk), lk.shape[0], float(cut),
                                           int(min_cluster_size), _p(out))
    return out


def clusters_from_spanning_tree(mst, min_cluster_size=10, cluster_selection_method="eom",
                                max_cluster_size=np.inf, allow_single_cluster=False,
                                cluster_selection_epsilon=0.0,
                                cluster_selection_persistence=0.0, sample_weights=None):
    """hdbscan.py:497 clusters_from_spanning_tree (unsupervised)."""
    n_points = mst.shape[0] + 1
    smst = sort_mst(mst)
    linkage = mst_to_linkage_tree(smst, sample_weights)
    ct = condense_tree(linkage, min_cluster_size, sample_weights=sample_weights)
    if cluster_selection_persistence > 0.0 and len(ct.parent) > 0:
        ct = simplify_hierarchy(ct, cluster_selection_persistence)
    n_ct = int((ct.child_size > 1).sum())
    if cluster_selection_method == "eom":
        sel = extract_eom_clusters(ct, max_cluster_size, allow_single_cluster)
    elif cluster_selection_method == "leaf":
        sel = (np.empty(0, np.int64) if n_ct == 0 else cluster_tree_leaves(ct, n_points))
    else:
        raise ValueError(f"Invalid cluster_selection_method {cluster_selection_method}")
    if len(sel) > 1 and cluster_selection_epsilon > 0.0:
        sel = cluster_epsilon_search(ct, sel, cluster_selection_epsilon)
    labels = get_cluster_label_vector(ct, sel, cluster_selection_epsilon, n_points)
    probs = get_point_membership_strength_vector(ct, sel, labels)
    return labels, probs, linkage, ct, smst, sel


Fit = namedtuple("Fit", ["labels", "probabilities", "linkage", "condensed", "sorted_mst",
                         "mst", "neighbors", "core", "selected", "rounds"])


def fit(X, min_samples=None, min_cluster_size=5, mode=0, nthreads=1, sample_weights=None, **kw):
    """hdbscan.py:199 fast_hdbscan restated for the Euclidean Boruvka path."""
    X = np.ascontiguousarray(X, np.float32)
    if X.ndim == 1:
        X = X.reshape(-1, 1)
    ms = min_cluster_size if min_samples is None else min_samples
    tree = build_kdtree(X)
    mst, nbrs, core, rounds = parallel_boruvka(tree, ms, mode, nthreads, sample_weights)
    labels, probs, linkage, ct, smst, sel = clusters_from_spanning_tree(
        mst, min_cluster_size=min_cluster_size, sample_weights=sample_weights, **kw)
    return Fit(labels, probs, linkage, ct, smst, mst, nbrs, core, sel, rounds)
