"""GPU tree passes behind the reference's cluster_trees entry points.

Each function keeps the reference's signature and return types
(fast_hdbscan/cluster_trees.py) and runs on the CUDA engine through the C ABI
in include/fhg.h: NumPy arrays in, NumPy arrays out.
"""
import ctypes
from collections import namedtuple

import numpy as np

from . import _native

CondensedTree = namedtuple("CondensedTree", ["parent", "child", "lambda_val", "child_size"])


def empty_condensed_tree():
    """cluster_trees.py:185."""
    parents = np.empty(shape=0, dtype=np.intp)
    others = np.empty(shape=0, dtype=np.float32)
    return CondensedTree(parents, parents, others, others)


def _dev(a, dtype):
    return _native.to_device(np.ascontiguousarray(a, dtype=dtype), dtype)


def _ct_dev(ct):
    return (_dev(ct.parent, np.int64), _dev(ct.child, np.int64),
            _dev(ct.lambda_val, np.float32), _dev(ct.child_size, np.float32))


def sort_mst(mst):
    """The np.lexsort((mst[:,1], mst[:,0], mst[:,2])) of hdbscan.py:511."""
    mst = np.ascontiguousarray(mst, dtype=np.float64)
    m = mst.shape[0]
    if m == 0:
        return mst.copy()
    d_in = _dev(mst, np.float64)
    d_out = _native.empty((m, 3), np.float64)
    _native.check(_native.load().fhg_sort_mst(_native.vptr(d_in), m, _native.vptr(d_out),
                                              _native.stream_ptr()))
    return d_out.cpu().numpy()


def _linkage(sorted_mst, sample_weights):
    sorted_mst = np.ascontiguousarray(sorted_mst, dtype=np.float64)
    m = sorted_mst.shape[0]
    if m == 0:
        return np.empty((0, 4), dtype=np.float64)
    d_in = _dev(sorted_mst, np.float64)
    d_w = None if sample_weights is None else _dev(sample_weights, np.float32)
    d_out = _native.empty((m, 4), np.float64)
    _native.check(_native.load().fhg_mst_to_linkage_tree(
        _native.vptr(d_in), m, _native.vptr(d_w), _native.vptr(d_out), _native.stream_ptr()))
    return d_out.cpu().numpy()


def mst_to_linkage_tree(sorted_mst):
    """cluster_trees.py:65."""
    return _linkage(sorted_mst, None)


def mst_to_linkage_tree_w_sample_weights(sorted_mst, sample_weights):
    """cluster_trees.py:98: sizes are float32 sums of the sample weights."""
    return _linkage(sorted_mst, np.asarray(sample_weights, dtype=np.float32))


def condense_tree(hierarchy, min_cluster_size=10, max_cluster_size=np.inf, sample_weights=None,
                  lambda_method="hdbscan"):
    """cluster_trees.py:205 (hdbscan lambda).  With sample weights the
    hierarchy's size column holds weight sums (mst_to_linkage_tree_w_sample_weights)."""
    if lambda_method != "hdbscan":
        raise NotImplementedError("only lambda_method='hdbscan' is on the fit path")
    h = np.ascontiguousarray(hierarchy, dtype=np.float64)
    m = h.shape[0]
    if m == 0:
        return empty_condensed_tree()
    d_h = _dev(h, np.float64)
    d_w = None if sample_weights is None else _dev(sample_weights, np.float32)
    cap = 2 * m
    p, c = _native.empty(cap, np.int64), _native.empty(cap, np.int64)
    lam, sz = _native.empty(cap, np.float32), _native.empty(cap, np.float32)
    rows = ctypes.c_int64(0)
    _native.check(_native.load().fhg_condense_tree(
        _native.vptr(d_h), m, int(min_cluster_size), float(max_cluster_size), _native.vptr(d_w),
        _native.vptr(p),
        _native.vptr(c), _native.vptr(lam), _native.vptr(sz), ctypes.byref(rows),
        _native.stream_ptr()))
    r = rows.value
    return CondensedTree(p[:r].cpu().numpy(), c[:r].cpu().numpy(), lam[:r].cpu().numpy(),
                         sz[:r].cpu().numpy())


def mask_condensed_tree(condensed_tree, mask):
    """cluster_trees.py:677."""
    return CondensedTree(condensed_tree.parent[mask], condensed_tree.child[mask],
                         condensed_tree.lambda_val[mask], condensed_tree.child_size[mask])


def cluster_tree_from_condensed_tree(condensed_tree):
    """cluster_trees.py:672."""
    return mask_condensed_tree(condensed_tree, condensed_tree.child_size > 1)


def extract_eom_clusters(condensed_tree, cluster_tree, max_cluster_size=np.inf,
                         allow_single_cluster=False):
    """cluster_trees.py:724.  The cluster tree is the child_size > 1 subset of
    the condensed tree, which is all the GPU kernel reads."""
    if len(cluster_tree.parent) == 0:
        return np.zeros(0, dtype=np.int64)
    ct = condensed_tree
    rows = len(ct.parent)
    d = _ct_dev(ct)
    sel = _native.empty(rows, np.int64)
    k = ctypes.c_int64(0)
    _native.check(_native.load().fhg_extract_eom_clusters(
        *[_native.vptr(x) for x in d], rows, float(max_cluster_size), int(bool(allow_single_cluster)),
        _native.vptr(sel), ctypes.byref(k), _native.stream_ptr()))
    return sel[:k.value].cpu().numpy()


def cluster_tree_leaves(cluster_tree, n_points):
    """cluster_trees.py:369 (the cluster tree's rows are a condensed tree of
    their own for the kernel: every row has child_size > 1)."""
    rows = len(cluster_tree.parent)
    if rows == 0:
        return np.zeros(0, dtype=np.int64)
    d = _ct_dev(cluster_tree)
    sel = _native.empty(rows + 1, np.int64)
    k = ctypes.c_int64(0)
    _native.check(_native.load().fhg_cluster_tree_leaves(
        *[_native.vptr(x) for x in d], rows, _native.vptr(sel), ctypes.byref(k),
        _native.stream_ptr()))
    return sel[:k.value].cpu().numpy()


def get_cluster_label_vector(tree, clusters, cluster_selection_epsilon, n_samples):
    """cluster_trees.py:944."""
    clusters = np.asarray(clusters, dtype=np.int64)
    if len(tree.parent) == 0 or len(clusters) == 0:
        return np.full(n_samples, -1, dtype=np.intp)
    rows = len(tree.parent)
    d = _ct_dev(tree)
    d_sel = _dev(clusters, np.int64)
    labels = _native.empty(n_samples, np.int64)
    probs = _native.empty(n_samples, np.float32)
    rc = _native.load().fhg_label_points(
        *[_native.vptr(x) for x in d], rows, _native.vptr(d_sel), len(clusters),
        float(cluster_selection_epsilon), int(n_samples), _native.vptr(labels),
        _native.vptr(probs), _native.stream_ptr())
    if rc == _native.FHG_ERR_INVALID and "KeyError" in _native.load().fhg_last_error().decode():
        raise KeyError(_native.load().fhg_last_error().decode())
    _native.check(rc)
    return labels.cpu().numpy().astype(np.intp, copy=False)


def get_point_membership_strength_vector(tree, clusters, labels):
    """cluster_trees.py:1011."""
    labels = np.ascontiguousarray(labels, dtype=np.int64)
    n = labels.shape[0]
    clusters = np.asarray(clusters, dtype=np.int64)
    rows = len(tree.parent)
    if rows == 0 or len(clusters) == 0:
        return np.zeros(n, dtype=np.float32)
    d = _ct_dev(tree)
    d_sel = _dev(clusters, np.int64)
    d_lab = _dev(labels, np.int64)
    probs = _native.empty(n, np.float32)
    _native.check(_native.load().fhg_membership_strengths(
        *[_native.vptr(x) for x in d], rows, _native.vptr(d_sel), len(clusters),
        _native.vptr(d_lab), n, _native.vptr(probs), _native.stream_ptr()))
    return probs.cpu().numpy()


def simplify_hierarchy(condensed_tree, persistence_threshold):
    """cluster_trees.py:774.  Like the reference, relabels the rows it keeps in
    the argument's arrays in place and returns the simplified tree."""
    ct = condensed_tree
    rows = len(ct.parent)
    if rows == 0:
        return ct
    d = _ct_dev(ct)
    E = _native.empty
    op, oc, ol, os_ = E(rows, np.int64), E(rows, np.int64), E(rows, np.float32), E(rows, np.float32)
    k = ctypes.c_int64(0)
    V = _native.vptr
    _native.check(_native.load().fhg_simplify_hierarchy(
        *[V(x) for x in d], rows, float(persistence_threshold), V(op), V(oc), V(ol), V(os_),
        ctypes.byref(k), _native.stream_ptr()))
    for host, dev in zip((ct.parent, ct.child, ct.lambda_val), d[:3]):
        if isinstance(host, np.ndarray) and host.flags.writeable:
            np.copyto(host, dev.cpu().numpy().astype(host.dtype, copy=False))
    r = k.value
    return CondensedTree(op[:r].cpu().numpy(), oc[:r].cpu().numpy(), ol[:r].cpu().numpy(),
                         os_[:r].cpu().numpy())


def cluster_epsilon_search(clusters, cluster_tree, min_epsilon=0.0):
    """cluster_trees.py:834."""
    clusters = np.asarray(clusters, dtype=np.int64)
    if len(clusters) == 0:
        return np.zeros(0, dtype=np.int64)
    rows = len(cluster_tree.parent)
    d = _ct_dev(cluster_tree)
    d_sel = _dev(clusters, np.int64)
    out = _native.empty(len(clusters), np.int64)
    k = ctypes.c_int64(0)
    V = _native.vptr
    _native.check(_native.load().fhg_cluster_epsilon_search(
        *[V(x) for x in d], rows, V(d_sel), len(clusters), float(min_epsilon), V(out),
        ctypes.byref(k), _native.stream_ptr()))
    return out[:k.value].cpu().numpy()


def get_cluster_labelling_at_cut(linkage_tree, cut, min_cluster_size):
    """cluster_trees.py:906 (HDBSCAN.dbscan_clustering)."""
    lk = np.ascontiguousarray(linkage_tree, dtype=np.float64)
    m = lk.shape[0]
    labels = _native.empty(m + 1, np.int64)
    d_lk = _dev(lk, np.float64) if m > 0 else None
    _native.check(_native.load().fhg_labelling_at_cut(
        _native.vptr(d_lk), m, float(cut), int(min_cluster_size), _native.vptr(labels),
        _native.stream_ptr()))
    return labels.cpu().numpy().astype(np.intp, copy=False)
