"""Drop-in for fast_hdbscan/hdbscan.py on the Euclidean fit path.

``HDBSCAN(...).fit`` / ``fit_predict``, ``fast_hdbscan``,
``compute_minimum_spanning_tree`` and ``clusters_from_spanning_tree`` keep the
reference's signatures, validation, error types and return conventions; the
work runs in the GB300 engine (libfhg.so) with no CPU fallback.  On the GPU:
the Euclidean Boruvka fit (with or without sample weights, either tie rule),
algorithm="kruskal" with an integer knn_k, metric="precomputed" sparse
graphs and the d > 30 kNN-graph route.  The rest (other metrics, the
full-pairwise Kruskal, cannot-link constraints, semi-supervised selection)
raises NotImplementedError.
"""
import ctypes
import numbers
from collections import namedtuple

import numpy as np

from . import _native
from .boruvka import parallel_boruvka, weighted_knn_k
from .cluster_trees import (
    CondensedTree,
    cluster_tree_from_condensed_tree,
    cluster_tree_leaves,
    condense_tree,
    extract_eom_clusters,
    get_cluster_label_vector,
    get_point_membership_strength_vector,
    mst_to_linkage_tree,
    sort_mst,
)
from .numba_kdtree import build_kdtree

try:  # scikit-learn is optional: the estimator mirrors its protocol either way
    from sklearn.base import BaseEstimator as _BaseEstimator
    from sklearn.base import ClusterMixin as _ClusterMixin
    from sklearn.utils import check_array as _sk_check_array

    _HAVE_SKLEARN = True
except ImportError:  # pragma: no cover - exercised where sklearn is absent
    _HAVE_SKLEARN = False

    class _BaseEstimator:
        def get_params(self, deep=True):
            import inspect

            sig = inspect.signature(type(self).__init__)
            return {k: getattr(self, k) for k in sig.parameters if k != "self"}

        def set_params(self, **params):
            for k, v in params.items():
                setattr(self, k, v)
            return self

    class _ClusterMixin:
        def fit_predict(self, X, y=None, **kwargs):
            self.fit(X, y=y, **kwargs)
            return self.labels_

    _sk_check_array = None


def check_array(X, ensure_all_finite=True, dtype="numeric"):
    """sklearn.utils.check_array for dense 2-D numeric input."""
    if _HAVE_SKLEARN:
        return _sk_check_array(X, ensure_all_finite=ensure_all_finite)
    if X is None:
        raise ValueError("Expected 2D array, got None")
    if isinstance(X, str):
        raise ValueError(f"Expected 2D array, got scalar array instead:\narray={X}.")
    arr = np.asarray(X)
    if arr.dtype.kind not in "biuf":
        try:
            arr = arr.astype(np.float64)
        except (TypeError, ValueError) as e:
            raise ValueError(f"could not convert input to float: {e}") from None
    if arr.ndim != 2:
        raise ValueError(f"Expected 2D array, got {arr.ndim}D array instead")
    if arr.dtype.kind in "biu":
        arr = arr.astype(np.float64)
    if arr.shape[0] < 1:
        raise ValueError(f"Found array with 0 sample(s) (shape={arr.shape}) while a minimum "
                         "of 1 is required.")
    if ensure_all_finite and not np.all(np.isfinite(arr)):
        raise ValueError("Input contains NaN or infinity.")
    return arr


def _is_tensor(X):
    mod = type(X).__module__
    return mod.startswith("torch") and hasattr(X, "is_cuda")


def _tensor_input(X):
    """A 2-D float32 CUDA copy of a torch tensor (asynchronous from pinned
    host memory) and whether every value is finite (checked on the device)."""
    import torch

    if X.dim() != 2:
        raise ValueError(f"Expected 2D array, got {X.dim()}D array instead")
    Xd = X.to(device="cuda", dtype=torch.float32, non_blocking=True).contiguous()
    return Xd, bool(torch.isfinite(Xd).all().item())


def _check_sample_weight(sample_weight, X, dtype):
    """hdbscan.py:43 simplified check (shape and non-zero)."""
    n = X.shape[0]
    if isinstance(sample_weight, numbers.Number):
        return np.full(n, sample_weight, dtype=dtype)
    sw = np.asarray(sample_weight, dtype=dtype)
    if sw.ndim != 1:
        raise ValueError(f"Sample weights must be 1D array or scalar, got {sw.ndim}D array.")
    if sw.shape != (n,):
        raise ValueError(f"sample_weight.shape == {sw.shape}, expected {(n,)}!")
    if np.all(sw == 0):
        raise ValueError("Sample weights must contain at least one non-zero number.")
    return sw


_REC_DTYPE = np.dtype([("parent", np.intp), ("child", np.intp), ("lambda_val", float),
                       ("child_size", np.float32)])


def to_numpy_rec_array(named_tuple_tree):
    """hdbscan.py:93."""
    if isinstance(named_tuple_tree, np.ndarray) and named_tuple_tree.dtype.names is not None:
        return named_tuple_tree
    size = named_tuple_tree.parent.shape[0]
    result = np.empty(size, dtype=_REC_DTYPE)
    result["parent"] = named_tuple_tree.parent
    result["child"] = named_tuple_tree.child
    result["lambda_val"] = named_tuple_tree.lambda_val
    result["child_size"] = named_tuple_tree.child_size
    return result


def remap_condensed_tree(tree, internal_to_raw, outliers):
    """hdbscan.py:119: re-insert non-finite rows at lambda 0 under the root."""
    finite_count = len(internal_to_raw)
    outlier_count = len(outliers)
    for i, (parent, child, lambda_val, child_size) in enumerate(tree):
        child = internal_to_raw[child] if child < finite_count else child + outlier_count
        tree[i] = (parent + outlier_count, child, lambda_val, child_size)
    root = tree[0][0]
    outlier_tree = np.array([(root, o, 0, 1) for o in outliers],
                            dtype=[("parent", np.intp), ("child", np.intp),
                                   ("lambda_val", float), ("child_size", np.intp)])
    return np.append(outlier_tree, tree)


def remap_single_linkage_tree(tree, internal_to_raw, outliers):
    """hdbscan.py:161: non-finite rows join last at infinite distance."""
    finite_count = len(internal_to_raw)
    outlier_count = len(outliers)
    for i, (left, right, distance, size) in enumerate(tree):
        tree[i, 0] = internal_to_raw[left] if left < finite_count else left + outlier_count
        tree[i, 1] = internal_to_raw[right] if right < finite_count else right + outlier_count
    outlier_tree = np.zeros((len(outliers), 4))
    last_cluster_id = tree[tree.shape[0] - 1][0:2].max()
    last_cluster_size = tree[tree.shape[0] - 1][3]
    for i, outlier in enumerate(outliers):
        outlier_tree[i] = (outlier, last_cluster_id + 1, np.inf, last_cluster_size + 1)
        last_cluster_id += 1
        last_cluster_size += 1
    return np.vstack([tree, outlier_tree])


def _validate_params(min_samples, min_cluster_size, cluster_selection_epsilon,
                     cluster_selection_persistence):
    """hdbscan.py:254-275."""
    if ((not (np.issubdtype(type(min_samples), np.integer) or min_samples is None))
            or not np.issubdtype(type(min_cluster_size), np.integer)
            or (min_samples is not None and min_samples <= 0)
            or min_cluster_size <= 0):
        raise ValueError("Min samples and min cluster size must be positive integers!")
    if (not np.issubdtype(type(cluster_selection_epsilon), np.floating)
            or cluster_selection_epsilon < 0.0):
        raise ValueError("Cluster selection epsilon must be a positive floating point number!")
    if (not np.issubdtype(type(cluster_selection_persistence), np.floating)
            or cluster_selection_persistence < 0.0):
        raise ValueError(
            "Cluster selection persistence must be a positive floating point number!")


def _unsupported_routes(metric, algorithm, sample_weights, semi_supervised, data=None,
                        cannot_link=None, cannot_link_groups=None, knn_k=None):
    if metric not in ("euclidean", "precomputed"):
        raise NotImplementedError(f"metric={metric!r} is outside the GPU engine's Euclidean and "
                                  "precomputed paths")
    if algorithm not in ("boruvka", "kruskal"):
        raise ValueError("algorithm must be 'boruvka' or 'kruskal'. Got: %s" % algorithm)
    has_cl = cannot_link is not None or cannot_link_groups is not None
    if has_cl and algorithm != "kruskal":
        raise ValueError("cannot_link constraints are only supported with algorithm='kruskal'. "
                         "Got algorithm=%r." % algorithm)
    if has_cl:
        raise NotImplementedError("cannot-link constraints are not on the GPU path")
    if metric == "precomputed":
        if sample_weights is not None:
            raise NotImplementedError("sample_weights is not supported with metric='precomputed'.")
        if semi_supervised:
            raise NotImplementedError("semi-supervised selection is outside the GPU engine's path")
        return
    if algorithm == "kruskal":
        if knn_k is None:
            raise NotImplementedError(
                "algorithm='kruskal' with knn_k=None (exact MST from the full pairwise distance "
                "matrix) is not on the GPU path; pass an integer knn_k or use "
                "algorithm='boruvka'")
    if semi_supervised:
        raise NotImplementedError("semi-supervised selection is outside the GPU engine's path")
    if data is not None and _knn_graph_route(metric, data, sample_weights):
        if data.shape[1] > KNN_GRAPH_MAX_DIM:
            raise NotImplementedError(
                f"{data.shape[1]}-dimensional data: the GPU kNN graph supports up to "
                f"{KNN_GRAPH_MAX_DIM} dimensions")
        return
    if data is not None and data.shape[1] > 32:
        raise NotImplementedError(
            f"{data.shape[1]}-dimensional data: the GPU spatial path supports up to 32 dimensions")


KNN_GRAPH_MAX_DIM = 96


def _knn_graph_route(metric, data, sample_weights):
    """hdbscan.py:446-449: Euclidean data with more than 30 dimensions and no
    sample weights takes the kNN-graph back-end (nndescent.py:179), here on
    the GPU's exact high-dimensional kNN."""
    return metric == "euclidean" and data.shape[1] > 30 and sample_weights is None


def resolve_knn_graph_k(min_samples, knn_k):
    """nndescent.py:214-217: knn_k None -> max(3 min_samples, 15); at least
    min_samples."""
    if knn_k is None:
        knn_k = max(3 * min_samples, 15)
    return max(int(knn_k), int(min_samples))


def _degenerate(n, return_trees):
    """hdbscan.py:278-304 (fewer than two points)."""
    labels = np.full(n, -1, dtype=np.intp)
    probabilities = np.zeros(n, dtype=np.float64)
    single_linkage_tree = np.zeros((0, 4), dtype=np.float64)
    condensed_tree = np.zeros(0, dtype=[("parent", np.intp), ("child", np.intp),
                                        ("lambda_val", np.float64), ("child_size", np.intp)])
    mst = np.zeros((0, 3), dtype=np.float64)
    neighbors = np.zeros((n, 0), dtype=np.intp)
    core_distances = np.full(n, np.inf, dtype=np.float64)
    result = (labels, probabilities, single_linkage_tree, condensed_tree, mst, neighbors,
              core_distances)
    return result[: (None if return_trees else 2)]


FitResult = namedtuple("FitResult", ["labels", "probabilities", "linkage", "condensed",
                                     "sorted_mst", "neighbors", "core_distances", "selected"])


def gpu_fit(X, min_samples, min_cluster_size, cluster_selection_method="eom",
            max_cluster_size=np.inf, allow_single_cluster=False, cluster_selection_epsilon=0.0,
            cluster_selection_persistence=0.0, return_trees=True, sample_weights=None,
            condensed_records=False):
    """One call of fhg_hdbscan_fit: every stage on the GPU, outputs copied back.

    X may be a NumPy array, a CPU torch tensor (pinned for asynchronous
    copies) or a CUDA tensor; it is used as float32.  Outputs come back
    through pinned host buffers (one batch of asynchronous copies).  With
    condensed_records the condensed tree comes back as the record array
    HDBSCAN.fit stores (hdbscan.py:93), laid out on the GPU."""
    torch = _native._torch()
    if isinstance(X, torch.Tensor):
        Xd = X.to(device="cuda", dtype=torch.float32, non_blocking=True).contiguous()
    else:
        Xd = _native.to_device(np.ascontiguousarray(X, dtype=np.float32), np.float32)
    n, d = Xd.shape
    ms = min_cluster_size if min_samples is None else min_samples
    d_w, wk = None, 0
    if sample_weights is not None and len(sample_weights) > 1:
        w = np.ascontiguousarray(sample_weights, dtype=np.float32)
        wk = weighted_knn_k(w, ms)
        d_w = _native.to_device(w, np.float32)
    kcols = max(wk - 1, 1) if d_w is not None else (ms if ms > 1 else 1)
    method = {"eom": 0, "leaf": 1}.get(cluster_selection_method)
    if method is None:
        raise ValueError(f"Invalid cluster_selection_method {cluster_selection_method}")
    E = _native.empty
    labels, probs = E(n, np.int64), E(n, np.float32)
    trees = return_trees
    mst = E((n - 1, 3), np.float64) if trees else None
    linkage = E((n - 1, 4), np.float64) if trees else None
    ctp, ctc = (E(2 * n, np.int64), E(2 * n, np.int64)) if trees else (None, None)
    ctl, cts = (E(2 * n, np.float32), E(2 * n, np.float32)) if trees else (None, None)
    nbrs = E((n, kcols), np.int32) if trees else None
    core = E(n, np.float32) if trees else None
    sel = E(n, np.int64)
    rows, nsel = ctypes.c_int64(0), ctypes.c_int64(0)
    V, H = _native.vptr, _native.hptr
    lib = _native.load()

    def pinned(t):
        return torch.empty(t.shape, dtype=t.dtype, pin_memory=True)

    if trees:
        # the large outputs travel to host while the later stages run
        h_nbrs, h_core, h_mst, h_link = pinned(nbrs), pinned(core), pinned(mst), pinned(linkage)
        rec = h_rec = None
        if condensed_records:
            rec = torch.empty(2 * n * 28, dtype=torch.uint8, device="cuda")
            h_rec = pinned(rec)
        rc = lib.fhg_hdbscan_fit_export(
            V(Xd), n, d, int(ms), int(min_cluster_size), method, float(max_cluster_size),
            int(bool(allow_single_cluster)), float(cluster_selection_epsilon),
            float(cluster_selection_persistence), V(d_w), wk, V(labels), V(probs), V(mst),
            V(linkage), V(ctp), V(ctc), V(ctl), V(cts), ctypes.byref(rows), V(nbrs), V(core),
            V(sel), ctypes.byref(nsel), H(h_nbrs), H(h_core), H(h_mst), H(h_link), V(rec),
            H(h_rec), _native.stream_ptr())
    else:
        rc = lib.fhg_hdbscan_fit(
            V(Xd), n, d, int(ms), int(min_cluster_size), method, float(max_cluster_size),
            int(bool(allow_single_cluster)), float(cluster_selection_epsilon),
            float(cluster_selection_persistence), V(d_w), wk, V(labels), V(probs), None, None,
            None, None, None, None, ctypes.byref(rows), None, None, V(sel), ctypes.byref(nsel),
            _native.stream_ptr())
    if rc == _native.FHG_ERR_INVALID and "KeyError" in lib.fhg_last_error().decode():
        raise KeyError(lib.fhg_last_error().decode())
    _native.check(rc)
    r, k = rows.value, nsel.value
    outs = [labels, probs, sel[:k]]
    if trees and not condensed_records:
        outs += [ctp[:r], ctc[:r], ctl[:r], cts[:r]]
    host = []
    for t in outs:
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t, non_blocking=True)
        host.append(h)
    torch.cuda.current_stream().synchronize()
    host = [h.numpy() for h in host]
    if trees:
        host[3:3] = [h_mst.numpy(), h_link.numpy(), h_nbrs.numpy(), h_core.numpy()]
        if condensed_records:
            host.append(h_rec.numpy()[: r * 28])
    labels_h = host[0].astype(np.intp, copy=False)
    if not trees:
        return FitResult(labels_h, host[1], None, None, None, None, None, host[2])
    if condensed_records:
        ct = host[7].view(_REC_DTYPE)
    else:
        ct = CondensedTree(host[7], host[8], host[9], host[10])
    return FitResult(labels_h, host[1], host[4], ct, host[3], host[5], host[6], host[2])


def gpu_fit_kruskal(X, min_samples, min_cluster_size, knn_k, cluster_selection_method="eom",
                    max_cluster_size=np.inf, allow_single_cluster=False,
                    cluster_selection_epsilon=0.0, cluster_selection_persistence=0.0,
                    return_trees=True, sample_weights=None, knn_graph=False,
                    condensed_records=False):
    """One call of fhg_hdbscan_fit_kruskal: the kNN-graph Kruskal MST
    (kruskal.py:950) and the tree passes on the GPU, outputs copied back.
    knn_graph: fhg_hdbscan_fit_knn_graph instead, the d > 30 route
    (nndescent.py:179) on the exact brute-force kNN; knn_k as resolved by
    resolve_knn_graph_k."""
    from .kruskal import kruskal_query_k

    torch = _native._torch()
    if isinstance(X, torch.Tensor):
        Xd = X.to(device="cuda", dtype=torch.float32, non_blocking=True).contiguous()
    else:
        Xd = _native.to_device(np.ascontiguousarray(X, dtype=np.float32), np.float32)
    n, d = Xd.shape
    ms = min_cluster_size if min_samples is None else min_samples
    w = None if sample_weights is None else np.ascontiguousarray(sample_weights, np.float32)
    kq = int(knn_k) + 1 if knn_graph else kruskal_query_k(int(ms), int(knn_k), w)
    kq_max = 64 if knn_graph else 2048  # the kNN graph's lists; the spatial index's
    if kq > kq_max:
        raise NotImplementedError(f"a kNN query of {kq} neighbours exceeds the GPU kNN's "
                                  f"{kq_max}")
    d_w = _native.to_device(w, np.float32) if w is not None else None
    cols = kq - 1 if w is not None else (ms if ms > 1 else 1)
    method = {"eom": 0, "leaf": 1}.get(cluster_selection_method)
    if method is None:
        raise ValueError(f"Invalid cluster_selection_method {cluster_selection_method}")
    E = _native.empty
    labels, probs, sel = E(n, np.int64), E(n, np.float32), E(n, np.int64)
    trees = return_trees
    mst = E((n - 1, 3), np.float64) if trees else None
    linkage = E((n - 1, 4), np.float64) if trees else None
    ctp, ctc = (E(2 * n, np.int64), E(2 * n, np.int64)) if trees else (None, None)
    ctl, cts = (E(2 * n, np.float32), E(2 * n, np.float32)) if trees else (None, None)
    nbrs = E((n, cols), np.int32) if trees else None
    core = E(n, np.float64) if trees else None
    rows, nsel = ctypes.c_int64(0), ctypes.c_int64(0)
    V, lib = _native.vptr, _native.load()
    if knn_graph:
        rc = lib.fhg_hdbscan_fit_knn_graph(
            V(Xd), n, d, int(ms), int(knn_k), int(min_cluster_size), method,
            float(max_cluster_size), int(bool(allow_single_cluster)),
            float(cluster_selection_epsilon), float(cluster_selection_persistence),
            V(labels), V(probs), V(mst), V(linkage), V(ctp), V(ctc), V(ctl), V(cts),
            ctypes.byref(rows), V(nbrs), V(core), V(sel), ctypes.byref(nsel),
            _native.stream_ptr())
    else:
        rc = lib.fhg_hdbscan_fit_kruskal(
            V(Xd), n, d, int(ms), int(knn_k), kq, int(min_cluster_size), method,
            float(max_cluster_size), int(bool(allow_single_cluster)),
            float(cluster_selection_epsilon), float(cluster_selection_persistence), V(d_w),
            V(labels), V(probs), V(mst), V(linkage), V(ctp), V(ctc), V(ctl), V(cts),
            ctypes.byref(rows), V(nbrs), V(core), V(sel), ctypes.byref(nsel),
            _native.stream_ptr())
    if rc == _native.FHG_ERR_INVALID and "KeyError" in lib.fhg_last_error().decode():
        raise KeyError(lib.fhg_last_error().decode())
    _native.check(rc)
    return _fit_outputs_to_host(labels, probs, sel, nsel.value, trees, rows.value, linkage,
                                ctp, ctc, ctl, cts, mst, nbrs, core, condensed_records)


def _fit_outputs_to_host(labels, probs, sel, k, trees, r=0, linkage=None, ctp=None, ctc=None,
                         ctl=None, cts=None, mst=None, nbrs=None, core=None, records=False):
    """A fit's device outputs as a FitResult of NumPy arrays: every copy
    queued at once into pinned host memory, one synchronisation.  With
    records the condensed tree comes back as the record array HDBSCAN.fit
    stores (hdbscan.py:93), laid out on the GPU."""
    torch = _native._torch()
    outs = [labels, probs, sel[:k]]
    if trees:
        if records:
            rec = torch.empty(max(r, 1) * _REC_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
            if r > 0:
                _native.check(_native.load().fhg_condensed_record_array(
                    _native.vptr(ctp), _native.vptr(ctc), _native.vptr(ctl), _native.vptr(cts),
                    r, _native.vptr(rec), _native.stream_ptr()))
            cts_out = [rec[: r * _REC_DTYPE.itemsize]]
        else:
            cts_out = [ctp[:r], ctc[:r], ctl[:r], cts[:r]]
        outs += [linkage, mst, nbrs, core] + cts_out
    host = []
    for t in outs:
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t, non_blocking=True)
        host.append(h)
    torch.cuda.current_stream().synchronize()
    host = [h.numpy() for h in host]
    labels_h = host[0].astype(np.intp, copy=False)
    if not trees:
        return FitResult(labels_h, host[1], None, None, None, None, None, host[2])
    ct = host[7].view(_REC_DTYPE) if records else CondensedTree(*host[7:11])
    return FitResult(labels_h, host[1], host[3], ct, host[4], host[5], host[6], host[2])


def gpu_fit_precomputed(G, min_samples, min_cluster_size, algorithm="boruvka",
                        cluster_selection_method="eom", max_cluster_size=np.inf,
                        allow_single_cluster=False, cluster_selection_epsilon=0.0,
                        cluster_selection_persistence=0.0, return_trees=True,
                        condensed_records=False):
    """One call of fhg_hdbscan_fit_precomputed on a scipy sparse graph's COO
    entries (metric="precomputed"), outputs copied back (the condensed tree
    as the record array with condensed_records)."""
    from .precomputed import graph_to_device, validate_precomputed_sparse_graph

    validate_precomputed_sparse_graph(G, check_values=False)
    n = G.shape[0]
    ms = min_cluster_size if min_samples is None else min_samples
    k = max(1, int(ms))
    method = {"eom": 0, "leaf": 1}.get(cluster_selection_method)
    if method is None:
        raise ValueError(f"Invalid cluster_selection_method {cluster_selection_method}")
    rows, cols, data = graph_to_device(G)
    E = _native.empty
    labels, probs, sel = E(n, np.int64), E(n, np.float32), E(n, np.int64)
    trees = return_trees
    mst = E((n - 1, 3), np.float64) if trees else None
    linkage = E((n - 1, 4), np.float64) if trees else None
    ctp, ctc = (E(2 * n, np.int64), E(2 * n, np.int64)) if trees else (None, None)
    ctl, cts = (E(2 * n, np.float32), E(2 * n, np.float32)) if trees else (None, None)
    nbrs = E((n, k), np.int32) if trees else None
    core = E(n, np.float64) if trees else None
    rows_c, nsel = ctypes.c_int64(0), ctypes.c_int64(0)
    V, lib = _native.vptr, _native.load()
    rc = lib.fhg_hdbscan_fit_precomputed(
        V(rows), V(cols), V(data), int(data.numel()), n, int(ms),
        1 if algorithm == "kruskal" else 0, int(min_cluster_size), method,
        float(max_cluster_size), int(bool(allow_single_cluster)),
        float(cluster_selection_epsilon), float(cluster_selection_persistence), V(labels),
        V(probs), V(mst), V(linkage), V(ctp), V(ctc), V(ctl), V(cts), ctypes.byref(rows_c),
        V(nbrs), V(core), V(sel), ctypes.byref(nsel), _native.stream_ptr())
    if rc == _native.FHG_ERR_INVALID and "KeyError" in lib.fhg_last_error().decode():
        raise KeyError(lib.fhg_last_error().decode())
    _native.check(rc)
    return _fit_outputs_to_host(labels, probs, sel, nsel.value, trees, rows_c.value, linkage,
                                ctp, ctc, ctl, cts, mst, nbrs, core, condensed_records)


def fast_hdbscan(data, data_labels=None, semi_supervised=False, ss_algorithm="bc",
                 min_samples=10, min_cluster_size=10, cluster_selection_method="eom",
                 max_cluster_size=np.inf, allow_single_cluster=False,
                 cluster_selection_epsilon=0.0, cluster_selection_persistence=0.0,
                 sample_weights=None, reproducible=False, return_trees=False,
                 metric="euclidean", algorithm="boruvka", knn_k=None, cannot_link=None,
                 validate_cannot_link=True, cannot_link_groups=None, metric_kwds=None):
    """hdbscan.py:199 fast_hdbscan on the GPU engine.  Besides NumPy input,
    `data` may be a torch tensor (CUDA, or pinned host memory) of finite values."""
    return _fast_hdbscan(
        data, data_labels, semi_supervised, ss_algorithm, min_samples, min_cluster_size,
        cluster_selection_method, max_cluster_size, allow_single_cluster,
        cluster_selection_epsilon, cluster_selection_persistence, sample_weights, reproducible,
        return_trees, metric, algorithm, knn_k, cannot_link, validate_cannot_link,
        cannot_link_groups, metric_kwds)


def _fast_hdbscan(data, data_labels=None, semi_supervised=False, ss_algorithm="bc",
                  min_samples=10, min_cluster_size=10, cluster_selection_method="eom",
                  max_cluster_size=np.inf, allow_single_cluster=False,
                  cluster_selection_epsilon=0.0, cluster_selection_persistence=0.0,
                  sample_weights=None, reproducible=False, return_trees=False,
                  metric="euclidean", algorithm="boruvka", knn_k=None, cannot_link=None,
                  validate_cannot_link=True, cannot_link_groups=None, metric_kwds=None,
                  condensed_records=False):
    """fast_hdbscan with one more option for HDBSCAN.fit: the condensed tree
    as the record array the estimator stores, laid out on the GPU."""
    host_rows = False  # finiteness of a NumPy input still to check
    if _is_tensor(data):
        pass
    elif metric == "euclidean":
        data = check_array(data, ensure_all_finite=False)
        host_rows = True
        if sample_weights is not None:
            sample_weights = _check_sample_weight(sample_weights, data, dtype=np.float32)
    elif metric != "precomputed":
        data = check_array(data)
    if semi_supervised:
        if data_labels is None:
            raise ValueError("data_labels must not be None when semi_supervised is set to True!")
        if ss_algorithm not in ["bc", "bc_simple"]:
            raise ValueError(f"Invalid ss_algorithm {ss_algorithm}")
    _validate_params(min_samples, min_cluster_size, cluster_selection_epsilon,
                     cluster_selection_persistence)
    if cluster_selection_method not in ("eom", "leaf"):
        raise ValueError(f"Invalid cluster_selection_method {cluster_selection_method}")
    if data.shape[0] < 2:
        if host_rows:
            check_array(data)
        return _degenerate(data.shape[0], return_trees)
    _unsupported_routes(metric, algorithm, sample_weights, semi_supervised, data, cannot_link,
                        cannot_link_groups, knn_k)
    if host_rows:
        # finiteness checked on the uploaded float32 copy, which every route
        # takes from here; a copy that fails it gets the host check's error
        Xd = _native.to_device(np.ascontiguousarray(data, dtype=np.float32), np.float32)
        if not bool(_native._torch().isfinite(Xd).all().item()):
            check_array(data)
        data = Xd
    if metric == "precomputed":  # hdbscan.py:306-337 on a precomputed sparse graph
        fr = gpu_fit_precomputed(data, min_samples, min_cluster_size, algorithm,
                                 cluster_selection_method, max_cluster_size,
                                 allow_single_cluster, cluster_selection_epsilon,
                                 cluster_selection_persistence, return_trees=return_trees,
                                 condensed_records=condensed_records)
    elif _knn_graph_route(metric, data, sample_weights):  # hdbscan.py:446 -> nndescent.py:179
        ms = min_cluster_size if min_samples is None else min_samples
        fr = gpu_fit_kruskal(data, min_samples, min_cluster_size,
                             resolve_knn_graph_k(ms, knn_k), cluster_selection_method,
                             max_cluster_size, allow_single_cluster, cluster_selection_epsilon,
                             cluster_selection_persistence, return_trees=return_trees,
                             knn_graph=True, condensed_records=condensed_records)
    elif algorithm == "kruskal":  # hdbscan.py:306-337 on the kNN-graph Kruskal MST
        fr = gpu_fit_kruskal(data, min_samples, min_cluster_size, knn_k,
                             cluster_selection_method, max_cluster_size, allow_single_cluster,
                             cluster_selection_epsilon, cluster_selection_persistence,
                             return_trees=return_trees, sample_weights=sample_weights,
                             condensed_records=condensed_records)
    else:
        # reproducible=True: the reference's own Boruvka tie choices
        with _native.tie_rule(bool(reproducible)):
            fr = gpu_fit(data, min_samples, min_cluster_size, cluster_selection_method,
                         max_cluster_size, allow_single_cluster, cluster_selection_epsilon,
                         cluster_selection_persistence, return_trees=return_trees,
                         sample_weights=sample_weights, condensed_records=condensed_records)
    result = (fr.labels, fr.probabilities, fr.linkage, fr.condensed, fr.sorted_mst,
              fr.neighbors, fr.core_distances)
    return result[: (None if return_trees else 2)]


def compute_minimum_spanning_tree(data, min_samples=10, sample_weights=None, reproducible=False,
                                  metric="euclidean", algorithm="boruvka", knn_k=None,
                                  cannot_link=None, validate_cannot_link=True,
                                  cannot_link_groups=None, metric_kwds=None):
    """hdbscan.py:339: (mst float64[n-1, 3] in Boruvka order, neighbors, core)."""
    if algorithm not in ("boruvka", "kruskal"):
        raise ValueError("algorithm must be 'boruvka' or 'kruskal'. Got: %s" % algorithm)
    if cannot_link is not None and cannot_link_groups is not None:
        raise ValueError("cannot_link and cannot_link_groups are mutually exclusive. "
                         "Provide one or the other, not both.")
    if metric == "precomputed":  # hdbscan.py:427-442
        _unsupported_routes(metric, algorithm, sample_weights, False, None, cannot_link,
                            cannot_link_groups, knn_k)
        from .precomputed import (compute_mst_from_precomputed_sparse,
                                  compute_mst_from_precomputed_sparse_kruskal)

        if algorithm == "kruskal":
            return compute_mst_from_precomputed_sparse_kruskal(data, min_samples)
        return compute_mst_from_precomputed_sparse(data, min_samples)
    data = check_array(data)
    _unsupported_routes(metric, algorithm, sample_weights, False, data, cannot_link,
                        cannot_link_groups, knn_k)
    if _knn_graph_route(metric, data, sample_weights):  # hdbscan.py:446-463
        from .nndescent import compute_mst_from_knn_graph

        return compute_mst_from_knn_graph(data, min_samples=min_samples, metric=metric,
                                          metric_kwds=metric_kwds, knn_k=knn_k)
    tree = build_kdtree(data)
    if algorithm == "kruskal":
        from .kruskal import kruskal_mst_from_feature_matrix

        return kruskal_mst_from_feature_matrix(tree, min_samples, knn_k=knn_k,
                                               sample_weights=sample_weights,
                                               reproducible=reproducible)
    if sample_weights is None:
        return parallel_boruvka(tree, 1, min_samples=min_samples, reproducible=reproducible)
    return parallel_boruvka(tree, 1, min_samples=min_samples,
                            sample_weights=np.asarray(sample_weights, dtype=np.float32),
                            reproducible=reproducible)


def _clusters_from_mst(mst, method, min_cluster_size, max_cluster_size, allow_single_cluster,
                       epsilon, persistence, sample_weights):
    """clusters_from_spanning_tree's stages in one fhg_clusters_from_mst call."""
    torch = _native._torch()
    mst = np.ascontiguousarray(mst, dtype=np.float64).reshape(-1, 3)
    m = mst.shape[0]
    n = m + 1
    if sample_weights is not None and np.shape(sample_weights) != (n,):
        raise ValueError(f"sample_weights has shape {np.shape(sample_weights)}; a tree of "
                         f"{m} edges needs one weight per point ({n})")
    d_mst = _native.to_device(mst, np.float64)
    d_w = (_native.to_device(np.ascontiguousarray(sample_weights, dtype=np.float32), np.float32)
           if sample_weights is not None else None)
    E = _native.empty
    labels, probs, sel = E(n, np.int64), E(n, np.float32), E(n, np.int64)
    smst, linkage = E((m, 3), np.float64), E((m, 4), np.float64)
    ctp, ctc = E(2 * n, np.int64), E(2 * n, np.int64)
    ctl, cts = E(2 * n, np.float32), E(2 * n, np.float32)
    rows, nsel = ctypes.c_int64(0), ctypes.c_int64(0)
    V = _native.vptr
    lib = _native.load()
    rc = lib.fhg_clusters_from_mst(
        V(d_mst), n, int(min_cluster_size), method, float(max_cluster_size),
        int(bool(allow_single_cluster)), float(epsilon), float(persistence), V(d_w), V(labels),
        V(probs), V(smst), V(linkage), V(ctp), V(ctc), V(ctl), V(cts), ctypes.byref(rows),
        V(sel), ctypes.byref(nsel), _native.stream_ptr())
    if rc == _native.FHG_ERR_INVALID and "KeyError" in lib.fhg_last_error().decode():
        raise KeyError(lib.fhg_last_error().decode())
    _native.check(rc)
    r = rows.value
    host = []
    for t in (labels, probs, linkage, ctp[:r], ctc[:r], ctl[:r], cts[:r], smst):
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t, non_blocking=True)
        host.append(h)
    torch.cuda.current_stream().synchronize()
    host = [h.numpy() for h in host]
    ct = CondensedTree(host[3], host[4], host[5], host[6])
    return host[0].astype(np.intp, copy=False), host[1], host[2], ct, host[7]


def clusters_from_spanning_tree(minimum_spanning_tree, data_labels=None, semi_supervised=False,
                                ss_algorithm="bc", min_cluster_size=10,
                                cluster_selection_method="eom", max_cluster_size=np.inf,
                                allow_single_cluster=False, cluster_selection_epsilon=0.0,
                                cluster_selection_persistence=0.0, sample_weights=None):
    """hdbscan.py:497: labels, probabilities, linkage, condensed tree, sorted MST.

    One call of fhg_clusters_from_mst (every stage on the GPU, one upload,
    one batch of copies back); a single point goes through the step-by-step
    functions."""
    if semi_supervised:
        raise NotImplementedError("semi-supervised selection is not on the GPU path")
    n_points = minimum_spanning_tree.shape[0] + 1
    if n_points >= 2:
        method = {"eom": 0, "leaf": 1}.get(cluster_selection_method)
        if method is None:
            raise ValueError(f"Invalid cluster_selection_method {cluster_selection_method}")
        return _clusters_from_mst(minimum_spanning_tree, method, min_cluster_size,
                                  max_cluster_size, allow_single_cluster,
                                  cluster_selection_epsilon, cluster_selection_persistence,
                                  sample_weights)
    sorted_mst = sort_mst(minimum_spanning_tree)
    if sample_weights is None:
        linkage_tree = mst_to_linkage_tree(sorted_mst)
    else:
        from .cluster_trees import mst_to_linkage_tree_w_sample_weights

        linkage_tree = mst_to_linkage_tree_w_sample_weights(sorted_mst, sample_weights)
    condensed_tree = condense_tree(linkage_tree, min_cluster_size=min_cluster_size,
                                   sample_weights=sample_weights)
    if cluster_selection_persistence > 0.0 and len(condensed_tree.parent) > 0:
        from .cluster_trees import simplify_hierarchy

        condensed_tree = simplify_hierarchy(condensed_tree, cluster_selection_persistence)
    cluster_tree = cluster_tree_from_condensed_tree(condensed_tree)
    if cluster_selection_method == "eom":
        selected_clusters = extract_eom_clusters(condensed_tree, cluster_tree,
                                                 max_cluster_size=max_cluster_size,
                                                 allow_single_cluster=allow_single_cluster)
    elif cluster_selection_method == "leaf":
        if cluster_tree.parent.shape[0] == 0:
            selected_clusters = np.empty(0, dtype=np.int64)
        else:
            selected_clusters = cluster_tree_leaves(cluster_tree, n_points)
    else:
        raise ValueError(f"Invalid cluster_selection_method {cluster_selection_method}")
    if len(selected_clusters) > 1 and cluster_selection_epsilon > 0.0:
        from .cluster_trees import cluster_epsilon_search

        selected_clusters = cluster_epsilon_search(selected_clusters, cluster_tree,
                                                   min_epsilon=cluster_selection_epsilon)
    clusters = get_cluster_label_vector(condensed_tree, selected_clusters,
                                        cluster_selection_epsilon, n_samples=n_points)
    membership_strengths = get_point_membership_strength_vector(condensed_tree,
                                                                selected_clusters, clusters)
    return clusters, membership_strengths, linkage_tree, condensed_tree, sorted_mst


class HDBSCAN(_ClusterMixin, _BaseEstimator):
    """hdbscan.py:577 HDBSCAN estimator, fitted by the GB300 engine.

    Same parameters and attributes as the reference (labels_, probabilities_,
    _single_linkage_tree, _condensed_tree, _min_spanning_tree, _neighbors,
    _core_distances)."""

    def __init__(self, *, min_cluster_size=5, min_samples=None, cluster_selection_method="eom",
                 allow_single_cluster=False, max_cluster_size=np.inf,
                 cluster_selection_epsilon=0.0, cluster_selection_persistence=0.0,
                 semi_supervised=False, ss_algorithm="bc", reproducible=False,
                 metric="euclidean", algorithm="boruvka", knn_k=None, cannot_link=None,
                 validate_cannot_link=True, cannot_link_groups=None, metric_kwds=None):
        self.min_cluster_size = min_cluster_size
        self.min_samples = min_samples
        self.cluster_selection_method = cluster_selection_method
        self.allow_single_cluster = allow_single_cluster
        self.max_cluster_size = max_cluster_size
        self.cluster_selection_epsilon = cluster_selection_epsilon
        self.cluster_selection_persistence = cluster_selection_persistence
        self.semi_supervised = semi_supervised
        self.ss_algorithm = ss_algorithm
        self.reproducible = reproducible
        self.metric = metric
        self.algorithm = algorithm
        self.knn_k = knn_k
        self.cannot_link = cannot_link
        self.validate_cannot_link = validate_cannot_link
        self.cannot_link_groups = cannot_link_groups
        self.metric_kwds = metric_kwds

    def fit(self, X, y=None, sample_weight=None, **fit_params):
        """hdbscan.py:686: validation, non-finite row filter, GPU fit, remap."""
        if self.semi_supervised:
            raise NotImplementedError("semi-supervised fits are not on the GPU path")
        if self.metric == "precomputed":  # hdbscan.py:688-697: a scipy sparse graph
            from .precomputed import validate_precomputed_sparse_graph

            validate_precomputed_sparse_graph(X, check_values=False)  # weights: on the GPU
            if sample_weight is not None:
                raise NotImplementedError(
                    "sample_weights is not supported with metric='precomputed'.")
            self._raw_data = None
            self._all_finite = True
            kwargs = self.get_params()
            (self.labels_, self.probabilities_, self._single_linkage_tree,
             self._condensed_tree, self._min_spanning_tree, self._neighbors,
             self._core_distances) = _fast_hdbscan(X, None, return_trees=True,
                                                   condensed_records=True, **kwargs)
            self._condensed_tree = to_numpy_rec_array(self._condensed_tree)
            return self
        if _is_tensor(X):
            Xd, finite = _tensor_input(X)
            if finite and sample_weight is None:
                self._raw_data = X
                self._all_finite = True
                kwargs = self.get_params()
                (self.labels_, self.probabilities_, self._single_linkage_tree,
                 self._condensed_tree, self._min_spanning_tree, self._neighbors,
                 self._core_distances) = _fast_hdbscan(Xd, None, return_trees=True,
                                                       condensed_records=True, **kwargs)
                self._condensed_tree = to_numpy_rec_array(self._condensed_tree)
                return self
            X = Xd.cpu().numpy()
        X = check_array(X, ensure_all_finite=False)
        self._raw_data = X
        if sample_weight is None and X.ndim == 2 and X.shape[0] >= 2:
            # upload first, check finiteness on the GPU: a finite input goes
            # straight on from the device copy (the float32 the engine uses)
            Xd = _native.to_device(np.ascontiguousarray(X, dtype=np.float32), np.float32)
            if bool(_native._torch().isfinite(Xd).all().item()):
                self._all_finite = True
                kwargs = self.get_params()
                (self.labels_, self.probabilities_, self._single_linkage_tree,
                 self._condensed_tree, self._min_spanning_tree, self._neighbors,
                 self._core_distances) = _fast_hdbscan(Xd, None, return_trees=True,
                                                       condensed_records=True, **kwargs)
                self._condensed_tree = to_numpy_rec_array(self._condensed_tree)
                return self
        if sample_weight is not None:
            sample_weight = _check_sample_weight(sample_weight, X, dtype=np.float32)
        self._all_finite = bool(np.all(np.isfinite(X)))
        if not self._all_finite:
            finite_index = np.where(np.isfinite(X).sum(axis=1) == X.shape[1])[0]
            clean_data = X[finite_index]
            sample_weight = sample_weight[finite_index] if sample_weight is not None else None
            internal_to_raw = {x: y for x, y in zip(range(len(finite_index)), finite_index)}
            outliers = list(set(range(X.shape[0])) - set(finite_index))
        else:
            clean_data = X
        kwargs = self.get_params()
        (self.labels_, self.probabilities_, self._single_linkage_tree, self._condensed_tree,
         self._min_spanning_tree, self._neighbors, self._core_distances) = _fast_hdbscan(
            clean_data, None, return_trees=True, sample_weights=sample_weight,
            condensed_records=True, **kwargs)
        self._condensed_tree = to_numpy_rec_array(self._condensed_tree)
        if not self._all_finite:
            self._condensed_tree = remap_condensed_tree(self._condensed_tree, internal_to_raw,
                                                        outliers)
            self._single_linkage_tree = remap_single_linkage_tree(self._single_linkage_tree,
                                                                  internal_to_raw, outliers)
            new_labels = np.full(X.shape[0], -1)
            new_labels[finite_index] = self.labels_
            self.labels_ = new_labels
            new_probabilities = np.zeros(X.shape[0])
            new_probabilities[finite_index] = self.probabilities_
            self.probabilities_ = new_probabilities
        return self

    def fit_predict(self, X, y=None, **kwargs):
        self.fit(X, y=y, **kwargs)
        return self.labels_

    def dbscan_clustering(self, epsilon):
        """hdbscan.py:824."""
        if not hasattr(self, "_single_linkage_tree"):
            raise AttributeError("You first need to fit the HDBSCAN model before picking a "
                                 "DBSCAN clustering")
        from .cluster_trees import get_cluster_labelling_at_cut

        return get_cluster_labelling_at_cut(
            self._single_linkage_tree, epsilon,
            self.min_samples if self.min_samples is not None else self.min_cluster_size)
