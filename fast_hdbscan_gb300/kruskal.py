"""GPU kNN-graph Kruskal behind the reference's ``kruskal_mst_from_feature_matrix``
(kruskal.py:821), the algorithm="kruskal" back-end for Euclidean features."""
import ctypes

import numpy as np

from . import _native


def kruskal_query_k(min_samples, knn_k, sample_weights=None):
    """kruskal.py:981-1007: the kNN query size of ``_kruskal_mst_knn``, the
    point itself included."""
    if sample_weights is not None:
        mean_sw = float(np.mean(np.asarray(sample_weights, dtype=np.float32)))
        return max(int(knn_k), int(2 * min_samples / mean_sw)) + 1
    if min_samples > 1:
        return max(int(knn_k), int(min_samples)) + 1
    return int(knn_k) + 1


def kruskal_mst_from_feature_matrix(numba_tree, min_samples, knn_k=None, sample_weights=None,
                                    reproducible=False, cannot_link=None,
                                    validate_cannot_link=True, cannot_link_groups=None):
    """Kruskal MST for feature data (kruskal.py:821).

    Returns ``(mst_edges float64[n-1, 3], neighbors int32[n, k], core_distances
    float64[n])`` like the reference: the minimum spanning forest of the kNN
    graph's mutual-reachability edges in Kruskal's acceptance order, then
    +inf bridges between the components of a disconnected kNN graph.
    ``reproducible`` is accepted for signature compatibility (Kruskal is
    deterministic).  The exact full-pairwise variant (``knn_k=None``, an
    O(n^2) float64 distance matrix) and cannot-link constraints are not on the
    GPU path.
    """
    if knn_k is None:
        raise NotImplementedError(
            "algorithm='kruskal' with knn_k=None (exact MST from the full pairwise distance "
            "matrix) is not on the GPU path; pass an integer knn_k or use algorithm='boruvka'")
    if cannot_link is not None or cannot_link_groups is not None:
        raise NotImplementedError("cannot-link constraints are not on the GPU path")
    torch = _native._torch()
    n = numba_tree.data.shape[0]
    ms = int(min_samples)
    w = None
    if sample_weights is not None:
        w = np.ascontiguousarray(sample_weights, dtype=np.float32)
    kq = kruskal_query_k(ms, knn_k, w)
    if kq > 2048:  # kNN lists of the spatial index: up to 64 in registers, longer in shared memory
        raise NotImplementedError(f"a kNN query of {kq} neighbours exceeds the GPU kNN's 2048")
    cols = kq - 1 if w is not None else (ms if ms > 1 else 1)
    edges = torch.empty((max(n - 1, 0), 3), dtype=torch.float64, device="cuda")
    nbrs = torch.empty((n, cols), dtype=torch.int32, device="cuda")
    core = torch.empty((n,), dtype=torch.float64, device="cuda")
    d_w = torch.from_numpy(w).cuda() if w is not None else None
    ncomp = ctypes.c_int64(0)
    _native.check(_native.load().fhg_index_kruskal_knn(
        numba_tree.index.handle, ms, kq, _native.vptr(d_w), _native.dptr(edges),
        _native.vptr(nbrs), _native.dptr(core), ctypes.byref(ncomp), _native.stream_ptr()))
    kruskal_mst_from_feature_matrix.last_components = ncomp.value
    return edges.cpu().numpy(), nbrs.cpu().numpy(), core.cpu().numpy()
