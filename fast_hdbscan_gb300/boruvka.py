"""GPU Boruvka behind the reference's ``parallel_boruvka`` (boruvka.py:542)."""
import ctypes

import numpy as np

from . import _native


def weighted_knn_k(sample_weights, min_samples):
    """boruvka.py:561-563: the weighted path queries
    k = int(2 * min_samples / mean(sample_weights)) neighbours.  The mean is
    taken in float64; the reference accumulates float32, which can only move k
    when 2 * min_samples / mean lies within rounding of an integer."""
    w = np.asarray(sample_weights, dtype=np.float32)
    mean = float(np.sum(w, dtype=np.float64)) / w.shape[0]
    return int(2 * (min_samples / mean))


def parallel_boruvka(tree, n_threads=None, min_samples=10,
                     sample_weights=np.zeros(1, dtype=np.float32), reproducible=False):
    """Minimum spanning tree of the mutual-reachability graph.

    Returns ``(edges float64[n-1, 3], neighbors int32[n, k-1],
    core_distances float32[n])`` like the reference (k = min_samples + 1, at
    least 2; with sample weights, weighted_knn_k).  ``n_threads`` is accepted
    for signature compatibility.  The GPU result is deterministic either way;
    ``reproducible`` selects whose choices it makes among edges of equal
    weight: False (default), a total order on point indices; True, the
    reference's own -- its sequential rule, its KD-tree's traversal order and
    its kNN query's order among equal distances (fhg_set_tie_rule) -- so that
    the tree and the neighbour matrix equal the reference's, duplicates
    included.
    """
    torch = _native._torch()
    sample_weights = np.asarray(sample_weights, dtype=np.float32)
    n = tree.data.shape[0]
    ms = int(min_samples)
    weighted = sample_weights.shape[0] > 1
    wk = weighted_knn_k(sample_weights, ms) if weighted else 0
    kcols = max(wk - 1, 0) if weighted else (ms if ms > 1 else 1)
    edges = torch.empty((max(n - 1, 0), 3), dtype=torch.float64, device="cuda")
    nbrs = torch.empty((n, kcols), dtype=torch.int32, device="cuda")
    core = torch.empty((n,), dtype=torch.float32, device="cuda")
    d_w = torch.from_numpy(np.ascontiguousarray(sample_weights)).cuda() if weighted else None
    rounds = ctypes.c_int32(0)
    lib = _native.load()
    with _native.tie_rule(bool(reproducible)):
        _native.check(lib.fhg_index_boruvka(tree.index.handle, ms, _native.vptr(d_w), wk,
                                            _native.dptr(edges), _native.vptr(nbrs),
                                            _native.dptr(core), ctypes.byref(rounds),
                                            _native.stream_ptr()))
    parallel_boruvka.last_rounds = rounds.value
    return edges.cpu().numpy(), nbrs.cpu().numpy(), core.cpu().numpy()
