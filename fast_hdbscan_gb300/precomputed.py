"""GPU minimum spanning forests of precomputed sparse graphs behind the
reference's precomputed.py (metric="precomputed")."""
import ctypes

import numpy as np

from . import _native


def validate_precomputed_sparse_graph(X, check_values=True):
    """precomputed.py:30: a square scipy sparse matrix with finite,
    non-negative stored weights (check_values=False: the shape only, the
    weights being checked on the GPU by graph_to_device)."""
    import scipy.sparse

    if not scipy.sparse.issparse(X):
        raise ValueError(
            "When metric='precomputed', X must be a scipy sparse matrix "
            "(CSR, CSC, or COO). Got: %s" % type(X).__name__)
    if X.ndim != 2 or X.shape[0] != X.shape[1]:
        raise ValueError("When metric='precomputed', X must be a square matrix. "
                         "Got shape: %s" % str(X.shape))
    if check_values:
        _check_weights(np.asarray(X.data), np)


def _check_weights(data, xp):
    """The stored weights' checks of precomputed.py:30, on NumPy or torch
    arrays."""
    if len(data) > 0:
        if bool(xp.any(~xp.isfinite(data))):
            raise ValueError("When metric='precomputed', all stored edge weights must be "
                             "finite. Found NaN or Inf values.")
        if bool(xp.any(data < 0)):
            raise ValueError("When metric='precomputed', all stored edge weights must be "
                             "non-negative. Found negative values.")


def graph_to_device(X):
    """The stored entries of a scipy sparse graph as device arrays (rows
    int32, cols int32, weights float64) in the order X.tocoo() lists them:
    row by row for CSR, column by column for CSC, as stored for COO.  The
    compressed index of CSR / CSC is expanded on the GPU, and the weights are
    checked there."""
    torch = _native._torch()
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dt)).cuda()  # noqa: E731
    if X.format in ("csr", "csc"):
        ptr = dev(X.indptr, np.int64)
        major = torch.repeat_interleave(
            torch.arange(X.shape[0] if X.format == "csr" else X.shape[1], dtype=torch.int32,
                         device="cuda"), ptr[1:] - ptr[:-1])
        minor = dev(X.indices, np.int32)
        rows, cols = (major, minor) if X.format == "csr" else (minor, major)
    else:
        coo = X.tocoo()
        rows, cols = dev(coo.row, np.int32), dev(coo.col, np.int32)
        X = coo
    data = dev(X.data, np.float64)
    _check_weights(data, torch)
    return rows.contiguous(), cols.contiguous(), data


def _precomputed_mst(X, min_samples, algorithm):
    torch = _native._torch()
    validate_precomputed_sparse_graph(X, check_values=False)
    n = X.shape[0]
    k = max(1, int(min_samples))
    rows, cols, data = graph_to_device(X)
    edges = torch.empty((max(n - 1, 0), 3), dtype=torch.float64, device="cuda")
    nbrs = torch.empty((n, k), dtype=torch.int32, device="cuda")
    core = torch.empty((n,), dtype=torch.float64, device="cuda")
    ncomp = ctypes.c_int64(0)
    V = _native.vptr
    _native.check(_native.load().fhg_precomputed_mst(
        V(rows), V(cols), V(data), int(data.numel()), n, int(min_samples),
        1 if algorithm == "kruskal" else 0, V(edges), V(nbrs), V(core), ctypes.byref(ncomp),
        _native.stream_ptr()))
    return edges.cpu().numpy(), nbrs.cpu().numpy(), core.cpu().numpy()


def compute_mst_from_precomputed_sparse(X, min_samples):
    """precomputed.py:410 (the metric="precomputed" Boruvka back-end):
    ``(edges float64[n-1, 3], neighbors int32[n, max(1, min_samples)],
    core_distances float64[n])``.  The forest is the minimum spanning forest
    of the float64 mutual-reachability weights, in Kruskal's order, with +inf
    bridges between components; the reference's float32 Boruvka returns a
    forest of the same weights, whose equal-weight choices and order are its
    own."""
    return _precomputed_mst(X, min_samples, "boruvka")


def compute_mst_from_precomputed_sparse_kruskal(X, min_samples, cannot_link=None,
                                                validate_cannot_link=True,
                                                cannot_link_groups=None):
    """precomputed.py:479 (the metric="precomputed" Kruskal back-end), without
    cannot-link constraints (not on the GPU path)."""
    if cannot_link is not None or cannot_link_groups is not None:
        raise NotImplementedError("cannot-link constraints are not on the GPU path")
    return _precomputed_mst(X, min_samples, "kruskal")
