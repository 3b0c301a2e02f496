"""The reference's kNN-graph back-end (nndescent.py, the route of Euclidean
data with more than 30 dimensions and no sample weights, hdbscan.py:446) on
the GPU.  pynndescent's approximate kNN graph is replaced by the engine's
exact brute-force kNN (bfloat16 tensor-core candidates, certified exact
float32 re-rank), so the graph is the one NNDescent converges towards; the
mutual-reachability Kruskal forest and its +inf bridges follow the reference.
Only the Euclidean metric is on the GPU path."""
import ctypes

import numpy as np

from . import _native


def _device_points(data):
    torch = _native._torch()
    if isinstance(data, torch.Tensor):
        return data.to(device="cuda", dtype=torch.float32).contiguous()
    return _native.to_device(np.ascontiguousarray(data, dtype=np.float32), np.float32)


def build_knn_graph(data, n_neighbors, metric="euclidean", metric_kwds=None, random_state=None):
    """nndescent.py:41: ``(index, knn_indices int32[n, n_neighbors],
    knn_distances float64[n, n_neighbors])`` without the point itself.  The
    index slot is None (there is no NNDescent search index); distances are
    the float64 square roots of the exact float32 squared distances."""
    if metric != "euclidean":
        raise NotImplementedError(f"metric={metric!r} is not on the GPU path")
    torch = _native._torch()
    Xd = _device_points(data)
    n, d = Xd.shape
    k = int(n_neighbors) + 1
    rd = torch.empty((n, k), dtype=torch.float32, device="cuda")
    ix = torch.empty((n, k), dtype=torch.int32, device="cuda")
    fb = ctypes.c_int64(0)
    _native.check(_native.load().fhg_highd_knn(_native.vptr(Xd), n, d, k, _native.vptr(rd),
                                               _native.vptr(ix), ctypes.byref(fb),
                                               _native.stream_ptr()))
    build_knn_graph.last_fallbacks = int(fb.value)
    rd_h = rd.cpu().numpy()
    return None, ix.cpu().numpy()[:, 1:].copy(), np.sqrt(rd_h[:, 1:].astype(np.float64))


def compute_mst_from_knn_graph(data, min_samples, metric="euclidean", metric_kwds=None,
                               knn_k=None, random_state=None):
    """nndescent.py:179: ``(mst_edges float64[n-1, 3], neighbors
    int32[n, min_samples], core_distances float64[n])``."""
    from .hdbscan import resolve_knn_graph_k

    if metric != "euclidean":
        raise NotImplementedError(f"metric={metric!r} is not on the GPU path")
    torch = _native._torch()
    Xd = _device_points(data)
    n, d = Xd.shape
    ms = int(min_samples)
    kk = resolve_knn_graph_k(ms, knn_k)
    edges = torch.empty((max(n - 1, 0), 3), dtype=torch.float64, device="cuda")
    nbrs = torch.empty((n, max(ms, 1)), dtype=torch.int32, device="cuda")
    core = torch.empty((n,), dtype=torch.float64, device="cuda")
    ncomp = ctypes.c_int64(0)
    _native.check(_native.load().fhg_knn_graph_mst(
        _native.vptr(Xd), n, d, ms, kk, _native.vptr(edges), _native.vptr(nbrs),
        _native.vptr(core), ctypes.byref(ncomp), _native.stream_ptr()))
    compute_mst_from_knn_graph.last_components = ncomp.value
    return edges.cpu().numpy(), nbrs.cpu().numpy(), core.cpu().numpy()
