"""GPU Boruvka behind the reference's ``parallel_boruvka`` (boruvka.py:542)."""
import ctypes

import numpy as np

from . import _native


def parallel_boruvka(tree, n_threads=None, min_samples=10,
                     sample_weights=np.zeros(1, dtype=np.float32), reproducible=False):
    """Minimum spanning tree of the mutual-reachability graph.

    Returns ``(edges float64[n-1, 3], neighbors int32[n, max(min_samples, 1)],
    core_distances float32[n])`` like the reference.  ``n_threads`` and
    ``reproducible`` are accepted for signature compatibility: the GPU result
    is deterministic in every mode.
    """
    torch = _native._torch()
    sample_weights = np.asarray(sample_weights)
    if sample_weights.shape[0] > 1:
        raise NotImplementedError("sample_weights are not supported by the GPU engine yet")
    n = tree.data.shape[0]
    ms = int(min_samples)
    kcols = ms if ms > 1 else 1
    edges = torch.empty((max(n - 1, 0), 3), dtype=torch.float64, device="cuda")
    nbrs = torch.empty((n, kcols), dtype=torch.int32, device="cuda")
    core = torch.empty((n,), dtype=torch.float32, device="cuda")
    rounds = ctypes.c_int32(0)
    lib = _native.load()
    _native.check(lib.fhg_index_boruvka(tree.index.handle, ms, _native.dptr(edges),
                                        _native.dptr(nbrs), _native.dptr(core),
                                        ctypes.byref(rounds), _native.stream_ptr()))
    parallel_boruvka.last_rounds = rounds.value
    return edges.cpu().numpy(), nbrs.cpu().numpy(), core.cpu().numpy()
