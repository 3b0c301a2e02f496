"""ctypes binding of libfhg.so (the C ABI declared in include/fhg.h).

The library is built in-tree by ``fast_hdbscan_gb300.build`` and loaded from
``fast_hdbscan_gb300/_lib/libfhg.so``.  There is no fallback: if the library
or a CUDA device is missing, every engine call raises.
"""
import contextlib
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libfhg.so")

FHG_OK = 0
FHG_ERR_INVALID = 1
FHG_ERR_OOM = 2
FHG_ERR_CUDA = 3
FHG_ERR_NO_CONVERGENCE = 4
FHG_ERR_UNSUPPORTED = 5

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_INT = ctypes.c_int
_D = ctypes.c_double

# name -> (restype, argtypes); kept in the order of include/fhg.h
SIGNATURES = {
    "fhg_last_error": (ctypes.c_char_p, []),
    "fhg_abi_version": (_INT, []),
    "fhg_set_tie_rule": (_INT, [_INT]),
    "fhg_set_highd_kernel": (_INT, [_INT]),
    "fhg_release_cached_memory": (_INT, []),
    "fhg_index_build": (_INT, [_P, _I64, _I32, _P, ctypes.POINTER(_P)]),
    "fhg_reference_kdtree_levels": (_I32, [_I64]),
    "fhg_reference_kdtree": (_INT, [_P, _I64, _I32, _P, _P, _P]),
    "fhg_index_free": (_INT, [_P, _P]),
    "fhg_index_shape": (_INT, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I32)]),
    "fhg_index_knn": (_INT, [_P, _I32, _P, _P, _P]),
    "fhg_index_boruvka": (_INT, [_P, _I32, _P, _I32, _P, _P, _P, ctypes.POINTER(_I32), _P]),
    "fhg_sort_mst": (_INT, [_P, _I64, _P, _P]),
    "fhg_clusters_from_mst": (_INT, [_P, _I64, _I64, _I32, _D, _INT, _D, _D, _P, _P, _P, _P,
                                     _P, _P, _P, _P, _P, ctypes.POINTER(_I64), _P,
                                     ctypes.POINTER(_I64), _P]),
    "fhg_mst_to_linkage_tree": (_INT, [_P, _I64, _P, _P, _P]),
    "fhg_condense_tree": (_INT, [_P, _I64, _I64, _D, _P, _P, _P, _P, _P, ctypes.POINTER(_I64),
                                 _P]),
    "fhg_extract_eom_clusters": (_INT, [_P, _P, _P, _P, _I64, _D, _INT, _P,
                                        ctypes.POINTER(_I64), _P]),
    "fhg_label_points": (_INT, [_P, _P, _P, _P, _I64, _P, _I64, _D, _I64, _P, _P, _P]),
    "fhg_cluster_tree_leaves": (_INT, [_P, _P, _P, _P, _I64, _P, ctypes.POINTER(_I64), _P]),
    "fhg_membership_strengths": (_INT, [_P, _P, _P, _P, _I64, _P, _I64, _P, _I64, _P, _P]),
    "fhg_condensed_record_array": (_INT, [_P, _P, _P, _P, _I64, _P, _P]),
    "fhg_simplify_hierarchy": (_INT, [_P, _P, _P, _P, _I64, _D, _P, _P, _P, _P,
                                      ctypes.POINTER(_I64), _P]),
    "fhg_cluster_epsilon_search": (_INT, [_P, _P, _P, _P, _I64, _P, _I64, _D, _P,
                                          ctypes.POINTER(_I64), _P]),
    "fhg_labelling_at_cut": (_INT, [_P, _I64, _D, _I64, _P, _P]),
    "fhg_hdbscan_fit_batch": (_INT, [_I64, _P, _P, _P, _P, _P, _I32, _D, _INT, _P, _P, _I32,
                                     _P, _P]),
    "fhg_hdbscan_fit": (_INT, [_P, _I64, _I32, _I32, _I64, _I32, _D, _INT, _D, _D, _P, _I32,
                               _P, _P, _P, _P, _P, _P, _P, _P, ctypes.POINTER(_I64),
                               _P, _P, _P, ctypes.POINTER(_I64), _P]),
    "fhg_hdbscan_fit_kruskal": (_INT, [_P, _I64, _I32, _I32, _I32, _I32, _I64, _I32, _D, _INT,
                                       _D, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                       ctypes.POINTER(_I64), _P, _P, _P, ctypes.POINTER(_I64),
                                       _P]),
    "fhg_hdbscan_fit_precomputed": (_INT, [_P, _P, _P, _I64, _I64, _I32, _I32, _I64, _I32, _D,
                                           _INT, _D, _D, _P, _P, _P, _P, _P, _P, _P, _P,
                                           ctypes.POINTER(_I64), _P, _P, _P,
                                           ctypes.POINTER(_I64), _P]),
    "fhg_precomputed_mst": (_INT, [_P, _P, _P, _I64, _I64, _I32, _I32, _P, _P, _P,
                                   ctypes.POINTER(_I64), _P]),
    "fhg_index_kruskal_knn": (_INT, [_P, _I32, _I32, _P, _P, _P, _P, ctypes.POINTER(_I64), _P]),
    "fhg_hdbscan_fit_export": (_INT, [_P, _I64, _I32, _I32, _I64, _I32, _D, _INT, _D, _D, _P,
                                      _I32, _P, _P, _P, _P, _P, _P, _P, _P,
                                      ctypes.POINTER(_I64), _P, _P, _P, ctypes.POINTER(_I64),
                                      _P, _P, _P, _P, _P, _P, _P]),
    "fhg_radius_param_count": (_INT, []),
    "fhg_radius_features": (_INT, [_P, _P, _P]),
    "fhg_radius_targets": (_INT, [_P, _I32, _P, _P]),
    "fhg_radius_init": (_INT, [_P, _P, _P, _I64, ctypes.c_uint64, _P]),
    "fhg_radius_forward": (_INT, [_P, _P, _I64, _P, _P]),
    "fhg_radius_backward": (_INT, [_P, _P, _P, _P, _I64, _P, _P, _P]),
    "fhg_radius_train": (_INT, [_P, _P, _P, _I64, _I32, _I32, ctypes.c_float, ctypes.c_uint64,
                                _P, _P]),
    "fhg_radius_use": (_INT, [_P, ctypes.c_float]),
    "fhg_radius_fallbacks": (_INT, [ctypes.POINTER(_I64), _P]),
    "fhg_index_knn_radius": (_INT, [_P, _I32, _P, ctypes.c_float, _P, _P, ctypes.POINTER(_I64),
                                    _P]),
    "fhg_highd_knn": (_INT, [_P, _I64, _I32, _I32, _P, _P, ctypes.POINTER(_I64), _P]),
    "fhg_knn_graph_mst": (_INT, [_P, _I64, _I32, _I32, _I32, _P, _P, _P, ctypes.POINTER(_I64),
                                 _P]),
    "fhg_hdbscan_fit_knn_graph": (_INT, [_P, _I64, _I32, _I32, _I32, _I64, _I32, _D, _INT, _D,
                                         _D, _P, _P, _P, _P, _P, _P, _P, _P,
                                         ctypes.POINTER(_I64), _P, _P, _P,
                                         ctypes.POINTER(_I64), _P]),
    "fhg_propagate_labels": (_INT, [_I64, _P, _P, _P, _P, _P, _P, _P]),
    "fhg_core_graphs": (_INT, [_I64, _I32, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P,
                               _P, _P, ctypes.POINTER(_I64), _P]),
    "fhg_core_graph_mst": (_INT, [_P, _P, _P, _P, _I64, _P, ctypes.POINTER(_I64), _P]),
    "fhg_knn_scan_count": (_INT, [_P, _I32, _P, ctypes.c_float, ctypes.POINTER(_I64),
                                  ctypes.POINTER(_I64), _P]),
}

_lib = None


class EngineError(RuntimeError):
    pass


def load(path=LIB_PATH):
    """Loads libfhg.so and binds every exported entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise EngineError(
            f"{path} is missing: build the CUDA engine first "
            "(python -c 'import fast_hdbscan_gb300.build as b; b.build()')")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc):
    if rc == FHG_OK:
        return
    msg = (load().fhg_last_error() or b"").decode(errors="replace")
    if rc == FHG_ERR_INVALID:
        raise ValueError(msg)
    if rc == FHG_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if rc == FHG_ERR_OOM:
        raise MemoryError(msg)
    raise EngineError(f"fhg error {rc}: {msg}")


def release_cached_memory():
    """Returns the device memory the engine's pool keeps cached between calls."""
    check(load().fhg_release_cached_memory())


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise EngineError("the GB300 HDBSCAN engine needs a CUDA device")
    return torch


def stream_ptr():
    return _P(_torch().cuda.current_stream().cuda_stream)


def dptr(t):
    """Device pointer of a contiguous CUDA tensor."""
    assert t.is_cuda and t.is_contiguous()
    return _P(t.data_ptr())


def to_device(a, dtype):
    torch = _torch()
    a = np.ascontiguousarray(a, dtype=dtype)
    return torch.from_numpy(a).to("cuda", non_blocking=False)


def empty(shape, dtype):
    """Uninitialised CUDA tensor with a numpy dtype."""
    torch = _torch()
    tdt = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
           np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64}[np.dtype(dtype)]
    if isinstance(shape, int):
        shape = (shape,)
    shape = tuple(max(int(s), 0) for s in shape)
    n = int(np.prod(shape)) if shape else 1
    if n == 0:  # keep a valid device pointer for zero-size outputs
        return torch.empty((1,), dtype=tdt, device="cuda")[:0].reshape(shape)
    return torch.empty(shape, dtype=tdt, device="cuda")


def vptr(t):
    """Device pointer of a contiguous CUDA tensor, or NULL for None."""
    if t is None:
        return _P()
    assert t.is_cuda and t.is_contiguous()
    return _P(t.data_ptr())


def hptr(t):
    """Host pointer of a contiguous CPU tensor (pinned or pageable), or NULL
    for None."""
    if t is None:
        return _P()
    assert not t.is_cuda and t.is_contiguous()
    return _P(t.data_ptr())


class Index:
    """Owner of an fhg_index handle (the spatial index of a point set)."""

    def __init__(self, X_dev):
        self._handle = None
        lib = load()
        n, d = X_dev.shape
        h = _P()
        check(lib.fhg_index_build(dptr(X_dev), n, d, stream_ptr(), ctypes.byref(h)))
        self._handle = h
        self.n, self.d = int(n), int(d)

    @property
    def handle(self):
        return self._handle

    def close(self):
        if self._handle is not None and _lib is not None:
            _lib.fhg_index_free(self._handle, stream_ptr())
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@contextlib.contextmanager
def tie_rule(reference):
    """Runs the engine calls made inside the block, on this thread, with the
    reference's Boruvka tie choices (``reference=True``: the ``reproducible``
    flag) or the canonical total order (the default), then restores the
    previous rule."""
    lib = load()
    old = lib.fhg_set_tie_rule(1 if reference else 0)
    try:
        yield
    finally:
        lib.fhg_set_tie_rule(old)
