"""The allocation-free linkage entry point (fhg_mst_to_linkage_tree_noalloc).

It serves callers that cannot allocate device memory while they run (a
process whose HBM is reserved up front by its own pool, or a loop that must
never enter the CUDA allocator): all of its scratch is a fixed device array
inside libfhg.so.  These tests call it through the C ABI and compare it with
the allocating entry point, fhg_mst_to_linkage_tree, on calls made back to
back (the second call finds the first call's data still in the scratch
array), and check that inputs above the fixed limit are refused.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

MAX_EDGES = 65536  # FHG_NOALLOC_MAX_EDGES in include/fhg.h


def _random_sorted_mst(m, seed):
    """A random spanning tree on m + 1 points, sorted by (weight, src, dst)."""
    rng = np.random.default_rng(seed)
    child = np.arange(1, m + 1)
    parent = (rng.random(m) * child).astype(np.int64)
    flip = rng.random(m) < 0.5
    src = np.where(flip, child, parent)
    dst = np.where(flip, parent, child)
    w = rng.random(m).astype(np.float32).astype(np.float64)  # duplicate weights occur
    mst = np.stack([src, dst, w], axis=1).astype(np.float64)
    return mst[np.lexsort((mst[:, 1], mst[:, 0], mst[:, 2]))]


def _call(lib, name, sorted_mst):
    import torch

    from fast_hdbscan_gb300 import _native

    m = sorted_mst.shape[0]
    d_in = torch.from_numpy(np.ascontiguousarray(sorted_mst)).cuda()
    d_out = torch.full((m, 4), -7.0, dtype=torch.float64, device="cuda")
    fn = getattr(lib, name)
    fn.restype = ctypes.c_int
    if name == "fhg_mst_to_linkage_tree":  # (sorted_mst, m, sample_weights, linkage, stream)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                       ctypes.c_void_p]
        rc = fn(ctypes.c_void_p(d_in.data_ptr()), m, None, ctypes.c_void_p(d_out.data_ptr()),
                _native.stream_ptr())
    else:
        fn.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
        rc = fn(ctypes.c_void_p(d_in.data_ptr()), m, ctypes.c_void_p(d_out.data_ptr()),
                _native.stream_ptr())
    torch.cuda.synchronize()
    return rc, d_out.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_back_to_back(engine):
    inputs = [
        np.load(os.path.join(GOLDEN, "blobs2d_20k.npz"))["sorted_mst"],
        _random_sorted_mst(MAX_EDGES, seed=1),
        np.load(os.path.join(GOLDEN, "vd3d_5k.npz"))["sorted_mst"],
        _random_sorted_mst(777, seed=2),
    ]
    for smst in inputs:
        rc_ref, ref = _call(engine, "fhg_mst_to_linkage_tree", smst)
        assert rc_ref == 0
        for _ in range(2):  # the same input twice in a row, then the next input
            rc, out = _call(engine, "fhg_mst_to_linkage_tree_noalloc", smst)
            assert rc == 0, engine.fhg_last_error()
            np.testing.assert_array_equal(out, ref)


def test_noalloc_matches_reference_linkage(engine):
    g = np.load(os.path.join(GOLDEN, "umap5d_5k.npz"))
    rc, out = _call(engine, "fhg_mst_to_linkage_tree_noalloc", g["sorted_mst"])
    assert rc == 0
    np.testing.assert_array_equal(out, g["linkage"])


def test_noalloc_rejects_inputs_above_the_limit(engine):
    rc, _ = _call(engine, "fhg_mst_to_linkage_tree_noalloc", _random_sorted_mst(MAX_EDGES + 1, 3))
    assert rc == 1  # FHG_ERR_INVALID
    assert b"FHG_NOALLOC_MAX_EDGES" in engine.fhg_last_error()
