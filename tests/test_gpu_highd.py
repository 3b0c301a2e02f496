"""The high-dimensional route (hdbscan.py:446 -> nndescent.py:179
compute_mst_from_knn_graph) on the GPU's exact brute-force kNN.

* The tensor-core kNN with its certified float32 re-rank equals the spatial
  index's kNN bit for bit where both exist (d <= 32) and the CPU oracle's
  exact kNN at 64 dimensions, including inputs whose certificate fails
  (duplicated points) and go through the exact fallback.
* Core distances agree with a float64 brute force within 1e-5 relative.
* The kNN-graph forest and the whole fit equal the oracle's Kruskal on the
  oracle's exact kNN lists (pynndescent's graph is approximate; the exact
  graph is what it converges to).
"""
import ctypes
import os

import numpy as np
import pytest

from fast_hdbscan_gb300 import synthetic

pytestmark = pytest.mark.gpu
NTH = os.cpu_count() or 1


def _highd(X, k):
    import torch

    from fast_hdbscan_gb300 import _native

    Xd = torch.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()
    n, d = X.shape
    rd = torch.empty((n, k), dtype=torch.float32, device="cuda")
    ix = torch.empty((n, k), dtype=torch.int32, device="cuda")
    fb = ctypes.c_int64(0)
    _native.check(_native.load().fhg_highd_knn(_native.vptr(Xd), n, d, k, _native.vptr(rd),
                                               _native.vptr(ix), ctypes.byref(fb),
                                               _native.stream_ptr()))
    return rd.cpu().numpy(), ix.cpu().numpy(), fb.value


@pytest.mark.parametrize("d,k", [(12, 11), (24, 31), (32, 16), (3, 5)])
def test_highd_knn_equals_spatial_knn(engine, d, k):
    from fast_hdbscan_gb300.numba_kdtree import build_kdtree, parallel_tree_query

    X = synthetic.aniso_highdim(n=6000, seed=20 + d, dim=d, n_comp=8)
    rd, ix, fb = _highd(X, k)
    rd_t, ix_t = parallel_tree_query(build_kdtree(X), X, k=k, output_rdist=True)
    np.testing.assert_array_equal(ix, ix_t)
    np.testing.assert_array_equal(rd, rd_t)


@pytest.mark.parametrize("d", [40, 64, 96])
def test_highd_knn_equals_oracle(engine, d):
    from oracle import oracle as O

    X = synthetic.aniso_highdim(n=8000, seed=30 + d, dim=d, n_comp=10)
    k = 31
    rd, ix, fb = _highd(X, k)
    rd_o, ix_o = O.tree_query(O.build_kdtree(X), k, mode=1, nthreads=NTH)
    np.testing.assert_array_equal(ix, ix_o)
    np.testing.assert_array_equal(rd, rd_o)
    print("d=%d fallbacks %d of %d" % (d, fb, len(X)))
    # float64 brute force on a sample of queries: the k-th distance
    rows = np.random.default_rng(d).choice(len(X), 64, replace=False)
    X64 = X.astype(np.float64)
    for i in rows:
        dd = np.sort(((X64 - X64[i]) ** 2).sum(1))
        assert abs(np.sqrt(rd[i, -1]) - np.sqrt(dd[k - 1])) <= 1e-5 * np.sqrt(dd[k - 1])


def test_highd_knn_fallback_path(engine):
    """Many copies of a few points: the L-th candidate estimate is 0, no
    certificate holds, and the exact fallback answers every such query."""
    from oracle import oracle as O

    rng = np.random.default_rng(7)
    base = rng.normal(0, 1, (20, 48)).astype(np.float32)
    X = np.concatenate([np.repeat(base, 60, axis=0),
                        rng.normal(0, 3, (800, 48)).astype(np.float32)])
    X = X[rng.permutation(len(X))]
    rd, ix, fb = _highd(X, 16)
    assert fb >= 1200
    rd_o, ix_o = O.tree_query(O.build_kdtree(X), 16, mode=1, nthreads=NTH)
    np.testing.assert_array_equal(ix, ix_o)
    np.testing.assert_array_equal(rd, rd_o)


@pytest.mark.parametrize("ms,knn_k", [(10, None), (5, 20), (1, None)])
def test_knn_graph_mst_equals_oracle(engine, ms, knn_k):
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree, resolve_knn_graph_k
    from oracle import oracle as O

    X = synthetic.aniso_highdim(n=5000, seed=41, dim=64, n_comp=6)
    mst, nbrs, core = compute_minimum_spanning_tree(X, min_samples=ms, knn_k=knn_k)
    kk = resolve_knn_graph_k(ms, knn_k)
    e_o, n_o, c_o = O.kruskal_knn(O.build_kdtree(X), ms, kk, mode=1, nthreads=NTH)
    np.testing.assert_array_equal(mst, e_o)
    np.testing.assert_array_equal(nbrs, n_o)
    np.testing.assert_array_equal(core, c_o)


def test_knn_graph_fit_equals_oracle(engine):
    from fast_hdbscan_gb300 import HDBSCAN
    from fast_hdbscan_gb300.hdbscan import resolve_knn_graph_k
    from oracle import oracle as O

    X = synthetic.aniso_highdim(n=12000, seed=42, dim=64, n_comp=12)
    est = HDBSCAN(min_samples=10, min_cluster_size=100).fit(X)
    mst, _, _ = O.kruskal_knn(O.build_kdtree(X), 10, resolve_knn_graph_k(10, None), mode=1,
                              nthreads=NTH)
    labels, probs, *_ = O.clusters_from_spanning_tree(mst, min_cluster_size=100)
    np.testing.assert_array_equal(est.labels_, labels)
    np.testing.assert_array_equal(est.probabilities_, probs)
    assert len(set(labels.tolist()) - {-1}) >= 2


@pytest.mark.parametrize("n,d,k", [(100, 40, 5), (1000, 20, 31), (4999, 64, 31),
                                   (20_000, 64, 16), (40_000, 48, 31), (3000, 64, 32),
                                   (3000, 64, 36)])
def test_tcgen05_pipeline_equals_mma_sync_kernel(engine, n, d, k):
    """The tcgen05 candidate pipeline (TMA, tensor memory, epilogue
    selection) and the mma.sync kernel give the same certified kNN, equal to
    the oracle's exact kNN -- on ragged last tiles, on fewer points than
    one tile, and on both sides of the largest candidate buffers the
    pipeline's shared memory holds (k 32 runs on tcgen05, k 36 falls back)."""
    from fast_hdbscan_gb300 import _native
    from oracle import oracle as O

    X = synthetic.aniso_highdim(n=n, seed=50 + d, dim=d, n_comp=7)
    lib = _native.load()
    assert lib.fhg_set_highd_kernel(0) == 0
    rd_tc, ix_tc, fb_tc = _highd(X, k)
    lib.fhg_set_highd_kernel(1)
    try:
        rd_ms, ix_ms, fb_ms = _highd(X, k)
    finally:
        lib.fhg_set_highd_kernel(0)
    np.testing.assert_array_equal(ix_tc, ix_ms)
    np.testing.assert_array_equal(rd_tc, rd_ms)
    rd_o, ix_o = O.tree_query(O.build_kdtree(X), k, mode=1, nthreads=NTH)
    np.testing.assert_array_equal(ix_tc, ix_o)
    np.testing.assert_array_equal(rd_tc, rd_o)
    print("n=%d d=%d k=%d: fallbacks tcgen05 %d, mma.sync %d" % (n, d, k, fb_tc, fb_ms))
