"""GPU kNN-graph Kruskal back-end (algorithm="kruskal" with an integer knn_k,
kruskal.py:950) against the reference fixtures and the CPU oracle.

The MST edge list is compared exactly: Kruskal's acceptance order (float64
weight, then edge position), the (row point, neighbour) orientation of every
edge and the +inf bridges that join a disconnected kNN graph.  Against the
reference fixtures (tie-free inputs) the neighbours, float64 core distances,
labels and probabilities are bit-identical too; on larger synthetic inputs
the oracle runs with the canonical kNN tie order the GPU kNN uses.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from fast_hdbscan_gb300 import synthetic

pytestmark = pytest.mark.gpu

KRUSKAL = ["kr_blobs200_k10", "kr_vd3d_5k_k8", "kr_blobs2d_2k_ms1", "kr_vd3d_3k_w",
           "kr_edge_n3", "kr_edge_ms_gt_k"]


def _golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.mark.parametrize("name", KRUSKAL)
def test_kruskal_vs_reference(engine, name):
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree, fast_hdbscan

    g = _golden(name)
    X = g["X"]
    ms, mcs, knn_k = int(g["min_samples"]), int(g["min_cluster_size"]), int(g["knn_k"])
    w = g["sample_weights"] if "sample_weights" in g else None
    mst, nbrs, core = compute_minimum_spanning_tree(X, min_samples=ms, sample_weights=w,
                                                    algorithm="kruskal", knn_k=knn_k)
    np.testing.assert_array_equal(mst, g["mst"])
    np.testing.assert_array_equal(nbrs, g["neighbors"])
    np.testing.assert_array_equal(core, g["core"])
    labels, probs = fast_hdbscan(X, min_samples=ms, min_cluster_size=mcs, sample_weights=w,
                                 algorithm="kruskal", knn_k=knn_k)
    np.testing.assert_array_equal(labels, g["labels"])
    np.testing.assert_array_equal(probs, g["probabilities"])


@pytest.mark.parametrize("gen,n,ms,knn_k,weighted", [
    ("varying_density", 100_000, 10, 16, False),
    ("blobs_2d", 60_000, 1, 4, False),
    ("umap_like", 40_000, 8, 12, False),
    ("varying_density", 50_000, 6, 10, True),
    ("varying_density", 30_000, 70, 16, False),  # kNN lists longer than 64
    ("blobs_2d", 20_000, 10, 150, False),
])
def test_kruskal_vs_oracle_synthetic(engine, gen, n, ms, knn_k, weighted):
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree
    from oracle import oracle as O

    X = getattr(synthetic, gen)(n, seed=31)
    w = None
    if weighted:
        w = (np.random.default_rng(32).integers(32, 129, n) / 64.0).astype(np.float32)
    mst, nbrs, core = compute_minimum_spanning_tree(X, min_samples=ms, sample_weights=w,
                                                    algorithm="kruskal", knn_k=knn_k)
    omst, onb, ocore = O.kruskal_knn(O.build_kdtree(X), ms, knn_k, mode=1, nthreads=8,
                                     sample_weights=w)
    np.testing.assert_array_equal(core, ocore)
    np.testing.assert_array_equal(nbrs, onb)
    np.testing.assert_array_equal(mst, omst)
    assert mst.shape == (n - 1, 3)


def test_kruskal_estimator_and_trees(engine):
    """HDBSCAN(algorithm="kruskal", knn_k=...) stores the same labels as
    fast_hdbscan and the trees of clusters_from_spanning_tree on its MST."""
    from fast_hdbscan_gb300 import HDBSCAN
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan

    g = _golden("kr_vd3d_5k_k8")
    X = g["X"]
    model = HDBSCAN(min_cluster_size=40, min_samples=10, algorithm="kruskal", knn_k=8).fit(X)
    np.testing.assert_array_equal(model.labels_, g["labels"])
    res = fast_hdbscan(X, min_samples=10, min_cluster_size=40, algorithm="kruskal", knn_k=8,
                       return_trees=True)
    np.testing.assert_array_equal(res[0], g["labels"])
    np.testing.assert_array_equal(res[5], g["neighbors"])
    np.testing.assert_array_equal(res[6], g["core"])
    assert np.isinf(res[4][:, 2]).sum() == np.isinf(g["mst"][:, 2]).sum()
