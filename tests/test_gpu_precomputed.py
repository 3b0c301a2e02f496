"""GPU metric="precomputed" back-ends (precomputed.py:410 Boruvka, :479
Kruskal) against the reference fixtures and the CPU oracle.

Kruskal: MST edges (acceptance order, orientation, +inf bridges),
neighbours, float64 core distances, labels and probabilities are
bit-identical to the reference.  Boruvka: the engine returns the same
forest as for Kruskal (the oracle's, bit for bit); the reference's float32
Boruvka picks a forest of the same weights with its own equal-weight choices,
so against it the weights, neighbours, core distances and probabilities are
identical and the labels are the same partition.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from fast_hdbscan_gb300 import synthetic

pytestmark = pytest.mark.gpu

PRECOMPUTED = ["pc_knn3d_kr", "pc_knn3d_bo", "pc_disconnected_kr", "pc_disconnected_bo",
               "pc_coo_dups_kr", "pc_edge_empty_kr", "pc_edge_isolated_kr",
               "pc_edge_isolated_bo"]


def _graph(g):
    import scipy.sparse

    n = int(g["n"])
    return scipy.sparse.coo_matrix((g["data"], (g["rows"], g["cols"])), shape=(n, n))


def _same_partition(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert np.array_equal(a == -1, b == -1)
    pairs = set(zip(a[a >= 0].tolist(), b[b >= 0].tolist()))
    assert len(pairs) == len({x for x, _ in pairs}) == len({y for _, y in pairs})


@pytest.mark.parametrize("name", PRECOMPUTED)
def test_precomputed_vs_reference(engine, name):
    from fast_hdbscan_gb300 import HDBSCAN
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree, fast_hdbscan
    from oracle import oracle as O

    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    G = _graph(g)
    ms, mcs, algo = int(g["min_samples"]), int(g["min_cluster_size"]), str(g["algorithm"])
    mst, nbrs, core = compute_minimum_spanning_tree(G, min_samples=ms, metric="precomputed",
                                                    algorithm=algo)
    np.testing.assert_array_equal(nbrs, g["neighbors"])
    np.testing.assert_array_equal(core, g["core"])
    omst, _, _ = O.precomputed_kruskal(G, ms)
    np.testing.assert_array_equal(mst, omst)
    # the COO as given: converting it to CSR would sum its duplicate entries
    labels, probs = fast_hdbscan(G, min_samples=ms, min_cluster_size=mcs,
                                 metric="precomputed", algorithm=algo)
    if algo == "kruskal":
        np.testing.assert_array_equal(mst, g["mst"])
        np.testing.assert_array_equal(labels, g["labels"])
    else:
        np.testing.assert_array_equal(np.sort(mst[:, 2]), np.sort(g["mst"][:, 2]))
        _same_partition(labels, g["labels"])
    np.testing.assert_array_equal(probs, g["probabilities"])
    model = HDBSCAN(min_cluster_size=mcs, min_samples=ms, metric="precomputed",
                    algorithm=algo).fit(G)
    np.testing.assert_array_equal(model.labels_, labels)


@pytest.mark.parametrize("n,k,ms", [(100_000, 15, 10), (30_000, 6, 1)])
def test_precomputed_vs_oracle_synthetic(engine, n, k, ms):
    import scipy.sparse
    from scipy.spatial import cKDTree

    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree
    from oracle import oracle as O

    X = synthetic.varying_density(n, seed=51).astype(np.float64)
    d, ix = cKDTree(X).query(X, k=k + 1)
    G = scipy.sparse.csr_matrix((d[:, 1:].ravel(), (np.repeat(np.arange(n), k),
                                                    ix[:, 1:].ravel())), shape=(n, n))
    mst, nbrs, core = compute_minimum_spanning_tree(G, min_samples=ms, metric="precomputed",
                                                    algorithm="kruskal")
    omst, onb, ocore = O.precomputed_kruskal(G, ms)
    np.testing.assert_array_equal(core, ocore)
    np.testing.assert_array_equal(nbrs, onb)
    np.testing.assert_array_equal(mst, omst)


def test_precomputed_validation(engine):
    import scipy.sparse

    from fast_hdbscan_gb300.hdbscan import fast_hdbscan

    with pytest.raises(ValueError):  # not sparse
        fast_hdbscan(np.zeros((5, 5)), metric="precomputed")
    with pytest.raises(ValueError):  # negative weight
        fast_hdbscan(scipy.sparse.csr_matrix(-np.eye(5, k=1)), metric="precomputed")
    with pytest.raises(NotImplementedError):
        fast_hdbscan(scipy.sparse.csr_matrix(np.eye(5, k=1)), metric="precomputed",
                     sample_weights=np.ones(5))


def test_graph_to_device_matches_tocoo(engine):
    """The device entries of a CSR, CSC or COO graph (the compressed index
    expanded on the GPU) list exactly what X.tocoo() lists, in its order; the
    weight checks on the GPU raise the reference's errors."""
    import scipy.sparse

    from fast_hdbscan_gb300.hdbscan import HDBSCAN
    from fast_hdbscan_gb300.precomputed import graph_to_device

    rng = np.random.default_rng(3)
    dense = rng.random((60, 60)) * (rng.random((60, 60)) < 0.2)
    for X in (scipy.sparse.csr_matrix(dense), scipy.sparse.csc_matrix(dense),
              scipy.sparse.coo_matrix(dense), scipy.sparse.csr_matrix(dense).tolil()):
        rows, cols, data = graph_to_device(X)
        coo = X.tocoo()
        np.testing.assert_array_equal(rows.cpu().numpy(), coo.row)
        np.testing.assert_array_equal(cols.cpu().numpy(), coo.col)
        np.testing.assert_array_equal(data.cpu().numpy(), coo.data)
    bad = scipy.sparse.csr_matrix(dense)
    bad.data[3] = np.inf
    with pytest.raises(ValueError, match="finite"):
        HDBSCAN(metric="precomputed").fit(bad)
    bad.data[3] = -1.0
    with pytest.raises(ValueError, match="non-negative"):
        HDBSCAN(metric="precomputed").fit(bad)
