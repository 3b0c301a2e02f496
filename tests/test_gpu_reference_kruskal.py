"""The reference's Kruskal and precomputed-graph tests
(fast_hdbscan/tests/test_kruskal.py:89-505, the cases without cannot-link
constraints or the full-pairwise knn_k=None back-end), restated against the
GPU engine.

The small graphs are the reference's own.  Its feature-matrix cases draw 60
points from scikit-learn, which is not needed here: the committed fixture
``blobs200`` (the reference's test_hdbscan.py data) stands in, with its
complete float32 distance graph for the precomputed cases.  For a
precomputed graph the engine's Boruvka returns the Kruskal forest, so each
graph case also checks algorithm="boruvka" against algorithm="kruskal".
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _csr(rows, cols, data, n):
    from scipy import sparse

    return sparse.csr_matrix((data, (rows, cols)), shape=(n, n), dtype=np.float64)


def _X():
    return np.load(os.path.join(GOLDEN, "blobs200.npz"))["X"]


def _complete_graph(X):
    """Every pairwise Euclidean distance of the float32 points (the zero
    diagonal is not stored)."""
    from scipy import sparse

    Y = X.astype(np.float32).astype(np.float64)
    D = np.sqrt(((Y[:, None, :] - Y[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(D, 0.0)
    return sparse.csr_matrix(D)


def _chain_plus_random(n, seed):
    """A path 0-1-...-(n-1) with weights in [0.1, 1) and n random extra
    edges with weights in [0.1, 2), both directions stored: connected."""
    from scipy import sparse

    rng = np.random.default_rng(seed)
    i = np.arange(n - 1)
    w = rng.uniform(0.1, 1.0, n - 1)
    a = rng.integers(0, n, n)
    b = (a + rng.integers(1, n, n)) % n
    w2 = rng.uniform(0.1, 2.0, n)
    rows = np.concatenate([i, i + 1, a, b])
    cols = np.concatenate([i + 1, i, b, a])
    return sparse.csr_matrix((np.concatenate([w, w, w2, w2]), (rows, cols)), shape=(n, n))


def _mst(G, min_samples):
    """(mst, neighbours, core) of both precomputed back-ends; Boruvka's
    equals Kruskal's."""
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree

    k = compute_minimum_spanning_tree(G, min_samples=min_samples, metric="precomputed",
                                      algorithm="kruskal")
    b = compute_minimum_spanning_tree(G, min_samples=min_samples, metric="precomputed",
                                      algorithm="boruvka")
    for u, v in zip(k, b):
        np.testing.assert_array_equal(u, v)
    return k


def test_kruskal_known_triangle(engine):
    """test_kruskal.py:89: edges 0-1 (1), 1-2 (2), 0-2 (3); the MST weighs 3."""
    mst, _, _ = _mst(_csr([0, 1, 1, 2, 0, 2], [1, 0, 2, 1, 2, 0], [1.0, 1, 2, 2, 3, 3], 3), 1)
    assert mst.shape == (2, 3)
    assert np.isclose(np.sort(mst[:, 2]).sum(), 3.0)


def test_kruskal_known_line_graph(engine):
    """test_kruskal.py:106: the path 0-1-2-3 (4, 1, 3) is its own MST."""
    mst, _, _ = _mst(_csr([0, 1, 1, 2, 2, 3], [1, 0, 2, 1, 3, 2], [4.0, 4, 1, 1, 3, 3], 4), 1)
    assert mst.shape == (3, 3)
    assert np.isclose(np.sort(mst[:, 2]).sum(), 1 + 3 + 4)


def test_kruskal_precomputed_edge_count(engine):
    """test_kruskal.py:127."""
    mst, neighbors, core = _mst(_chain_plus_random(15, 99), 3)
    assert mst.shape == (14, 3)
    assert neighbors.shape[0] == 15 and core.shape == (15,)


def test_kruskal_feature_matrix_edge_count(engine):
    """test_kruskal.py:137 and :450 (knn_k 10 and 15)."""
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree

    X = _X()
    n = X.shape[0]
    for knn_k in (10, 15):
        mst, neighbors, core = compute_minimum_spanning_tree(
            X, min_samples=5, metric="euclidean", algorithm="kruskal", knn_k=knn_k)
        assert mst.shape == (n - 1, 3)
        assert neighbors.shape[0] == n and core.shape == (n,)


@pytest.mark.parametrize("min_samples", [1, 3, 5])
def test_kruskal_boruvka_precomputed_mst_weights(engine, min_samples):
    """test_kruskal.py:153: on a complete distance graph both back-ends give
    the same sorted MST weights and core distances."""
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree

    G = _complete_graph(_X())
    mst_k, _, cd_k = compute_minimum_spanning_tree(G, min_samples=min_samples,
                                                   metric="precomputed", algorithm="kruskal")
    mst_b, _, cd_b = compute_minimum_spanning_tree(G, min_samples=min_samples,
                                                   metric="precomputed", algorithm="boruvka")
    assert mst_k.shape == mst_b.shape == (G.shape[0] - 1, 3)
    np.testing.assert_array_equal(np.sort(mst_k[:, 2]), np.sort(mst_b[:, 2]))
    np.testing.assert_array_equal(cd_k, cd_b)


def test_kruskal_disconnected_two_components(engine):
    """test_kruskal.py:188: two cliques, one +inf bridge."""
    mst, _, _ = _mst(_csr([0, 1, 1, 2, 3, 4], [1, 0, 2, 1, 4, 3], [1.0] * 6, 5), 1)
    assert mst.shape == (4, 3)
    assert int(np.sum(np.isinf(mst[:, 2]))) == 1


def test_kruskal_fully_isolated_nodes(engine):
    """test_kruskal.py:203: an empty graph is bridged by n - 1 +inf edges."""
    from scipy import sparse

    mst, _, _ = _mst(sparse.csr_matrix((6, 6), dtype=np.float64), 1)
    assert mst.shape == (5, 3)
    assert np.all(np.isinf(mst[:, 2]))


def test_kruskal_two_nodes(engine):
    """test_kruskal.py:214."""
    mst, _, _ = _mst(_csr([0, 1], [1, 0], [1.5, 1.5], 2), 1)
    assert mst.shape == (1, 3)
    assert np.isclose(mst[0, 2], 1.5)


@pytest.mark.parametrize("min_samples", [1, 5])
def test_hdbscan_kruskal_boruvka_precomputed_label_parity(engine, min_samples):
    """test_kruskal.py:235 (here the labels are equal outright)."""
    from fast_hdbscan_gb300 import HDBSCAN

    G = _complete_graph(_X())
    k = HDBSCAN(min_cluster_size=10, min_samples=min_samples, metric="precomputed",
                algorithm="kruskal").fit(G)
    b = HDBSCAN(min_cluster_size=10, min_samples=min_samples, metric="precomputed",
                algorithm="boruvka").fit(G)
    assert len(set(k.labels_.tolist()) - {-1}) >= 1
    np.testing.assert_array_equal(k.labels_, b.labels_)
    np.testing.assert_array_equal(k.probabilities_, b.probabilities_)


@pytest.mark.parametrize("min_samples", [1, 5])
def test_hdbscan_kruskal_boruvka_euclidean_label_parity(engine, min_samples):
    """test_kruskal.py:266: the kNN-graph Kruskal (knn_k=10) finds as many
    clusters as Boruvka."""
    from fast_hdbscan_gb300 import HDBSCAN

    X = _X()
    k = HDBSCAN(min_cluster_size=10, min_samples=min_samples, algorithm="kruskal",
                knn_k=10).fit(X)
    b = HDBSCAN(min_cluster_size=10, min_samples=min_samples, algorithm="boruvka").fit(X)
    assert len(set(k.labels_.tolist()) - {-1}) == len(set(b.labels_.tolist()) - {-1})


def test_fast_hdbscan_kruskal_routes(engine):
    """test_kruskal.py:292, :298, :489 and :498: fast_hdbscan and the
    estimator with algorithm="kruskal" on points (knn_k 10, 15, 20) and on a
    precomputed graph."""
    from fast_hdbscan_gb300 import HDBSCAN, fast_hdbscan

    X = _X()
    for knn_k in (10, 15):
        labels, probs = fast_hdbscan(X, min_cluster_size=10, algorithm="kruskal", knn_k=knn_k)
        assert labels.shape == (X.shape[0],) and len(set(labels.tolist()) - {-1}) >= 1
    h = HDBSCAN(min_cluster_size=10, min_samples=5, algorithm="kruskal", knn_k=20).fit(X)
    assert h.labels_.shape == (X.shape[0],) and len(set(h.labels_.tolist()) - {-1}) >= 1
    G = _complete_graph(X)
    labels, probs = fast_hdbscan(G, min_cluster_size=10, metric="precomputed",
                                 algorithm="kruskal")
    assert labels.shape == (G.shape[0],) and len(set(labels.tolist()) - {-1}) >= 1


def _assert_valid_spanning_tree(mst, n):
    """test_kruskal.py:320: finite edges join distinct points in range."""
    finite = mst[~np.isinf(mst[:, 2])]
    if len(finite):
        assert finite[:, :2].min() >= 0 and finite[:, :2].max() < n
    assert np.all(finite[:, 0] != finite[:, 1])


def test_kruskal_valid_spanning_tree(engine):
    """test_kruskal.py:331 and :339."""
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree

    mst, _, _ = _mst(_chain_plus_random(20, 42), 3)
    _assert_valid_spanning_tree(mst, 20)
    X = _X()
    mst, _, _ = compute_minimum_spanning_tree(X, min_samples=5, metric="euclidean",
                                              algorithm="kruskal", knn_k=10)
    _assert_valid_spanning_tree(mst, X.shape[0])


def test_kruskal_explicit_zero_edge_preserved(engine):
    """test_kruskal.py:351: an explicit zero weight stays an edge."""
    mst, _, _ = _mst(_csr([0, 1, 1, 2, 2, 3], [1, 0, 2, 1, 3, 2], [0.0, 0, 1, 1, 1, 1], 4), 1)
    assert mst.shape == (3, 3)
    assert np.any(mst[:, 2] == 0.0)


def test_kruskal_asymmetric_min_symmetrization(engine):
    """test_kruskal.py:365: (0, 1) stored as 5 and 1 weighs min(5, 1) = 1."""
    mst, _, _ = _mst(_csr([0, 1, 1, 2], [1, 0, 2, 1], [5.0, 1.0, 2.0, 2.0], 3), 1)
    e01 = mst[((mst[:, 0] == 0) & (mst[:, 1] == 1)) | ((mst[:, 0] == 1) & (mst[:, 1] == 0))]
    assert len(e01) == 1 and np.isclose(e01[0, 2], 1.0)


def test_kruskal_feature_matrix_small_min_samples_and_k(engine):
    """test_kruskal.py:387 (min_samples=1: zero core distances) and :462
    (knn_k below min_samples still spans)."""
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree

    X = _X()
    n = X.shape[0]
    mst, _, core = compute_minimum_spanning_tree(X, min_samples=1, metric="euclidean",
                                                 algorithm="kruskal", knn_k=10)
    assert mst.shape == (n - 1, 3) and np.all(core == 0.0)
    mst, _, _ = compute_minimum_spanning_tree(X, min_samples=10, metric="euclidean",
                                              algorithm="kruskal", knn_k=3)
    assert mst.shape == (n - 1, 3)


def test_bad_algorithm_raises(engine):
    """test_kruskal.py:311."""
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree

    with pytest.raises(ValueError, match="algorithm"):
        compute_minimum_spanning_tree(_X(), algorithm="invalid_algo")
