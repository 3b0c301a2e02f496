"""The reference's own estimator and edge-case tests
(fast_hdbscan/tests/test_hdbscan.py, test_edge_cases.py), restated against
the GPU engine.

The reference's module-level data -- make_blobs(n_samples=200,
random_state=10), shuffled with random_state=7 and standardised, with
n_clusters = 3 -- is the committed fixture ``blobs200`` (written by the
reference's generator; scikit-learn is not needed here).  The other inputs
are made with NumPy as the reference's tests make them, except the three
blobs of the epsilon edge cases, which NumPy draws in place of make_blobs.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

N_CLUSTERS = 3


def _X():
    return np.load(os.path.join(GOLDEN, "blobs200.npz"))["X"]


def _n_clusters(labels):
    return len(set(labels.tolist())) - int(-1 in labels)


def test_hdbscan_feature_vector(engine):
    """test_hdbscan.py:84."""
    from fast_hdbscan_gb300 import HDBSCAN, fast_hdbscan

    X = _X()
    labels, p, ltree, ctree, mtree, neighbors, cdists = fast_hdbscan(X, return_trees=True)
    assert _n_clusters(labels) == N_CLUSTERS
    assert _n_clusters(HDBSCAN().fit(X).labels_) == N_CLUSTERS


def test_hdbscan_dbscan_clustering(engine):
    """test_hdbscan.py:96."""
    from fast_hdbscan_gb300 import HDBSCAN

    labels = HDBSCAN().fit(_X()).dbscan_clustering(0.3)
    assert _n_clusters(labels) == N_CLUSTERS


def test_hdbscan_no_clusters(engine):
    """test_hdbscan.py:103 (the estimator's min_samples is then n + 1:
    every core distance is infinite)."""
    from fast_hdbscan_gb300 import HDBSCAN, fast_hdbscan

    X = _X()
    labels, p = fast_hdbscan(X, min_cluster_size=len(X) + 1)
    assert _n_clusters(labels) == 0
    assert _n_clusters(HDBSCAN(min_cluster_size=len(X) + 1).fit(X).labels_) == 0


def test_hdbscan_min_cluster_size(engine):
    """test_hdbscan.py:120: every min_cluster_size from 2 to n, through both
    entry points; no cluster is smaller than min_cluster_size.
    (fast_hdbscan's min_samples defaults to 10, the estimator's to
    min_cluster_size, so the estimator's kNN lists grow to the whole set.)"""
    from fast_hdbscan_gb300 import HDBSCAN, fast_hdbscan

    X = _X()
    for mcs in range(2, len(X) + 1):
        for labels in (fast_hdbscan(X, min_cluster_size=mcs)[0],
                       HDBSCAN(min_cluster_size=mcs).fit(X).labels_):
            kept = labels[labels != -1]
            if kept.size:
                assert np.bincount(kept).min() >= mcs


def test_hdbscan_input_lists(engine):
    """test_hdbscan.py:133: a list of lists fits without raising."""
    from fast_hdbscan_gb300 import HDBSCAN

    HDBSCAN().fit([[1.0, 2.0], [3.0, 4.0]])


def test_hdbscan_allow_single_cluster_with_epsilon(engine):
    """test_hdbscan.py:169: 150 uniform points (np.random.seed(0)): 8 labels
    and 69 noise points without epsilon; 2 labels and 2 noise points with
    cluster_selection_epsilon=0.2."""
    from fast_hdbscan_gb300 import HDBSCAN

    np.random.seed(0)
    no_structure = np.random.rand(150, 2)
    c = HDBSCAN(min_cluster_size=5, cluster_selection_epsilon=0.0).fit(no_structure)
    u, counts = np.unique(c.labels_, return_counts=True)
    assert len(u) == 8 and counts[u == -1] == 69
    c = HDBSCAN(min_cluster_size=5, cluster_selection_epsilon=0.2).fit(no_structure)
    u, counts = np.unique(c.labels_, return_counts=True)
    assert len(u) == 2 and counts[u == -1] == 2


def test_hdbscan_max_cluster_size(engine):
    """test_hdbscan.py:189."""
    from fast_hdbscan_gb300 import HDBSCAN

    model = HDBSCAN(max_cluster_size=30).fit(_X())
    assert len(set(model.labels_.tolist())) >= 3
    for label in set(model.labels_.tolist()) - {-1}:
        assert np.sum(model.labels_ == label) <= 30


def test_hdbscan_persistence_threshold(engine):
    """test_hdbscan.py:197."""
    from fast_hdbscan_gb300 import HDBSCAN

    model = HDBSCAN(min_cluster_size=5, cluster_selection_method="leaf",
                    cluster_selection_persistence=20.0).fit(_X())
    assert np.all(model.labels_ == -1)


def test_mst_entry(engine):
    """test_hdbscan.py:204: clusters_from_spanning_tree on the fitted MST
    gives the estimator's labels, probabilities and trees (here bit for bit)."""
    from fast_hdbscan_gb300 import HDBSCAN
    from fast_hdbscan_gb300.hdbscan import clusters_from_spanning_tree

    model = HDBSCAN(min_cluster_size=5).fit(_X())
    labels, probabilities, linkage_tree, condensed_tree, sorted_mst = (
        clusters_from_spanning_tree(model._min_spanning_tree, min_cluster_size=5))
    np.testing.assert_array_equal(model.labels_, labels)
    np.testing.assert_array_equal(model.probabilities_, probabilities)
    np.testing.assert_array_equal(model._min_spanning_tree, sorted_mst)
    np.testing.assert_array_equal(model._single_linkage_tree, linkage_tree)
    np.testing.assert_array_equal(model._condensed_tree["parent"], condensed_tree.parent)
    np.testing.assert_array_equal(model._condensed_tree["child"], condensed_tree.child)
    np.testing.assert_array_equal(model._condensed_tree["lambda_val"], condensed_tree.lambda_val)
    np.testing.assert_array_equal(model._condensed_tree["child_size"], condensed_tree.child_size)


def test_function_api_matches_class_api(engine):
    """test_hdbscan.py:717 (there on a precomputed graph; here on both the
    Euclidean input and the complete distance graph of the same points)."""
    from scipy.sparse import csr_matrix

    from fast_hdbscan_gb300 import HDBSCAN, fast_hdbscan

    X = _X()
    est = HDBSCAN(min_cluster_size=10).fit(X)
    labels, probs = fast_hdbscan(X, min_cluster_size=10)
    np.testing.assert_array_equal(est.labels_, labels)
    np.testing.assert_array_equal(est.probabilities_, probs)
    D = np.sqrt(((X[:, None, :] - X[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(D, 0.0)
    G = csr_matrix(D)
    pre = HDBSCAN(min_cluster_size=10, metric="precomputed").fit(G)
    labels_g, probs_g = fast_hdbscan(G, min_cluster_size=10, metric="precomputed")
    np.testing.assert_array_equal(pre.labels_, labels_g)
    np.testing.assert_array_equal(pre.probabilities_, probs_g)


def test_issue_63_no_spurious_noise(engine):
    """test_hdbscan.py:742: three Gaussian blobs of 200 points per seed; with
    min_cluster_size=192, min_samples=1, epsilon 0.05957 and a single cluster
    allowed, the fit keeps at least one cluster and less than 90 % noise."""
    from fast_hdbscan_gb300 import HDBSCAN

    for seed in (700, 727):
        rng = np.random.default_rng(seed)
        centers = rng.uniform(-10, 10, size=(3, 3))
        data = np.vstack([rng.normal(loc=c, scale=0.5, size=(200, 3)) for c in centers])
        labels = HDBSCAN(min_cluster_size=192, min_samples=1, cluster_selection_epsilon=0.05957,
                         allow_single_cluster=True).fit_predict(data)
        assert len(set(labels.tolist()) - {-1}) >= 1, seed
        assert np.sum(labels == -1) / len(labels) < 0.9, seed


def _three_blobs(seed=42):
    """200 points around three centres in 2-D (the reference's edge-case
    tests draw theirs from scikit-learn's make_blobs)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-10, 10, size=(3, 2))
    return np.vstack([rng.normal(c, 1.0, size=(67 if i < 2 else 66, 2))
                      for i, c in enumerate(centres)])


def test_edge_case_inputs(engine):
    """test_edge_cases.py:8-69: a single point, two points, 50 identical
    points, min_cluster_size above n, 1-D data, min_samples near n, and
    epsilon 0 or very large with a single cluster allowed."""
    from fast_hdbscan_gb300 import HDBSCAN

    assert HDBSCAN(min_cluster_size=2).fit_predict(np.array([[1.0, 2.0]]))[0] == -1
    two = HDBSCAN(min_cluster_size=2).fit_predict(np.array([[0.0, 0.0], [0.1, 0.0]]))
    assert len(set(two.tolist()) - {-1}) <= 1
    assert len(HDBSCAN(min_cluster_size=5).fit_predict(np.full((50, 3), 1.0))) == 50
    np.random.seed(42)
    assert np.all(HDBSCAN(min_cluster_size=100).fit_predict(np.random.rand(10, 2)) == -1)
    np.random.seed(42)
    X1 = np.concatenate([np.random.normal(0, 0.1, 50),
                         np.random.normal(5, 0.1, 50)]).reshape(-1, 1)
    assert len(set(HDBSCAN(min_cluster_size=10).fit_predict(X1).tolist()) - {-1}) >= 1
    np.random.seed(42)
    assert len(HDBSCAN(min_cluster_size=5, min_samples=18).fit_predict(
        np.random.rand(20, 2))) == 20
    X = _three_blobs()
    labels = HDBSCAN(min_cluster_size=10, cluster_selection_epsilon=0.0).fit_predict(X)
    assert len(set(labels.tolist()) - {-1}) >= 1
    labels = HDBSCAN(min_cluster_size=10, cluster_selection_epsilon=1000.0,
                     allow_single_cluster=True).fit_predict(X)
    assert len(set(labels.tolist()) - {-1}) <= 1
