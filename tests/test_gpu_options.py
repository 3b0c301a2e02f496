"""GPU parity of the selection options: the DBSCAN cut (cluster_trees.py:906,
HDBSCAN.dbscan_clustering), cluster_epsilon_search (:834) and
simplify_hierarchy (:774) -- against the reference's fixtures where they
exist and against the CPU oracle at sizes the reference cannot reach."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from fast_hdbscan_gb300 import synthetic

pytestmark = pytest.mark.gpu

CUT_FIXTURES = ["ka150", "blobs200", "blobs200_ms1", "blobs2d_2k", "blobs2d_20k",
                "umap5d_5k", "vd3d_5k", "vd3d_20k", "edge_two", "edge_1d", "edge_highms",
                "edge_dups"]


def _golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.mark.parametrize("name", CUT_FIXTURES)
def test_dbscan_cut_vs_reference(engine, name):
    from fast_hdbscan_gb300.cluster_trees import get_cluster_labelling_at_cut

    g = _golden(name)
    for cut, want in zip(g["dbscan_cuts"], g["dbscan_labels"]):
        got = get_cluster_labelling_at_cut(g["linkage"], float(cut),
                                           int(g["dbscan_min_cluster_size"]))
        assert got.dtype == np.intp
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("gen,n", [("varying_density", 300_000), ("blobs_2d", 200_000)])
def test_dbscan_cut_vs_oracle_large(engine, gen, n):
    """Deep, unbalanced single-linkage trees: every cut quantile and both
    ends (nothing merged, everything merged)."""
    from fast_hdbscan_gb300.cluster_trees import get_cluster_labelling_at_cut
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan
    from oracle import oracle as O

    X = getattr(synthetic, gen)(n, seed=77)
    lk = fast_hdbscan(X, min_samples=10, min_cluster_size=50, return_trees=True)[2]
    cuts = list(np.quantile(lk[:, 2], [0.0, 0.3, 0.7, 0.95, 0.999, 1.0])) + [np.inf, 0.0]
    for cut in cuts:
        for mcs in (1, 10, 1000):
            np.testing.assert_array_equal(get_cluster_labelling_at_cut(lk, cut, mcs),
                                          O.get_cluster_labelling_at_cut(lk, cut, mcs))


def test_dbscan_clustering_method(engine):
    """hdbscan.py:824: the estimator's cut uses min_samples, else
    min_cluster_size; fast_hdbscan/tests/test_hdbscan.py:96-100 checks the
    cluster count of a cut at 0.3."""
    from fast_hdbscan_gb300 import HDBSCAN
    from oracle import oracle as O

    g = _golden("blobs200")
    model = HDBSCAN().fit(g["X"])
    labels = model.dbscan_clustering(0.3)
    np.testing.assert_array_equal(
        labels, O.get_cluster_labelling_at_cut(model._single_linkage_tree, 0.3, 5))
    assert len(set(labels.tolist()) - {-1}) == 3


def test_epsilon_search_crafted_tree(engine):
    """The reference's outputs on a tree where segments_in_branch marks
    clusters outside the chosen branch."""
    from fast_hdbscan_gb300.cluster_trees import CondensedTree, cluster_epsilon_search

    g = np.load(os.path.join(GOLDEN, "fn_eps_search.npz"))
    tree = CondensedTree(g["parent"], g["child"], g["lambda_val"], g["child_size"])
    i = 0
    while f"sel_{i}" in g.files:
        got = cluster_epsilon_search(g[f"sel_{i}"], tree, min_epsilon=float(g[f"eps_{i}"]))
        np.testing.assert_array_equal(got, g[f"out_{i}"])
        i += 1


@pytest.mark.parametrize("name,thr", [("blobs200", 0.5), ("blobs200", 2.0),
                                      ("blobs2d_20k", 0.05), ("vd3d_20k", 0.01),
                                      ("umap5d_5k", 0.1)])
def test_simplify_hierarchy_vs_oracle(engine, name, thr):
    from fast_hdbscan_gb300.cluster_trees import CondensedTree, simplify_hierarchy
    from oracle import oracle as O

    g = _golden(name)
    ct = CondensedTree(g["ct_parent"].copy(), g["ct_child"].copy(), g["ct_lambda"].copy(),
                       g["ct_size"].copy())
    want = O.simplify_hierarchy(CondensedTree(g["ct_parent"], g["ct_child"], g["ct_lambda"],
                                              g["ct_size"]), thr)
    got = simplify_hierarchy(ct, thr)
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)
    # As in the reference, the argument's kept rows are relabelled in place and
    # the result is those rows in order: reading the argument's rows in order,
    # each is either the next output row or an untouched original row.
    orig = (g["ct_parent"], g["ct_child"], g["ct_lambda"], g["ct_size"])
    j = 0
    for i in range(len(ct.parent)):
        row = tuple(a[i] for a in ct)
        if j < len(got.parent) and row == tuple(a[j] for a in got):
            j += 1
        else:
            assert row == tuple(a[i] for a in orig)
    assert j == len(got.parent)


@pytest.mark.parametrize("gen,n,ms,mcs,eps,pers", [
    ("varying_density", 100_000, 10, 100, 0.0, 0.05),
    ("varying_density", 100_000, 10, 100, 1.5, 0.0),
    ("blobs_2d", 100_000, 10, 50, 0.3, 0.02),
    ("umap_like", 50_000, 10, 100, 0.5, 0.0),
])
def test_fit_with_options_vs_oracle(engine, gen, n, ms, mcs, eps, pers):
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan
    from oracle import oracle as O

    X = getattr(synthetic, gen)(n, seed=5)
    kw = dict(cluster_selection_epsilon=eps, cluster_selection_persistence=pers)
    labels, probs, linkage, ct = fast_hdbscan(X, min_samples=ms, min_cluster_size=mcs,
                                              return_trees=True, **kw)[:4]
    orc = O.fit(X, ms, mcs, mode=1, nthreads=8, **kw)
    for a, b in zip(ct, orc.condensed):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(labels, orc.labels)
    np.testing.assert_array_equal(probs, orc.probabilities)
