"""GPU parity of the tree passes, fed the reference's own intermediates.

Every stage takes the reference's input from the fixtures (its raw MST, its
linkage tree, its condensed tree), so tie-breaking in the MST cannot enter:
sort, linkage tree, condensed tree, EOM / leaf selection, labels and
membership strengths must equal the reference's arrays exactly.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = ["ka150", "blobs200", "blobs200_ms1", "blobs200_leaf", "blobs200_maxcs",
         "blobs200_single", "blobs2d_2k", "blobs2d_20k", "umap5d_5k", "vd3d_5k", "vd3d_20k",
         "edge_two", "edge_1d", "edge_highms", "edge_dups"]


def _golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def _ct(g):
    from fast_hdbscan_gb300.cluster_trees import CondensedTree

    return CondensedTree(g["ct_parent"], g["ct_child"], g["ct_lambda"], g["ct_size"])


@pytest.mark.parametrize("name", CASES)
def test_sort_and_linkage_bitexact(engine, name):
    from fast_hdbscan_gb300.cluster_trees import mst_to_linkage_tree, sort_mst

    g = _golden(name)
    smst = sort_mst(g["mst_raw"])
    np.testing.assert_array_equal(smst, g["sorted_mst"])
    np.testing.assert_array_equal(mst_to_linkage_tree(g["sorted_mst"]), g["linkage"])


@pytest.mark.parametrize("name", CASES)
def test_condense_bitexact(engine, name):
    from fast_hdbscan_gb300.cluster_trees import condense_tree

    g = _golden(name)
    # hdbscan.py:521 condenses without max_cluster_size (only EOM reads it)
    ct = condense_tree(g["linkage"], int(g["min_cluster_size"]))
    ref = _ct(g)
    for a, b in zip(ct, ref):
        np.testing.assert_array_equal(a, b)
        assert a.dtype == b.dtype


@pytest.mark.parametrize("name", CASES)
def test_selection_labels_bitexact(engine, name):
    from fast_hdbscan_gb300.cluster_trees import (
        cluster_tree_from_condensed_tree, cluster_tree_leaves, extract_eom_clusters,
        get_cluster_label_vector, get_point_membership_strength_vector)

    g = _golden(name)
    if str(g["cluster_selection_method"]) == "eom" and float(g["cluster_selection_epsilon"]) > 0:
        pytest.skip("epsilon search is checked elsewhere")
    if float(g["cluster_selection_persistence"]) > 0:
        pytest.skip("persistence is checked elsewhere")
    ct = _ct(g)
    n = g["X"].shape[0]
    cl_tree = cluster_tree_from_condensed_tree(ct)
    if str(g["cluster_selection_method"]) == "leaf":
        sel = cluster_tree_leaves(cl_tree, n) if len(cl_tree.parent) else np.empty(0, np.int64)
    else:
        sel = extract_eom_clusters(ct, cl_tree, float(g["max_cluster_size"]),
                                   bool(g["allow_single_cluster"]))
        if "selected_eom" in g.files:
            np.testing.assert_array_equal(sel, g["selected_eom"])
    labels = get_cluster_label_vector(ct, sel, 0.0, n)
    np.testing.assert_array_equal(labels, g["labels"])
    probs = get_point_membership_strength_vector(ct, sel, labels)
    np.testing.assert_array_equal(probs, g["probabilities"])


WEIGHTED = ["blobs200_w_labels", "blobs2d_2k_w", "vd3d_5k_w"]


@pytest.mark.parametrize("name", WEIGHTED)
def test_weighted_linkage_and_condense_bitexact(engine, name):
    """cluster_trees.py:98 mst_to_linkage_tree_w_sample_weights and :205
    condense_tree(sample_weights=...) on the reference's own sorted MST and
    linkage tree.  The fixtures' weights (integers, multiples of 1/64) have
    exact float32 sums, so the weighted sizes are bit-identical."""
    from fast_hdbscan_gb300.cluster_trees import (
        condense_tree, mst_to_linkage_tree_w_sample_weights, sort_mst)

    g = _golden(name)
    w = g["sample_weights"]
    np.testing.assert_array_equal(sort_mst(g["mst_raw"]), g["sorted_mst"])
    np.testing.assert_array_equal(mst_to_linkage_tree_w_sample_weights(g["sorted_mst"], w),
                                  g["linkage"])
    ct = condense_tree(g["linkage"], int(g["min_cluster_size"]), sample_weights=w)
    for a, b in zip(ct, _ct(g)):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("name", CASES + WEIGHTED)
def test_clusters_from_spanning_tree_fused_bitexact(engine, name):
    """hdbscan.py:497 clusters_from_spanning_tree in one fused call
    (fhg_clusters_from_mst) on the reference's raw MST with the fixture's
    selection options: labels, probabilities, linkage tree, condensed tree and
    sorted MST equal the reference's arrays."""
    from fast_hdbscan_gb300.hdbscan import clusters_from_spanning_tree

    g = _golden(name)
    w = g["sample_weights"] if "sample_weights" in g.files else None
    labels, probs, linkage, ct, smst = clusters_from_spanning_tree(
        g["mst_raw"], min_cluster_size=int(g["min_cluster_size"]),
        cluster_selection_method=str(g["cluster_selection_method"]),
        max_cluster_size=float(g["max_cluster_size"]),
        allow_single_cluster=bool(g["allow_single_cluster"]),
        cluster_selection_epsilon=float(g["cluster_selection_epsilon"]),
        cluster_selection_persistence=float(g["cluster_selection_persistence"]),
        sample_weights=w)
    np.testing.assert_array_equal(smst, g["sorted_mst"])
    np.testing.assert_array_equal(linkage, g["linkage"])
    for a, b in zip(ct, _ct(g)):
        np.testing.assert_array_equal(a, b)
        assert a.dtype == b.dtype
    np.testing.assert_array_equal(labels, g["labels"])
    np.testing.assert_array_equal(probs, g["probabilities"])


@pytest.mark.parametrize("seed", range(6))
def test_clusters_from_spanning_tree_fused_vs_oracle(engine, seed):
    """The fused call against the oracle's clusters_from_spanning_tree on
    random trees with heavily tied integer weights (the sort's (weight, src,
    dst) order decides), both selection methods, epsilon, persistence,
    max_cluster_size, allow_single_cluster and sample weights."""
    from fast_hdbscan_gb300.hdbscan import clusters_from_spanning_tree
    from oracle import oracle as O

    rng = np.random.default_rng(seed)
    n = int(rng.integers(50, 3000))
    parent = np.array([rng.integers(0, i) for i in range(1, n)])
    child = np.arange(1, n)
    flip = rng.random(n - 1) < 0.5
    src, dst = np.where(flip, child, parent), np.where(flip, parent, child)
    wts = rng.integers(1, 12, size=n - 1).astype(np.float64) * 0.25
    mst = np.stack([src, dst, wts], axis=1).astype(np.float64)[rng.permutation(n - 1)]
    kw = dict(min_cluster_size=int(rng.integers(3, 40)),
              cluster_selection_method=["eom", "leaf"][seed % 2],
              max_cluster_size=[np.inf, float(n // 3)][(seed // 2) % 2],
              allow_single_cluster=bool(seed % 3 == 0),
              cluster_selection_epsilon=[0.0, 0.6][seed % 3 == 1],
              cluster_selection_persistence=[0.0, 0.3][seed % 4 == 2])
    w = (rng.integers(1, 5, size=n).astype(np.float32) if seed >= 4 else None)
    labels, probs, linkage, ct, smst = clusters_from_spanning_tree(mst, sample_weights=w, **kw)
    o_labels, o_probs, o_linkage, o_ct, o_smst, _ = O.clusters_from_spanning_tree(
        mst, sample_weights=w, **kw)
    np.testing.assert_array_equal(smst, o_smst)
    np.testing.assert_array_equal(linkage, o_linkage)
    for a, b in zip(ct, o_ct):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(labels, o_labels)
    np.testing.assert_array_equal(probs, o_probs)


def test_clusters_from_spanning_tree_weight_shape(engine):
    """A tree of m edges takes m + 1 sample weights; others are rejected
    before any device work."""
    from fast_hdbscan_gb300.hdbscan import clusters_from_spanning_tree

    mst = np.array([[0, 1, 0.5], [1, 2, 0.7], [2, 3, 0.2]])
    with pytest.raises(ValueError):
        clusters_from_spanning_tree(mst, min_cluster_size=2,
                                    sample_weights=np.ones(3, np.float32))
    labels, probs, *_ = clusters_from_spanning_tree(mst, min_cluster_size=2,
                                                    sample_weights=np.ones(4, np.float32))
    assert labels.shape == (4,) and probs.shape == (4,)
