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
