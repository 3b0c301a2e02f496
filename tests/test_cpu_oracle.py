"""CPU checks of the oracle (no GPU): pinned against the reference fixtures.

The fixtures in tests/golden were produced by the unmodified reference
(make_golden.py).  In reference tie mode the oracle must reproduce every
array of every fixture bit for bit; in canonical mode (the GPU engine's tie
rules) core distances and the MST weight multiset are identical and labels
agree up to the reference's tie choices.
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as O

# fit fixtures; fn_*.npz hold function-level cases, kr_*.npz the kNN-graph
# Kruskal back-end (algorithm="kruskal")
FIXTURES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith(("fn_", "kr_", "pc_", "sc_", "cg_")))
KRUSKAL = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "kr_*.npz")))
# metric="precomputed" on sparse graphs (precomputed.py:410 Boruvka, :479 Kruskal)
PRECOMPUTED = sorted(os.path.basename(p)[:-4]
                     for p in glob.glob(os.path.join(GOLDEN, "pc_*.npz")))
# The reference indexes knn[-1] when min_samples >= n (k exceeds the point
# count); its MST for that fixture has edges to "point -1".  Only its labels
# and probabilities (all noise) are meaningful there.
QUIRK = {"edge_mcs_gt_n"}


def _load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def _kw(g):
    return dict(cluster_selection_method=str(g["cluster_selection_method"]),
                max_cluster_size=float(g["max_cluster_size"]),
                allow_single_cluster=bool(g["allow_single_cluster"]),
                cluster_selection_epsilon=float(g["cluster_selection_epsilon"]),
                cluster_selection_persistence=float(g["cluster_selection_persistence"]))


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_reference_mode_bitexact(name):
    g = _load(name)
    X = g["X"]
    if X.shape[0] < 2:
        pytest.skip("degenerate input handled in Python")
    w = g["sample_weights"] if "sample_weights" in g.files else None
    tree = O.build_kdtree(X)
    if "kd_idx_array" in g.files:
        a = tree.arrays()
        for key in ("idx_array", "idx_start", "idx_end", "is_leaf", "node_bounds"):
            np.testing.assert_array_equal(a[key], g["kd_" + key])
    if "knn_rdist" in g.files:
        k = g["knn_rdist"].shape[1]
        rd, ix = O.tree_query(tree, k, mode=0)
        np.testing.assert_array_equal(rd, g["knn_rdist"])
        np.testing.assert_array_equal(ix, g["knn_idx"])
    if name in QUIRK:  # the canonical mode spans the points with +inf edges instead
        fit = O.fit(X, int(g["min_samples"]), int(g["min_cluster_size"]), mode=1, **_kw(g))
        np.testing.assert_array_equal(fit.labels, g["labels"])
        np.testing.assert_array_equal(fit.probabilities, g["probabilities"])
        return
    fit = O.fit(X, int(g["min_samples"]), int(g["min_cluster_size"]), mode=0, sample_weights=w,
                **_kw(g))
    np.testing.assert_array_equal(fit.labels, g["labels"])
    np.testing.assert_array_equal(fit.probabilities, g["probabilities"])
    np.testing.assert_array_equal(fit.mst, g["mst_raw"])
    np.testing.assert_array_equal(fit.core, g["core"])
    np.testing.assert_array_equal(fit.neighbors, g["neighbors"])
    np.testing.assert_array_equal(fit.sorted_mst, g["sorted_mst"])
    np.testing.assert_array_equal(fit.linkage, g["linkage"])
    for a, b in zip(fit.condensed, (g["ct_parent"], g["ct_child"], g["ct_lambda"], g["ct_size"])):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("name", sorted(set(FIXTURES) - QUIRK))
def test_oracle_canonical_mode_invariants(name):
    g = _load(name)
    X = g["X"]
    if X.shape[0] < 2:
        pytest.skip("degenerate input handled in Python")
    w = g["sample_weights"] if "sample_weights" in g.files else None
    fit = O.fit(X, int(g["min_samples"]), int(g["min_cluster_size"]), mode=1, sample_weights=w,
                **_kw(g))
    np.testing.assert_array_equal(fit.core, g["core"])
    np.testing.assert_array_equal(np.sort(fit.mst[:, 2]), np.sort(g["mst_raw"][:, 2]))
    assert len(set(fit.labels.tolist()) - {-1}) == len(set(g["labels"].tolist()) - {-1})


def test_oracle_known_answer():
    """fast_hdbscan/tests/test_hdbscan.py:169-186 through the oracle."""
    np.random.seed(0)
    X = np.random.rand(150, 2)
    f = O.fit(X, None, 5, mode=0)
    u, c = np.unique(f.labels, return_counts=True)
    assert len(u) == 8 and c[u == -1] == 69
    f = O.fit(X, None, 5, mode=0, cluster_selection_epsilon=0.2)
    u, c = np.unique(f.labels, return_counts=True)
    assert len(u) == 2 and c[u == -1] == 2


def test_oracle_min_cluster_size_invariant():
    """fast_hdbscan/tests/test_hdbscan.py:120-130: every cluster holds at
    least min_cluster_size points, for both tie modes."""
    X = _load("blobs200")["X"]
    for mcs in (2, 3, 5, 8, 13, 21, 34, 55, 89, 144, 200):
        for mode in (0, 1):
            labels = O.fit(X, None, mcs, mode=mode).labels
            kept = labels[labels != -1]
            if kept.size:
                assert np.bincount(kept).min() >= mcs


def test_oracle_parallel_threads_same_weights():
    """The reference's parallel loops race on the pruning bound, so its MST
    edge choice between equal weights can change with the thread count; the
    weight multiset cannot."""
    g = _load("vd3d_5k")
    a = O.fit(g["X"], 15, 25, mode=0, nthreads=1)
    b = O.fit(g["X"], 15, 25, mode=0, nthreads=4)
    np.testing.assert_array_equal(np.sort(a.mst[:, 2]), np.sort(b.mst[:, 2]))
    # the canonical mode is deterministic in any thread count
    c1 = O.fit(g["X"], 15, 25, mode=1, nthreads=1)
    c4 = O.fit(g["X"], 15, 25, mode=1, nthreads=4)
    np.testing.assert_array_equal(c1.mst, c4.mst)
    np.testing.assert_array_equal(c1.labels, c4.labels)


@pytest.mark.parametrize("name", sorted(set(FIXTURES) - QUIRK))
def test_oracle_parallel_reference_mode_fixtures(name):
    """Mode 2 (the reference's sequential tie rules evaluated in parallel)
    reproduces the reference's own fixtures bit for bit, on several threads."""
    g = _load(name)
    X = g["X"]
    if X.shape[0] < 2:
        pytest.skip("degenerate input handled in Python")
    w = g["sample_weights"] if "sample_weights" in g.files else None
    fit = O.fit(X, int(g["min_samples"]), int(g["min_cluster_size"]), mode=2, nthreads=4,
                sample_weights=w, **_kw(g))
    np.testing.assert_array_equal(fit.mst, g["mst_raw"])
    np.testing.assert_array_equal(fit.labels, g["labels"])
    np.testing.assert_array_equal(fit.probabilities, g["probabilities"])


@pytest.mark.parametrize("gen,n,ms", [("varying_density", 60_000, 15),
                                      ("blobs_2d", 60_000, 10),
                                      ("umap_like", 30_000, 10),
                                      ("varying_density", 40_000, 1)])
def test_oracle_parallel_reference_mode_equals_sequential(gen, n, ms):
    """Mode 2 on 8 threads equals mode 0 on one thread (the reference's loops
    run in order) edge for edge, on inputs large enough for many tie choices."""
    from fast_hdbscan_gb300 import synthetic

    X = getattr(synthetic, gen)(n, seed=11)
    tree = O.build_kdtree(X)
    seq = O.parallel_boruvka(tree, ms, mode=0, nthreads=1)
    par = O.parallel_boruvka(tree, ms, mode=2, nthreads=8)
    np.testing.assert_array_equal(par[0], seq[0])
    np.testing.assert_array_equal(par[2], seq[2])


@pytest.mark.parametrize("name", sorted(set(FIXTURES) - QUIRK))
def test_oracle_dbscan_cut_bitexact(name):
    """get_cluster_labelling_at_cut (cluster_trees.py:906) at several cuts of
    every fixture's reference linkage tree."""
    g = _load(name)
    if "dbscan_cuts" not in g.files:
        pytest.skip("no linkage tree")
    for cut, want in zip(g["dbscan_cuts"], g["dbscan_labels"]):
        got = O.get_cluster_labelling_at_cut(g["linkage"], float(cut),
                                             int(g["dbscan_min_cluster_size"]))
        np.testing.assert_array_equal(got, want)


def test_oracle_epsilon_search_crafted_tree():
    """cluster_epsilon_search (cluster_trees.py:834) on a tree where the
    reference's segments_in_branch lookup marks clusters outside the branch."""
    g = np.load(os.path.join(GOLDEN, "fn_eps_search.npz"))
    ct = O.CondensedTree(g["parent"], g["child"], g["lambda_val"], g["child_size"])
    i = 0
    while f"sel_{i}" in g.files:
        got = O.cluster_epsilon_search(ct, g[f"sel_{i}"], float(g[f"eps_{i}"]))
        np.testing.assert_array_equal(got, g[f"out_{i}"])
        i += 1
    assert i >= 5


@pytest.mark.parametrize("name", KRUSKAL)
def test_oracle_kruskal_knn_bitexact(name):
    """kruskal.py:950 _kruskal_mst_knn (algorithm="kruskal", integer knn_k):
    the oracle's MST edges (acceptance order and +inf bridges included),
    neighbours and float64 core distances equal the reference's, and the fit
    on that MST gives the reference's labels and probabilities."""
    g = _load(name)
    X = g["X"]
    ms, mcs, knn_k = int(g["min_samples"]), int(g["min_cluster_size"]), int(g["knn_k"])
    w = g["sample_weights"] if "sample_weights" in g else None
    mst, nbrs, core = O.kruskal_knn(O.build_kdtree(X), ms, knn_k, mode=0, sample_weights=w)
    np.testing.assert_array_equal(mst, g["mst"])
    np.testing.assert_array_equal(nbrs, g["neighbors"])
    np.testing.assert_array_equal(core, g["core"])
    labels, probs, *_ = O.clusters_from_spanning_tree(mst, min_cluster_size=mcs,
                                                      sample_weights=w)
    np.testing.assert_array_equal(labels, g["labels"])
    np.testing.assert_array_equal(probs, g["probabilities"])


@pytest.mark.parametrize("name", PRECOMPUTED)
def test_oracle_precomputed_bitexact(name):
    """precomputed.py:479 (algorithm="kruskal"): MST edges in acceptance order
    with their bridges, neighbours and core distances equal the reference's.
    precomputed.py:410 (algorithm="boruvka"): its float32 Boruvka finds a
    spanning forest of the same weights (restored to the same float64 values)
    -- mutual-reachability weights tie wherever a core distance dominates, and
    its tie choices are its own -- in another order.  Labels and
    probabilities equal the reference's for both."""
    import scipy.sparse

    g = _load(name)
    n = int(g["n"])
    G = scipy.sparse.coo_matrix((g["data"], (g["rows"], g["cols"])), shape=(n, n))
    ms, mcs = int(g["min_samples"]), int(g["min_cluster_size"])
    mst, nbrs, core = O.precomputed_kruskal(G, ms)
    np.testing.assert_array_equal(nbrs, g["neighbors"])
    np.testing.assert_array_equal(core, g["core"])
    if str(g["algorithm"]) == "kruskal":
        np.testing.assert_array_equal(mst, g["mst"])
    else:
        np.testing.assert_array_equal(np.sort(mst[:, 2]), np.sort(g["mst"][:, 2]))
    labels, probs, *_ = O.clusters_from_spanning_tree(mst, min_cluster_size=mcs)
    if str(g["algorithm"]) == "kruskal":
        np.testing.assert_array_equal(labels, g["labels"])
        np.testing.assert_array_equal(probs, g["probabilities"])
    else:  # same partition; equal-weight edges may number the clusters otherwise
        assert_same_partition(labels, g["labels"])
        np.testing.assert_array_equal(probs, g["probabilities"])


def assert_same_partition(a, b):
    """Labels equal up to renaming the clusters (noise stays noise)."""
    a, b = np.asarray(a), np.asarray(b)
    assert np.array_equal(a == -1, b == -1)
    pairs = set(zip(a[a >= 0].tolist(), b[b >= 0].tolist()))
    assert len(pairs) == len({x for x, _ in pairs}) == len({y for _, y in pairs})
