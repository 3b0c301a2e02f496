"""The reference tie mode (reproducible=True, fhg_set_tie_rule): the MST --
edge order, orientation and weights -- equals the reference's, and so do the
labels and probabilities.

* On the reference's own fixtures (written by the unmodified reference):
  the raw MST, sorted MST, labels and probabilities bit for bit.
* Against the oracle in the reference's tie mode (mode 0 on one thread, or
  mode 2 -- the same rules evaluated in parallel) on larger seeded inputs.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from fast_hdbscan_gb300 import synthetic

pytestmark = pytest.mark.gpu

FIT_FIXTURES = ["ka150", "ka150_eps", "blobs200", "blobs200_ms1", "blobs200_leaf",
                "blobs200_maxcs", "blobs200_single", "blobs200_persist", "blobs2d_2k",
                "blobs2d_20k", "umap5d_5k", "vd3d_5k", "vd3d_20k", "edge_two", "edge_1d",
                "edge_highms", "edge_dups", "blobs200_w_labels", "blobs2d_2k_w", "vd3d_5k_w",
                "hd12_2k", "hd24_1k"]


def _kw(g):
    return dict(cluster_selection_method=str(g["cluster_selection_method"]),
                max_cluster_size=float(g["max_cluster_size"]),
                allow_single_cluster=bool(g["allow_single_cluster"]),
                cluster_selection_epsilon=float(g["cluster_selection_epsilon"]),
                cluster_selection_persistence=float(g["cluster_selection_persistence"]))


@pytest.mark.parametrize("name", FIT_FIXTURES)
def test_reference_ties_fixture(engine, name):
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree, fast_hdbscan
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    X = g["X"]
    ms, mcs = int(g["min_samples"]), int(g["min_cluster_size"])
    w = g["sample_weights"] if "sample_weights" in g.files else None
    if X.shape[1] <= 30 or w is not None:
        mst, nbrs, core = compute_minimum_spanning_tree(X, min_samples=ms, sample_weights=w,
                                                        reproducible=True)
        np.testing.assert_array_equal(mst, g["mst_raw"])
        np.testing.assert_array_equal(core, g["core"])
        # the reference's query and heap order, equal distances included
        np.testing.assert_array_equal(nbrs, g["neighbors"])
    labels, probs, _, _, smst, _, _ = fast_hdbscan(X, min_samples=ms, min_cluster_size=mcs,
                                                   sample_weights=w, reproducible=True,
                                                   return_trees=True, **_kw(g))
    np.testing.assert_array_equal(smst, g["sorted_mst"])
    np.testing.assert_array_equal(labels, g["labels"])
    np.testing.assert_array_equal(probs, g["probabilities"])


@pytest.mark.parametrize("gen,n,ms,mcs,mode", [
    ("varying_density", 60_000, 15, 100, 0),
    ("blobs_2d", 60_000, 10, 50, 0),
    ("umap_like", 30_000, 10, 100, 0),
    ("varying_density", 40_000, 1, 20, 0),
    ("varying_density", 1_000_000, 15, 500, 2),
    ("umap_like", 400_000, 10, 200, 2),
])
def test_reference_ties_vs_oracle(engine, gen, n, ms, mcs, mode):
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree, fast_hdbscan
    from oracle import oracle as O

    X = getattr(synthetic, gen)(n, seed=17)
    orc = O.fit(X, ms, mcs, mode=mode, nthreads=1 if mode == 0 else (os.cpu_count() or 1))
    mst, _, core = compute_minimum_spanning_tree(X, min_samples=ms, reproducible=True)
    np.testing.assert_array_equal(core, orc.core)
    np.testing.assert_array_equal(mst, orc.mst)
    labels, probs = fast_hdbscan(X, min_samples=ms, min_cluster_size=mcs, reproducible=True)
    np.testing.assert_array_equal(labels, orc.labels)
    np.testing.assert_array_equal(probs, orc.probabilities)


def test_reference_ties_weighted_vs_oracle(engine):
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree
    from oracle import oracle as O

    X = synthetic.varying_density(50_000, seed=19)
    w = np.random.default_rng(19).integers(1, 5, len(X)).astype(np.float32)
    mst, _, core = compute_minimum_spanning_tree(X, min_samples=10, sample_weights=w,
                                                 reproducible=True)
    e, _, c, _ = O.parallel_boruvka(O.build_kdtree(X), 10, mode=0, nthreads=1,
                                    sample_weights=w)
    np.testing.assert_array_equal(core, c)
    np.testing.assert_array_equal(mst, e)


def test_tie_rule_is_restored(engine):
    """The rule applies inside the call only: a default fit afterwards is the
    canonical one again."""
    from fast_hdbscan_gb300 import _native
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree

    X = synthetic.varying_density(20_000, seed=23)
    a, _, _ = compute_minimum_spanning_tree(X, min_samples=10)
    compute_minimum_spanning_tree(X, min_samples=10, reproducible=True)
    b, _, _ = compute_minimum_spanning_tree(X, min_samples=10)
    np.testing.assert_array_equal(a, b)
    assert _native.load().fhg_set_tie_rule(0) == 0


def test_reference_ties_take_at_most_63_min_samples(engine):
    """The tie mode re-queries tied kNN rows with lists of up to 64; a larger
    min_samples raises there (the default rule takes it) and leaves the
    default rule in place."""
    from fast_hdbscan_gb300 import _native
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree

    X = synthetic.varying_density(3_000, seed=24)
    with pytest.raises(NotImplementedError, match="reference tie mode"):
        compute_minimum_spanning_tree(X, min_samples=64, reproducible=True)
    mst, _, _ = compute_minimum_spanning_tree(X, min_samples=64)
    assert mst.shape == (X.shape[0] - 1, 3)
    assert _native.load().fhg_set_tie_rule(0) == 0


@pytest.mark.parametrize("seed,d,side,n,ms,mcs", [
    (0, 2, 150, 12_000, 10, 20), (1, 3, 30, 15_000, 5, 10), (2, 4, 10, 6_000, 3, 5),
])
def test_reference_ties_integer_grid_vs_oracle(engine, seed, d, side, n, ms, mcs):
    """Distinct points of an integer grid, plus exact duplicates of some of
    them: equal distances inside every kNN list, which the reference orders
    by its query and heap.  The reference tie mode lists them as the
    reference does and equals the oracle's sequential reference semantics
    (mode 0) bit for bit."""
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree, fast_hdbscan
    from oracle import oracle as O

    rng = np.random.default_rng(2000 + seed)
    cells = rng.choice(side ** d, size=n, replace=False)
    X = np.stack([(cells // side ** j) % side for j in range(d)], axis=1).astype(np.float32)
    X = np.concatenate([X, X[rng.choice(n, n // 20, replace=False)]])
    orc = O.fit(X, ms, mcs, mode=0, nthreads=1)
    mst, nbrs, core = compute_minimum_spanning_tree(X, min_samples=ms, reproducible=True)
    np.testing.assert_array_equal(core, orc.core)
    np.testing.assert_array_equal(nbrs, orc.neighbors)
    np.testing.assert_array_equal(mst, orc.mst)
    labels, probs = fast_hdbscan(X, min_samples=ms, min_cluster_size=mcs, reproducible=True)
    np.testing.assert_array_equal(labels, orc.labels)
    np.testing.assert_array_equal(probs, orc.probabilities)
