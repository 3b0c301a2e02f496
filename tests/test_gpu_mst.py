"""GPU parity of the core-distance (kNN) and Boruvka MST kernels.

Against the reference fixtures (tests/golden, produced by the unmodified
reference): squared kNN distances and core distances are bit-identical and
the MST weight multiset is identical.  Against the CPU oracle in canonical
tie-breaking mode: kNN indices, core distances and the raw MST (edge order,
orientation and weights) are bit-identical.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from fast_hdbscan_gb300 import synthetic

pytestmark = pytest.mark.gpu

GOLDEN_CASES = ["ka150", "blobs200", "blobs200_ms1", "blobs2d_2k", "blobs2d_20k", "umap5d_5k",
                "vd3d_5k", "vd3d_20k", "edge_two", "edge_dups", "edge_1d", "edge_highms"]


def _golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_knn_bitexact_vs_reference(engine, name):
    from fast_hdbscan_gb300.numba_kdtree import build_kdtree, parallel_tree_query
    from oracle import oracle as O

    g = _golden(name)
    X = g["X"]
    k = g["knn_rdist"].shape[1]
    tree = build_kdtree(X)
    rd, ix = parallel_tree_query(tree, tree.data, k=k, output_rdist=True)
    np.testing.assert_array_equal(rd, g["knn_rdist"])
    ord_, oix = O.tree_query(O.build_kdtree(X), k, mode=1)
    np.testing.assert_array_equal(rd, ord_)
    np.testing.assert_array_equal(ix, oix)
    if name != "edge_dups":  # all-duplicate rows: the reference orders ties by traversal
        np.testing.assert_array_equal(ix, g["knn_idx"])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_boruvka_vs_reference_and_oracle(engine, name):
    from fast_hdbscan_gb300.numba_kdtree import build_kdtree
    from fast_hdbscan_gb300.boruvka import parallel_boruvka
    from oracle import oracle as O

    g = _golden(name)
    X = g["X"]
    ms = int(g["min_samples"])
    edges, nbrs, core = parallel_boruvka(build_kdtree(X), 1, min_samples=ms)
    # reference: core distances bit-exact, MST weight multiset identical
    np.testing.assert_array_equal(core, g["core"])
    np.testing.assert_array_equal(np.sort(edges[:, 2]), np.sort(g["mst_raw"][:, 2]))
    if name != "edge_dups":
        np.testing.assert_array_equal(nbrs, g["neighbors"])
    # canonical oracle: the raw edge list itself
    oe, onb, oc, _ = O.parallel_boruvka(O.build_kdtree(X), ms, mode=1)
    np.testing.assert_array_equal(edges, oe)
    np.testing.assert_array_equal(nbrs, onb)
    np.testing.assert_array_equal(core, oc)


@pytest.mark.parametrize("gen,n,ms", [
    ("varying_density", 100_000, 15),
    ("blobs_2d", 100_000, 10),
    ("umap_like", 50_000, 10),
    ("varying_density", 30_000, 5),
    ("blobs_2d", 30_000, 1),
])
def test_boruvka_vs_oracle_synthetic(engine, gen, n, ms):
    from fast_hdbscan_gb300.numba_kdtree import build_kdtree
    from fast_hdbscan_gb300.boruvka import parallel_boruvka
    from oracle import oracle as O

    X = getattr(synthetic, gen)(n, seed=123)
    edges, nbrs, core = parallel_boruvka(build_kdtree(X), 1, min_samples=ms)
    oe, onb, oc, _ = O.parallel_boruvka(O.build_kdtree(X), ms, mode=1, nthreads=8)
    np.testing.assert_array_equal(core, oc)
    np.testing.assert_array_equal(nbrs, onb)
    np.testing.assert_array_equal(edges, oe)
