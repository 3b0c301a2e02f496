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
                "vd3d_5k", "vd3d_20k", "edge_two", "edge_dups", "edge_1d", "edge_highms",
                "blobs2d_2k_ms100", "vd3d_3k_mcs120"]


# rows with equal distances inside the list: the reference lists them in its
# traversal order, the engine (and oracle mode 1) by index
TIED_ROWS = {"edge_dups", "vd3d_3k_mcs120"}


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
    if name not in TIED_ROWS:
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
    if name not in TIED_ROWS:
        np.testing.assert_array_equal(nbrs, g["neighbors"])
    # canonical oracle: the raw edge list itself
    oe, onb, oc, _ = O.parallel_boruvka(O.build_kdtree(X), ms, mode=1)
    np.testing.assert_array_equal(edges, oe)
    np.testing.assert_array_equal(nbrs, onb)
    np.testing.assert_array_equal(core, oc)


# kNN lists longer than 64 (kept in shared memory, a warp per query):
# every dimension family, ties on integer grids, k above n
@pytest.mark.parametrize("case,k", [
    ("vd3d_20k", 65), ("vd3d_20k", 200), ("blobs2d_2k", 129), ("umap5d_5k", 96),
    ("hd12_2k", 100), ("hd24_1k", 300), ("edge_1d", 150), ("grid2d", 97), ("grid3d", 250),
    ("ka150", 180),
])
def test_knn_long_lists_vs_oracle(engine, case, k):
    from fast_hdbscan_gb300.numba_kdtree import build_kdtree, parallel_tree_query
    from oracle import oracle as O

    if case.startswith("grid"):
        d = int(case[4])
        X = np.random.default_rng(d).integers(0, 12, size=(3000, d)).astype(np.float32)
    else:
        X = _golden(case)["X"]
    tree = build_kdtree(X)
    rd, ix = parallel_tree_query(tree, tree.data, k=k, output_rdist=True)
    ord_, oix = O.tree_query(O.build_kdtree(X), k, mode=1)
    np.testing.assert_array_equal(rd, ord_)
    np.testing.assert_array_equal(ix, oix)


@pytest.mark.parametrize("gen,n,ms", [
    ("varying_density", 30_000, 100),
    ("blobs_2d", 20_000, 250),
])
def test_boruvka_long_lists_vs_oracle(engine, gen, n, ms):
    from fast_hdbscan_gb300.numba_kdtree import build_kdtree
    from fast_hdbscan_gb300.boruvka import parallel_boruvka
    from oracle import oracle as O

    X = getattr(synthetic, gen)(n, seed=124)
    edges, nbrs, core = parallel_boruvka(build_kdtree(X), 1, min_samples=ms)
    oe, onb, oc, _ = O.parallel_boruvka(O.build_kdtree(X), ms, mode=1, nthreads=8)
    np.testing.assert_array_equal(core, oc)
    np.testing.assert_array_equal(nbrs, onb)
    np.testing.assert_array_equal(edges, oe)


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
