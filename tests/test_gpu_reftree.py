"""The reference's own KD-tree, built on the GPU (fhg_reference_kdtree):
idx_array, idx_start, idx_end, is_leaf and node_bounds equal the arrays of
the reference's build_kdtree (numba_kdtree.py:478) -- on the fixtures
written by the reference, and against the oracle's restatement of the
build on inputs that exercise every branch of its introselect (sizes up to
1M, duplicate coordinates, 1 to 12 dimensions, trees of a single leaf)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from fast_hdbscan_gb300 import synthetic

pytestmark = pytest.mark.gpu

FIXTURES = sorted(n[:-4] for n in os.listdir(GOLDEN)
                  if n.endswith(".npz") and "kd_idx_array" in np.load(os.path.join(GOLDEN, n)).files)


def _assert_tree_equal(tree, want):
    np.testing.assert_array_equal(tree.idx_array, want["idx_array"])
    np.testing.assert_array_equal(tree.idx_start, want["idx_start"])
    np.testing.assert_array_equal(tree.idx_end, want["idx_end"])
    np.testing.assert_array_equal(tree.is_leaf, want["is_leaf"])
    np.testing.assert_array_equal(tree.node_bounds, want["node_bounds"])


@pytest.mark.parametrize("name", FIXTURES)
def test_reference_kdtree_fixture(engine, name):
    from fast_hdbscan_gb300.numba_kdtree import build_reference_kdtree

    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    tree = build_reference_kdtree(g["X"])
    _assert_tree_equal(tree, {k: g["kd_" + k] for k in
                              ("idx_array", "idx_start", "idx_end", "is_leaf", "node_bounds")})


def _cases():
    rng = np.random.default_rng(4)
    grid = rng.integers(0, 6, size=(30_000, 2)).astype(np.float32)  # many equal coordinates
    return [
        ("varying_density_1m", synthetic.varying_density(1_000_000, seed=2)),
        ("varying_density_100k", synthetic.varying_density(100_000, seed=3)),
        ("blobs_2d_50k", synthetic.blobs_2d(50_000, seed=4)),
        ("umap_like_40k_5d", synthetic.umap_like(40_000, seed=5, dim=5)),
        ("grid_ties_30k", grid),
        ("line_1d_20k", rng.standard_normal((20_000, 1)).astype(np.float32)),
        ("d12_8k", rng.standard_normal((8_000, 12)).astype(np.float32)),
        ("sorted_axis_10k", np.sort(rng.standard_normal((10_000, 3)).astype(np.float32), axis=0)),
        ("tiny_70", rng.standard_normal((70, 3)).astype(np.float32)),
        ("tiny_2", rng.standard_normal((2, 2)).astype(np.float32)),
    ]


@pytest.mark.parametrize("case", range(10))
def test_reference_kdtree_vs_oracle(engine, case):
    from fast_hdbscan_gb300.numba_kdtree import build_reference_kdtree
    from oracle import oracle as O

    name, X = _cases()[case]
    tree = build_reference_kdtree(X)
    _assert_tree_equal(tree, O.build_kdtree(X).arrays())
