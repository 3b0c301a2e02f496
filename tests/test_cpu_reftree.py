"""Host side of the reference KD-tree (no GPU): the node ranges and leaf
flags follow from n alone, and the level count is the reference's formula
(numba_kdtree.py:486); both against the oracle's restated build."""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.mark.parametrize("n", [1, 2, 3, 40, 41, 81, 82, 83, 1000, 4097, 65_537, 300_001])
def test_node_ranges_match_the_reference_build(n):
    from fast_hdbscan_gb300 import _native
    from fast_hdbscan_gb300.numba_kdtree import node_ranges

    levels = int(np.log2(max(1, (n - 1) / 40)) + 1)
    assert _native.load().fhg_reference_kdtree_levels(n) == levels
    X = np.random.default_rng(n).standard_normal((n, 2)).astype(np.float32)
    a = O.build_kdtree(X).arrays()
    start, end, leaf = node_ranges(n, levels)
    np.testing.assert_array_equal(start, a["idx_start"])
    np.testing.assert_array_equal(end, a["idx_end"])
    np.testing.assert_array_equal(leaf, a["is_leaf"])
