"""Shared checks for comparing a GPU fit with the reference's tie choices.

The reference keeps, among equal mutual-reachability weights, the edge its
own KD-tree traversal meets first; the engine's default mode breaks the same
ties by a total order on point indices.  Both give a minimum spanning tree of
the same weights, so where they differ the difference is confined to
tie-broken edges -- which these helpers check instead of assuming.
"""
import numpy as np
import pytest

# At most this share of the points may sit on tie-broken edges; a larger
# divergence means a wrong tree, not a different tie choice.
MAX_TIE_POINT_SHARE = 0.02


def adjusted_rand_index(a, b):
    """Adjusted Rand index of two labelings (noise counts as one label), from
    the contingency table; numpy only."""
    a = np.asarray(a)
    b = np.asarray(b)
    _, ai = np.unique(a, return_inverse=True)
    _, bi = np.unique(b, return_inverse=True)
    pairs = ai.astype(np.int64) * (bi.max() + 1) + bi
    _, cnt = np.unique(pairs, return_counts=True)

    def comb2(x):
        x = x.astype(np.float64)
        return (x * (x - 1) / 2).sum()

    sum_ij = comb2(cnt)
    sum_a = comb2(np.bincount(ai))
    sum_b = comb2(np.bincount(bi))
    total = comb2(np.array([len(a)]))
    expected = sum_a * sum_b / total if total else 0.0
    top = 0.5 * (sum_a + sum_b)
    if top == expected:
        return 1.0
    return float((sum_ij - expected) / (top - expected))


def align_labels(ref, other):
    """Majority-vote relabelling of `other` onto `ref` (noise passes through),
    as the reference's own back-end parity tests do
    (fast_hdbscan/tests/test_hdbscan.py:501-566)."""
    ref = np.asarray(ref)
    other = np.asarray(other)
    keep = (ref != -1) & (other != -1)
    remap = {}
    if keep.any():
        o, r = other[keep], ref[keep]
        pairs, cnt = np.unique(np.stack([o, r], 1), axis=0, return_counts=True)
        order = np.lexsort((-cnt, pairs[:, 0]))  # per label of `other`, most common first
        pairs = pairs[order]
        first = np.r_[True, pairs[1:, 0] != pairs[:-1, 0]]
        remap = dict(zip(pairs[first, 0].tolist(), pairs[first, 1].tolist()))
    if not remap:
        return other.copy()
    keys = np.array(sorted(remap), dtype=np.int64)
    vals = np.array([remap[k] for k in keys.tolist()], dtype=np.int64)
    pos = np.clip(np.searchsorted(keys, other), 0, len(keys) - 1)
    hit = keys[pos] == other
    return np.where(hit, vals[pos], other).astype(other.dtype)


def _edge_keys(mst, n):
    a = np.minimum(mst[:, 0], mst[:, 1]).astype(np.int64)
    b = np.maximum(mst[:, 0], mst[:, 1]).astype(np.int64)
    return a * (n + 1) + b


def tie_report(labels, probs, mst, ref_labels, ref_probs, ref_mst,
               max_share=MAX_TIE_POINT_SHARE):
    """Checks that two fits differ only through equal-weight MST choices and
    returns (ari, differing label points, differing probability points,
    points on tie-broken edges).  Inputs with duplicate points tie
    everywhere and may pass a larger max_share."""
    n = len(labels)
    np.testing.assert_array_equal(np.sort(mst[:, 2]), np.sort(ref_mst[:, 2]))
    assert mst[:, 2].sum() == pytest.approx(ref_mst[:, 2].sum(), rel=1e-12)
    ko, kt = _edge_keys(mst, n), _edge_keys(ref_mst, n)
    only_o = ~np.isin(ko, kt)
    only_t = ~np.isin(kt, ko)
    np.testing.assert_array_equal(np.sort(mst[only_o, 2]), np.sort(ref_mst[only_t, 2]),
                                  err_msg="edges outside the other tree are not equal-weight "
                                          "alternatives")
    tie_points = np.unique(np.concatenate([mst[only_o, :2].ravel(),
                                           ref_mst[only_t, :2].ravel()]).astype(np.int64))
    aligned = align_labels(ref_labels, labels)
    bad_l = np.nonzero(aligned != ref_labels)[0]
    bad_p = np.nonzero(probs != ref_probs)[0]
    assert np.isin(bad_l, tie_points).all(), "a label differs away from every tie-broken edge"
    assert np.isin(bad_p, tie_points).all(), \
        "a probability differs away from every tie-broken edge"
    assert len(tie_points) <= max(20, max_share * n), \
        f"{len(tie_points)} points on tie-broken edges"
    return adjusted_rand_index(ref_labels, labels), len(bad_l), len(bad_p), len(tie_points)


def assert_reference_parity(labels, probs, mst, g, max_share=MAX_TIE_POINT_SHARE):
    """Parity with a reference fixture, up to the reference's tie choices."""
    ref_labels, ref_probs = g["labels"], g["probabilities"].astype(np.float32)
    assert len(set(labels.tolist()) - {-1}) == len(set(ref_labels.tolist()) - {-1})
    if np.array_equal(mst, g["mst_raw"]):
        np.testing.assert_array_equal(labels, ref_labels)
        np.testing.assert_array_equal(probs, ref_probs)
        return
    tie_report(labels, probs, mst, ref_labels, ref_probs, g["mst_raw"], max_share)
