"""Batched independent fits (fhg_hdbscan_fit_batch): every instance equals its
single fit, whatever the number of worker streams."""
import numpy as np
import pytest

from fast_hdbscan_gb300 import synthetic

pytestmark = pytest.mark.gpu


def test_fit_many_equals_single_fits(engine):
    from fast_hdbscan_gb300.batch import fit_many
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan

    inst = synthetic.batch_instances(48, seed=21, n_min=200, n_max=20_000)
    Xs = [X for X, _, _ in inst]
    ms = [m for _, m, _ in inst]
    mcs = [c for _, _, c in inst]
    many = fit_many(Xs, min_samples=ms, min_cluster_size=mcs, workers=8)
    for (X, m, c), (lab, prob) in zip(inst, many):
        want_l, want_p = fast_hdbscan(X, min_samples=m, min_cluster_size=c)
        np.testing.assert_array_equal(lab, want_l)
        np.testing.assert_array_equal(prob, want_p)
    one = fit_many(Xs, min_samples=ms, min_cluster_size=mcs, workers=1)
    for (a, b), (c, d) in zip(many, one):
        np.testing.assert_array_equal(a, c)
        np.testing.assert_array_equal(b, d)


def test_fit_many_degenerate_and_leaf(engine):
    from fast_hdbscan_gb300.batch import fit_many
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan

    X = synthetic.blobs_2d(3000, seed=3)
    res = fit_many([X, np.zeros((1, 2), np.float32), X[:500]], min_samples=5,
                   min_cluster_size=20, cluster_selection_method="leaf", workers=3)
    assert np.all(res[1][0] == -1) and res[1][1].shape == (1,)
    for got, Y in ((res[0], X), (res[2], X[:500])):
        want = fast_hdbscan(Y, min_samples=5, min_cluster_size=20,
                            cluster_selection_method="leaf")
        np.testing.assert_array_equal(got[0], want[0])
        np.testing.assert_array_equal(got[1], want[1])


def test_autotuned_workers(engine):
    """The worker autotuner picks one of its candidates, remembers it for the
    batch's size signature, and fit_many(workers="auto") gives the same
    results as any fixed count."""
    from fast_hdbscan_gb300 import batch

    inst = synthetic.batch_instances(40, seed=22, n_min=200, n_max=5_000)
    Xs = [X for X, _, _ in inst]
    ms = [m for _, m, _ in inst]
    mcs = [c for _, _, c in inst]
    best, times = batch.autotune_workers(Xs, ms, mcs, candidates=(2, 8), sample=16)
    assert best in (2, 8) and set(times) == {2, 8}
    assert batch._TUNED[batch._signature(Xs)] == best
    auto = batch.fit_many(Xs, ms, mcs, workers="auto")
    fixed = batch.fit_many(Xs, ms, mcs, workers=3)
    for (a, b), (c, d) in zip(auto, fixed):
        np.testing.assert_array_equal(a, c)
        np.testing.assert_array_equal(b, d)


def test_fit_many_input_checks(engine):
    """A non-finite instance is rejected (checked on the GPU after the one
    upload), as is a row wider than 30; float64 instances give the float32
    fits."""
    import pytest as _pytest

    from fast_hdbscan_gb300.batch import fit_many

    X = synthetic.blobs_2d(2000, seed=5)
    Y = X[:700].copy()
    Y[13, 1] = np.nan
    with _pytest.raises(ValueError):
        fit_many([X, Y], min_samples=5, min_cluster_size=20)
    with _pytest.raises(ValueError):
        fit_many([np.zeros((10, 31), np.float32)], min_samples=5, min_cluster_size=5)
    a = fit_many([X, X[:900]], min_samples=5, min_cluster_size=20)
    b = fit_many([X.astype(np.float64), X[:900].astype(np.float64)], min_samples=5,
                 min_cluster_size=20)
    for (p, q), (r, s) in zip(a, b):
        np.testing.assert_array_equal(p, r)
        np.testing.assert_array_equal(q, s)
