"""End-to-end GPU fit parity.

* Against the CPU oracle in canonical tie-breaking mode: every output of the
  fit (labels, probabilities, sorted MST, linkage tree, condensed tree,
  neighbours, core distances) is bit-identical.
* Against the reference fixtures: core distances and the MST weight multiset
  are bit-identical.  Where the reference's MST equals ours edge for edge,
  labels and probabilities are bit-identical.  Where the reference broke a
  tie between equal mutual-reachability weights differently (it keeps the
  first candidate met in its KD-tree traversal order, which no other index
  reproduces), the cluster count is equal and -- after the majority-vote
  label alignment the reference's own back-end parity tests use
  (fast_hdbscan/tests/test_hdbscan.py:501-566) -- labels and probabilities
  are identical at every point that is not an endpoint of a tie-broken edge.
"""
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN
from fast_hdbscan_gb300 import synthetic
from parity import assert_reference_parity

pytestmark = pytest.mark.gpu

GOLDEN_FIT = ["ka150", "ka150_eps", "blobs200", "blobs200_ms1", "blobs200_leaf",
              "blobs200_maxcs", "blobs200_single", "blobs200_persist", "blobs2d_2k",
              "blobs2d_20k", "umap5d_5k", "vd3d_5k", "vd3d_20k", "edge_two", "edge_1d",
              "edge_highms", "edge_dups", "edge_mcs_gt_n", "blobs200_w_labels", "blobs2d_2k_w",
              "vd3d_5k_w", "hd12_2k", "hd24_1k", "blobs2d_2k_ms100", "vd3d_3k_mcs120"]


def _golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def _kw(g):
    return dict(cluster_selection_method=str(g["cluster_selection_method"]),
                max_cluster_size=float(g["max_cluster_size"]),
                allow_single_cluster=bool(g["allow_single_cluster"]),
                cluster_selection_epsilon=float(g["cluster_selection_epsilon"]),
                cluster_selection_persistence=float(g["cluster_selection_persistence"]))


def _assert_fit_equal(res, orc):
    labels, probs, linkage, ct, smst, nbrs, core = res
    np.testing.assert_array_equal(core, orc.core)
    np.testing.assert_array_equal(nbrs, orc.neighbors)
    np.testing.assert_array_equal(smst, orc.sorted_mst)
    np.testing.assert_array_equal(linkage, orc.linkage)
    for a, b in zip(ct, orc.condensed):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(labels, orc.labels)
    np.testing.assert_array_equal(probs, orc.probabilities)


@pytest.mark.parametrize("name", GOLDEN_FIT)
def test_fit_vs_oracle_and_reference(engine, name):
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan
    from oracle import oracle as O

    g = _golden(name)
    X = g["X"]
    ms, mcs = int(g["min_samples"]), int(g["min_cluster_size"])
    w = g["sample_weights"] if "sample_weights" in g.files else None
    res = fast_hdbscan(X, min_samples=ms, min_cluster_size=mcs, return_trees=True,
                       sample_weights=w, **_kw(g))
    orc = O.fit(X, ms, mcs, mode=1, sample_weights=w, **_kw(g))
    _assert_fit_equal(res, orc)
    # reference fixtures
    if name != "edge_mcs_gt_n":  # the reference indexes [-1] when k exceeds n
        np.testing.assert_array_equal(res[6], g["core"])
        np.testing.assert_array_equal(np.sort(res[4][:, 2]), np.sort(g["sorted_mst"][:, 2]))
    if name != "edge_mcs_gt_n":  # duplicate points: every distance among them ties
        assert_reference_parity(res[0], res[1], orc.mst, g,
                                max_share=1.0 if name == "edge_dups" else 0.02)
    else:
        np.testing.assert_array_equal(res[0], g["labels"])
        np.testing.assert_array_equal(res[1], g["probabilities"])


@pytest.mark.parametrize("gen,n,ms,mcs", [
    ("varying_density", 200_000, 15, 100),
    ("blobs_2d", 200_000, 10, 50),
    ("umap_like", 100_000, 10, 100),
    ("varying_density", 50_000, 5, 20),
    ("blobs_2d", 50_000, 1, 10),
])
def test_fit_vs_oracle_synthetic(engine, gen, n, ms, mcs):
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan
    from oracle import oracle as O

    X = getattr(synthetic, gen)(n, seed=321)
    res = fast_hdbscan(X, min_samples=ms, min_cluster_size=mcs, return_trees=True)
    orc = O.fit(X, ms, mcs, mode=1, nthreads=8)
    _assert_fit_equal(res, orc)


def test_estimator_api(engine):
    from fast_hdbscan_gb300 import HDBSCAN

    np.random.seed(0)
    X = np.random.rand(150, 2)
    c = HDBSCAN(min_cluster_size=5).fit(X)
    u, counts = np.unique(c.labels_, return_counts=True)
    assert len(u) == 8 and counts[u == -1] == 69
    assert c.probabilities_.dtype == np.float32
    assert c._condensed_tree.dtype.names == ("parent", "child", "lambda_val", "child_size")
    assert np.array_equal(HDBSCAN(min_cluster_size=5).fit_predict(X), c.labels_)


def test_missing_data_remap(engine):
    from fast_hdbscan_gb300 import HDBSCAN

    g = _golden("blobs200")
    X = g["X"].astype(np.float64)
    Xm = X.copy()
    Xm[0] = [np.nan, 1]
    Xm[5] = [np.nan, np.nan]
    model = HDBSCAN().fit(Xm)
    assert model.labels_[0] == -1 and model.labels_[5] == -1
    assert model.probabilities_[0] == 0 and model.probabilities_[5] == 0
    clean = list(range(1, 5)) + list(range(6, 200))
    clean_model = HDBSCAN().fit(Xm[clean])
    assert np.allclose(clean_model.labels_, model.labels_[clean])


def test_fast_hdbscan_non_finite_raises(engine):
    """hdbscan.py:233 check_array: the functional entry point rejects NaN and
    infinity (checked on the device copy) with the host check's ValueError,
    and a finite float64 input fits as its float32 copy."""
    from fast_hdbscan_gb300.hdbscan import check_array, fast_hdbscan

    X = _golden("blobs200")["X"].astype(np.float64)
    for bad in (np.nan, np.inf, -np.inf):
        Xb = X.copy()
        Xb[7, 1] = bad
        with pytest.raises(ValueError) as host:
            check_array(Xb)
        with pytest.raises(ValueError, match=re.escape(str(host.value).splitlines()[0][:20])):
            fast_hdbscan(Xb)
    a = fast_hdbscan(X)
    b = fast_hdbscan(X.astype(np.float32))
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_cached_pool_release_between_fits(engine):
    """Scratch comes from the engine's caching pool: a fit after the pool has
    handed its cached blocks back gives the same result."""
    from fast_hdbscan_gb300 import _native
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan

    X = synthetic.varying_density(30_000, seed=5)
    a = fast_hdbscan(X, min_samples=10, min_cluster_size=40)
    _native.release_cached_memory()
    b = fast_hdbscan(X, min_samples=10, min_cluster_size=40)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_sample_weight_known_answer(engine):
    """fast_hdbscan/tests/test_hdbscan.py:112-117: weights = the blob labels
    (one blob weighs 0) leave n_clusters - 1 clusters."""
    from fast_hdbscan_gb300 import HDBSCAN
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan

    g = _golden("blobs200_w_labels")
    labels, _ = fast_hdbscan(g["X"], sample_weights=g["sample_weights"], min_cluster_size=5,
                             min_samples=None)
    assert len(set(labels.tolist()) - {-1}) == 2
    model = HDBSCAN(min_cluster_size=5).fit(g["X"], sample_weight=g["sample_weights"])
    np.testing.assert_array_equal(model.labels_, labels)


@pytest.mark.parametrize("n,seed", [(100_000, 8), (40_000, 9)])
def test_weighted_fit_vs_oracle_synthetic(engine, n, seed):
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan
    from oracle import oracle as O

    X = synthetic.varying_density(n, seed=seed)
    w = np.random.default_rng(seed).integers(1, 5, n).astype(np.float32)
    res = fast_hdbscan(X, min_samples=10, min_cluster_size=50, return_trees=True,
                       sample_weights=w)
    orc = O.fit(X, 10, 50, mode=1, nthreads=8, sample_weights=w)
    _assert_fit_equal(res, orc)


def test_estimator_condensed_record_array_on_gpu(engine):
    """HDBSCAN.fit stores hdbscan.py:93 to_numpy_rec_array(condensed tree); the
    engine lays the records out on the GPU -- same bytes as the host conversion."""
    from fast_hdbscan_gb300 import HDBSCAN
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan, to_numpy_rec_array

    g = _golden("blobs2d_2k")
    model = HDBSCAN(min_cluster_size=50, min_samples=10).fit(g["X"])
    ct = fast_hdbscan(g["X"], min_samples=10, min_cluster_size=50, return_trees=True)[3]
    want = to_numpy_rec_array(ct)
    assert model._condensed_tree.dtype == want.dtype
    assert model._condensed_tree.tobytes() == want.tobytes()
    np.testing.assert_array_equal(model.labels_, fast_hdbscan(g["X"], min_samples=10,
                                                              min_cluster_size=50)[0])


@pytest.mark.parametrize("n,dim,ms,mcs", [(100_000, 16, 10, 100), (30_000, 30, 10, 50),
                                          (50_000, 11, 5, 30)])
def test_high_dimensional_fit_vs_oracle(engine, n, dim, ms, mcs):
    """9-32 dimensions: the kernels run over the padded width (16 or 32); the
    padding adds exact zeros, so every output matches the oracle bit for bit."""
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan
    from oracle import oracle as O

    X = synthetic.umap_like(n, seed=40 + dim, dim=dim, n_blobs=12)
    res = fast_hdbscan(X, min_samples=ms, min_cluster_size=mcs, return_trees=True)
    orc = O.fit(X, ms, mcs, mode=1, nthreads=16)
    _assert_fit_equal(res, orc)


def test_fit_export_copies_match_device_outputs(engine):
    """fhg_hdbscan_fit_export: the host copies it overlaps with the later stages
    equal the device outputs of the same fit, byte for byte, whether the host
    destinations are pinned or pageable; an exported output without its device
    buffer is refused."""
    import ctypes

    import torch

    from fast_hdbscan_gb300 import _native

    X = synthetic.varying_density(50_000, seed=21)
    n, d, ms, mcs = X.shape[0], X.shape[1], 7, 40
    lib = _native.load()
    V = _native.vptr
    Xd = torch.from_numpy(X).cuda()

    def dev(shape, dt):
        return torch.empty(shape, dtype=dt, device="cuda")

    for pinned in (True, False):
        labels, probs = dev(n, torch.int64), dev(n, torch.float32)
        mst, link = dev((n - 1, 3), torch.float64), dev((n - 1, 4), torch.float64)
        ctp, ctc = dev(2 * n, torch.int64), dev(2 * n, torch.int64)
        ctl, cts = dev(2 * n, torch.float32), dev(2 * n, torch.float32)
        nbrs, core, sel = dev((n, ms), torch.int32), dev(n, torch.float32), dev(n, torch.int64)
        rec = dev(2 * n * 28, torch.uint8)
        hosts = [torch.empty(t.shape, dtype=t.dtype, pin_memory=pinned)
                 for t in (nbrs, core, mst, link, rec)]
        rows, nsel = ctypes.c_int64(0), ctypes.c_int64(0)
        _native.check(lib.fhg_hdbscan_fit_export(
            V(Xd), n, d, ms, mcs, 0, float("inf"), 0, 0.0, 0.0, None, 0, V(labels), V(probs),
            V(mst), V(link), V(ctp), V(ctc), V(ctl), V(cts), ctypes.byref(rows), V(nbrs),
            V(core), V(sel), ctypes.byref(nsel), *[_native.hptr(h) for h in hosts[:4]], V(rec),
            _native.hptr(hosts[4]), _native.stream_ptr()))
        torch.cuda.current_stream().synchronize()
        r = rows.value
        for h, t in zip(hosts[:4], (nbrs, core, mst, link)):
            assert torch.equal(h, t.cpu())
        assert torch.equal(hosts[4][: r * 28], rec[: r * 28].cpu())
        want = torch.empty(max(r, 1) * 28, dtype=torch.uint8, device="cuda")
        _native.check(lib.fhg_condensed_record_array(V(ctp), V(ctc), V(ctl), V(cts), r,
                                                      V(want), _native.stream_ptr()))
        assert torch.equal(hosts[4][: r * 28], want[: r * 28].cpu())
    # the same fit through fhg_hdbscan_fit
    labels2, probs2 = dev(n, torch.int64), dev(n, torch.float32)
    _native.check(lib.fhg_hdbscan_fit(
        V(Xd), n, d, ms, mcs, 0, float("inf"), 0, 0.0, 0.0, None, 0, V(labels2), V(probs2),
        None, None, None, None, None, None, ctypes.byref(rows), None, None, None,
        ctypes.byref(nsel), _native.stream_ptr()))
    assert torch.equal(labels, labels2) and torch.equal(probs, probs2)
    h = torch.empty(n, dtype=torch.float32, pin_memory=True)
    rc = lib.fhg_hdbscan_fit_export(
        V(Xd), n, d, ms, mcs, 0, float("inf"), 0, 0.0, 0.0, None, 0, V(labels), V(probs),
        None, None, None, None, None, None, ctypes.byref(rows), None, None, None,
        ctypes.byref(nsel), None, _native.hptr(h), None, None, None, None, _native.stream_ptr())
    assert rc == _native.FHG_ERR_INVALID
    assert "device buffer" in lib.fhg_last_error().decode()


@pytest.mark.parametrize("seed,d,side,n,ms,mcs", [
    (0, 2, 200, 20_000, 10, 20), (1, 3, 40, 30_000, 5, 10), (2, 5, 8, 20_000, 3, 5),
    (3, 2, 120, 8_000, 1, 5), (4, 3, 25, 12_000, 15, 40), (5, 4, 12, 15_000, 7, 15),
])
def test_fit_vs_oracle_integer_grid(engine, seed, d, side, n, ms, mcs):
    """Distinct points of an integer grid: squared distances and core
    distances tie everywhere, so every tie rule of the canonical mode (kNN
    lists by (distance, index), a point's candidate by (weight, index), a
    component's edge by (weight, min index, max index), orientation, sort,
    condensed tree) is exercised; every output equals the oracle's bit for
    bit."""
    from fast_hdbscan_gb300.hdbscan import fast_hdbscan
    from oracle import oracle as O

    rng = np.random.default_rng(1000 + seed)
    cells = rng.choice(side ** d, size=n, replace=False)
    X = np.stack([(cells // side ** j) % side for j in range(d)], axis=1).astype(np.float32)
    res = fast_hdbscan(X, min_samples=ms, min_cluster_size=mcs, return_trees=True)
    orc = O.fit(X, ms, mcs, mode=1, nthreads=8)
    _assert_fit_equal(res, orc)
