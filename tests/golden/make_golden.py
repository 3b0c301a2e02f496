"""Generate golden HDBSCAN fixtures from the unmodified fast_hdbscan reference.

The reference (fast_hdbscan 0.3.2, pure Python + Numba) is imported from a
checkout given by ``--reference`` (default: the read-only copy mounted in the
build container) with ``numba_shim/`` first on ``sys.path``: the shim turns
``@njit`` into a no-op and ``prange`` into ``range``, so the reference runs its
own code unmodified as plain Python, with its parallel loops sequential.

Each case writes ``<name>.npz`` beside this script holding the float32 input,
the parameters and every intermediate of the fit path:

  knn_rdist, knn_idx         parallel_tree_query(tree, data, k=ms+1, output_rdist=True)
  core                        sqrt of the k-th squared kNN distance (float32)
  mst_raw                     compute_minimum_spanning_tree edges, unsorted
  sorted_mst, linkage         clusters_from_spanning_tree outputs
  ct_parent/child/lambda/size the CondensedTree namedtuple
  selected                    the selected cluster ids
  labels, probabilities       final outputs
  kd_*                        the reference KD-tree arrays (small cases only)

Other families: ``fn_*`` (function-level cases), ``kr_*`` (algorithm="kruskal"),
``pc_*`` (metric="precomputed"), ``sc_*`` (BranchDetector / SubClusterDetector on
the reference's own fits) and ``cg_*`` (the reference's core graph and its
Boruvka forest, core_graph.py:19/:198).

Run:  python tests/golden/make_golden.py [--only NAME ...]
      (--kruskal-only / --precomputed-only / --subclusters-only for one family)
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(HERE, "numba_shim"))
sys.path.insert(0, REPO)

from fast_hdbscan_gb300 import synthetic  # noqa: E402


def _blobs200():
    from sklearn.datasets import make_blobs
    from sklearn.preprocessing import StandardScaler
    from sklearn.utils import shuffle

    X, y = make_blobs(n_samples=200, random_state=10)
    X, y = shuffle(X, y, random_state=7)
    return StandardScaler().fit_transform(X)


def _blobs200_labels():
    from sklearn.datasets import make_blobs
    from sklearn.utils import shuffle

    X, y = make_blobs(n_samples=200, random_state=10)
    X, y = shuffle(X, y, random_state=7)
    return y.astype(np.float32)


def _weights_sixty_fourths(n, seed):
    """Multiples of 1/64 in [0.5, 2]: float32 sums of them are exact, so the
    weighted k and the weighted tree sizes do not depend on summation order."""
    rng = np.random.default_rng(seed)
    return (rng.integers(32, 129, n) / 64.0).astype(np.float32)


def _rand(seed, n, d):
    np.random.seed(seed)
    return np.random.rand(n, d)


def _one_d():
    np.random.seed(42)
    return np.concatenate(
        [np.random.normal(0, 0.1, 50), np.random.normal(5, 0.1, 50)]
    ).reshape(-1, 1)


CASES = {
    # name: (data factory, fit kwargs)
    "ka150": (lambda: _rand(0, 150, 2), dict(min_cluster_size=5)),
    "ka150_eps": (lambda: _rand(0, 150, 2),
                  dict(min_cluster_size=5, cluster_selection_epsilon=0.2)),
    "blobs200": (_blobs200, dict(min_cluster_size=5)),
    "blobs200_ms1": (_blobs200, dict(min_cluster_size=5, min_samples=1)),
    "blobs200_leaf": (_blobs200, dict(min_cluster_size=5, cluster_selection_method="leaf")),
    "blobs200_maxcs": (_blobs200, dict(min_cluster_size=5, max_cluster_size=30)),
    "blobs200_single": (_blobs200, dict(min_cluster_size=5, allow_single_cluster=True)),
    "blobs200_persist": (_blobs200, dict(min_cluster_size=5, cluster_selection_persistence=0.5)),
    "blobs2d_2k": (lambda: synthetic.blobs_2d(2000, seed=10),
                   dict(min_samples=10, min_cluster_size=50)),
    "blobs2d_20k": (lambda: synthetic.blobs_2d(20000, seed=0),
                    dict(min_samples=10, min_cluster_size=50)),
    "umap5d_5k": (lambda: synthetic.umap_like(5000, seed=11),
                  dict(min_samples=10, min_cluster_size=25)),
    "vd3d_5k": (lambda: synthetic.varying_density(5000, seed=12),
                dict(min_samples=15, min_cluster_size=25)),
    "vd3d_20k": (lambda: synthetic.varying_density(20000, seed=13),
                 dict(min_samples=15, min_cluster_size=50)),
    # kNN lists longer than 64 (min_samples >= 64; the estimator's default
    # min_samples is min_cluster_size)
    "blobs2d_2k_ms100": (lambda: synthetic.blobs_2d(2000, seed=10),
                         dict(min_samples=100, min_cluster_size=100)),
    "vd3d_3k_mcs120": (lambda: synthetic.varying_density(3000, seed=14),
                       dict(min_cluster_size=120)),
    # sample weights (hdbscan.py:199 sample_weights; boruvka.py:527-573;
    # cluster_trees.py:98, :205)
    "blobs200_w_labels": (_blobs200, dict(min_cluster_size=5, sample_weights=_blobs200_labels)),
    "blobs2d_2k_w": (lambda: synthetic.blobs_2d(2000, seed=10),
                     dict(min_samples=10, min_cluster_size=50,
                          sample_weights=lambda: _weights_sixty_fourths(2000, 4))),
    "vd3d_5k_w": (lambda: synthetic.varying_density(5000, seed=12),
                  dict(min_samples=15, min_cluster_size=25,
                       sample_weights=lambda: np.random.default_rng(5).integers(
                           1, 4, 5000).astype(np.float32))),
    # more than 8 dimensions (the reference's KD-tree Boruvka path serves d <= 30)
    "hd12_2k": (lambda: synthetic.umap_like(2000, seed=31, dim=12, n_blobs=8),
                dict(min_samples=10, min_cluster_size=25)),
    "hd24_1k": (lambda: synthetic.umap_like(1000, seed=32, dim=24, n_blobs=6),
                dict(min_samples=8, min_cluster_size=20)),
    "edge_two": (lambda: np.array([[0.0, 0.0], [0.1, 0.0]]), dict(min_cluster_size=2)),
    "edge_dups": (lambda: np.full((50, 3), 1.0), dict(min_cluster_size=5)),
    "edge_1d": (_one_d, dict(min_cluster_size=10)),
    "edge_highms": (lambda: _rand(42, 20, 2), dict(min_cluster_size=5, min_samples=18)),
    "edge_mcs_gt_n": (lambda: _rand(42, 10, 2), dict(min_cluster_size=100)),
}


def run_case(name, factory, kwargs, ref):
    from fast_hdbscan.hdbscan import fast_hdbscan, compute_minimum_spanning_tree
    from fast_hdbscan.numba_kdtree import build_kdtree, parallel_tree_query
    from fast_hdbscan.cluster_trees import (
        cluster_tree_from_condensed_tree, extract_eom_clusters)

    X = np.ascontiguousarray(factory(), dtype=np.float32)
    kwargs = dict(kwargs)
    kwargs.setdefault("min_samples", None)  # the HDBSCAN estimator's default
    w = kwargs.pop("sample_weights", None)
    if w is not None:
        w = np.ascontiguousarray(w(), dtype=np.float32)
    mcs = kwargs.get("min_cluster_size", 5)
    ms = kwargs.get("min_samples") or mcs
    t0 = time.time()
    out = {"X": X, "min_samples": np.int64(ms), "min_cluster_size": np.int64(mcs)}
    for key in ("cluster_selection_epsilon", "cluster_selection_persistence",
                "max_cluster_size"):
        out[key] = np.float64(kwargs.get(key, np.inf if key == "max_cluster_size" else 0.0))
    out["allow_single_cluster"] = np.bool_(kwargs.get("allow_single_cluster", False))
    out["cluster_selection_method"] = np.array(kwargs.get("cluster_selection_method", "eom"))
    if w is not None:
        out["sample_weights"] = w

    if X.shape[0] >= 2 and w is not None:
        mst_raw, nbrs, core = compute_minimum_spanning_tree(X, min_samples=ms, sample_weights=w)
        out["mst_raw"] = mst_raw
        out["core"] = core
        out["neighbors"] = nbrs
    elif X.shape[0] >= 2:
        tree = build_kdtree(X)
        k = ms + 1 if ms > 1 else 2
        k = min(k, X.shape[0])
        rd, idx = parallel_tree_query(tree, tree.data, k=k, output_rdist=True)
        out["knn_rdist"], out["knn_idx"] = rd, idx
        if X.shape[0] <= 5000:
            out["kd_idx_array"] = tree.idx_array
            out["kd_idx_start"] = tree.idx_start
            out["kd_idx_end"] = tree.idx_end
            out["kd_is_leaf"] = tree.is_leaf
            out["kd_node_bounds"] = tree.node_bounds
        mst_raw, nbrs, core = compute_minimum_spanning_tree(X, min_samples=ms)
        out["mst_raw"] = mst_raw
        out["core"] = core
        out["neighbors"] = nbrs

    res = fast_hdbscan(X, return_trees=True, sample_weights=w, **kwargs)
    labels, probs, linkage, ct, smst, nbrs2, core2 = res
    out["labels"] = np.asarray(labels)
    out["probabilities"] = np.asarray(probs)
    out["linkage"] = np.asarray(linkage)
    out["sorted_mst"] = np.asarray(smst)
    if hasattr(ct, "parent") and not isinstance(ct, np.ndarray):
        out["ct_parent"] = np.asarray(ct.parent)
        out["ct_child"] = np.asarray(ct.child)
        out["ct_lambda"] = np.asarray(ct.lambda_val)
        out["ct_size"] = np.asarray(ct.child_size)
        if len(ct.parent) > 0:
            cl_tree = cluster_tree_from_condensed_tree(ct)
            out["selected_eom"] = np.asarray(extract_eom_clusters(
                ct, cl_tree, max_cluster_size=kwargs.get("max_cluster_size", np.inf),
                allow_single_cluster=kwargs.get("allow_single_cluster", False)))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(f"{name}: n={X.shape[0]} d={X.shape[1]} ms={ms} mcs={mcs} "
          f"clusters={len(set(out['labels'].tolist()) - {-1})} "
          f"noise={(out['labels'] == -1).sum()} ({time.time() - t0:.1f}s)")


def add_cuts(name):
    """DBSCAN cuts of the fixture's linkage tree (hdbscan.py:824 ->
    get_cluster_labelling_at_cut) at quantiles of its merge distances, with
    the estimator's min_cluster_size for the cut (min_samples when given)."""
    from fast_hdbscan.cluster_trees import get_cluster_labelling_at_cut

    path = os.path.join(HERE, name + ".npz")
    g = dict(np.load(path))
    lk = g["linkage"]
    if lk.shape[0] == 0:
        return
    finite = lk[:, 2][np.isfinite(lk[:, 2])]
    cuts = np.unique(np.quantile(finite, [0.1, 0.5, 0.9, 0.99])) if finite.size else np.zeros(0)
    cuts = np.concatenate([cuts, [np.inf]])
    mcs = int(g["min_samples"])
    g["dbscan_cuts"] = cuts.astype(np.float64)
    g["dbscan_min_cluster_size"] = np.int64(mcs)
    g["dbscan_labels"] = np.stack(
        [np.asarray(get_cluster_labelling_at_cut(lk, c, mcs), dtype=np.int64) for c in cuts])
    np.savez_compressed(path, **g)


def _crafted_cluster_tree():
    """A cluster tree (child_size > 1 rows) where segments_in_branch's
    unchecked searchsorted matters: root 10 -> (11, 12), 11 -> (13, 14),
    12 -> (15, 16), 15 -> (17, 18).  From leaf 13 the lookup lands on parent
    15, so 17 and 18 are marked as processed with 11's branch."""
    parent = np.array([10, 10, 11, 11, 12, 12, 15, 15], dtype=np.int64)
    child = np.array([11, 12, 13, 14, 15, 16, 17, 18], dtype=np.int64)
    lam = np.array([0.5, 0.5, 2.0, 2.0, 1.0, 1.0, 4.0, 4.0], dtype=np.float32)
    size = np.array([6, 8, 3, 3, 5, 3, 2, 3], dtype=np.float32)
    return parent, child, lam, size


def function_fixtures():
    """Function-level fixtures: cluster_epsilon_search on a crafted tree."""
    from fast_hdbscan.cluster_trees import CondensedTree, cluster_epsilon_search

    parent, child, lam, size = _crafted_cluster_tree()
    tree = CondensedTree(parent, child, lam, size)
    cases = [([13, 17], 1.5), ([13, 14, 16, 17, 18], 1.5), ([17, 13], 1.5),
             ([13, 17], 0.75), ([16, 17, 18], 3.0)]
    out = {"parent": parent, "child": child, "lambda_val": lam, "child_size": size}
    for i, (sel, eps) in enumerate(cases):
        res = cluster_epsilon_search(np.array(sel, dtype=np.int64), tree, min_epsilon=eps)
        out[f"sel_{i}"] = np.array(sel, dtype=np.int64)
        out[f"eps_{i}"] = np.float64(eps)
        out[f"out_{i}"] = np.asarray(res, dtype=np.int64)
        print(f"eps search {sel} eps={eps} -> {list(out[f'out_{i}'])}")
    np.savez_compressed(os.path.join(HERE, "fn_eps_search.npz"), **out)


KRUSKAL_CASES = {
    # name: (data factory, min_samples, min_cluster_size, knn_k, weights factory or None)
    "kr_blobs200_k10": (lambda: _blobs200(), 5, 10, 10, None),
    "kr_vd3d_5k_k8": (lambda: synthetic.varying_density(5000, seed=11), 10, 40, 8, None),
    "kr_blobs2d_2k_ms1": (lambda: synthetic.blobs_2d(2000, seed=12), 1, 20, 3, None),
    "kr_vd3d_3k_w": (lambda: synthetic.varying_density(3000, seed=13), 6, 30, 12,
                     lambda n: _weights_sixty_fourths(n, 14)),
    # edge cases: knn_k above the point count, and min_samples above knn_k
    "kr_edge_n3": (lambda: np.array([[0.0, 0.0], [1.0, 0.5], [3.0, -1.0]]), 2, 2, 5, None),
    "kr_edge_ms_gt_k": (lambda: _rand(15, 60, 2), 8, 5, 3, None),
}


def kruskal_fixtures(only=None):
    """The kNN-graph Kruskal MST (kruskal.py:950, algorithm='kruskal' with an
    integer knn_k) and the fit on it, from the reference's public API."""
    from fast_hdbscan.hdbscan import compute_minimum_spanning_tree, fast_hdbscan

    for name, (factory, ms, mcs, knn_k, wf) in KRUSKAL_CASES.items():
        if only and name not in only:
            continue
        X = np.ascontiguousarray(factory(), dtype=np.float32)
        w = None if wf is None else wf(X.shape[0])
        t0 = time.time()
        mst, nbrs, core = compute_minimum_spanning_tree(
            X, min_samples=ms, sample_weights=w, algorithm="kruskal", knn_k=knn_k)
        labels, probs = fast_hdbscan(X, min_samples=ms, min_cluster_size=mcs,
                                     sample_weights=w, algorithm="kruskal", knn_k=knn_k)
        out = dict(X=X, min_samples=np.int64(ms), min_cluster_size=np.int64(mcs),
                   knn_k=np.int64(knn_k), mst=np.asarray(mst, np.float64),
                   neighbors=np.asarray(nbrs, np.int32), core=np.asarray(core, np.float64),
                   labels=np.asarray(labels, np.int64), probabilities=np.asarray(probs))
        if w is not None:
            out["sample_weights"] = np.asarray(w, np.float32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(f"{name}: n={X.shape[0]} bridges={int(np.isinf(mst[:, 2]).sum())} "
              f"clusters={len(set(labels.tolist()) - {-1})} {time.time() - t0:.1f}s")


def _knn_graph(X, k, seed):
    """A directed kNN distance graph (float64 CSR, asymmetric), as a user
    would build one for metric="precomputed"."""
    import scipy.sparse
    from scipy.spatial import cKDTree

    X = np.asarray(X, np.float64)
    d, ix = cKDTree(X).query(X, k=k + 1)
    n = X.shape[0]
    rows = np.repeat(np.arange(n), k)
    return scipy.sparse.csr_matrix((d[:, 1:].ravel(), (rows, ix[:, 1:].ravel())), shape=(n, n))


def _blob_graph_disconnected():
    import scipy.sparse

    g1 = _knn_graph(synthetic.blobs_2d(600, seed=41), 6, 0)
    g2 = _knn_graph(synthetic.blobs_2d(400, seed=42) + 100.0, 6, 0)
    return scipy.sparse.block_diag([g1, g2], format="csr")


def _coo_with_duplicates():
    """Duplicate (i, j) entries, both orientations, explicit zeros and a
    diagonal: the min-symmetrisation keeps the least weight per pair."""
    import scipy.sparse

    rng = np.random.default_rng(43)
    n, m = 300, 2400
    rows = rng.integers(0, n, m)
    cols = rng.integers(0, n, m)
    data = rng.random(m) * 10.0
    # explicit zeros on pairs of distinct points: no row holds two equal
    # weights (the reference orders a row with np.argsort's default sort, whose
    # order of equal weights is not specified)
    rows = np.concatenate([rows, np.arange(8)])
    cols = np.concatenate([cols, 100 + np.arange(8)])
    data = np.concatenate([data, np.zeros(8)])
    return scipy.sparse.coo_matrix((data, (rows, cols)), shape=(n, n))


def _sparse_empty(n):
    import scipy.sparse

    return scipy.sparse.csr_matrix((n, n), dtype=np.float64)


def _graph_with_isolated():
    """A 5-NN graph of 40 points plus 5 points with no stored edge."""
    import scipy.sparse

    g = _knn_graph(_rand(16, 40, 2), 5, 0)
    return scipy.sparse.block_diag([g, scipy.sparse.csr_matrix((5, 5))], format="csr")


PRECOMPUTED_CASES = {
    # name: (graph factory, min_samples, min_cluster_size, algorithm)
    "pc_knn3d_kr": (lambda: _knn_graph(synthetic.varying_density(3000, seed=44), 10, 0), 5, 30,
                    "kruskal"),
    "pc_knn3d_bo": (lambda: _knn_graph(synthetic.varying_density(3000, seed=44), 10, 0), 5, 30,
                    "boruvka"),
    "pc_disconnected_kr": (_blob_graph_disconnected, 3, 20, "kruskal"),
    "pc_disconnected_bo": (_blob_graph_disconnected, 3, 20, "boruvka"),
    "pc_coo_dups_kr": (_coo_with_duplicates, 1, 5, "kruskal"),
    # edge cases: no stored edge at all, and isolated points beside a component
    "pc_edge_empty_kr": (lambda: _sparse_empty(6), 2, 2, "kruskal"),
    "pc_edge_isolated_kr": (_graph_with_isolated, 2, 3, "kruskal"),
    "pc_edge_isolated_bo": (_graph_with_isolated, 2, 3, "boruvka"),
}



def precomputed_fixtures(only=None):
    """metric="precomputed" on scipy sparse graphs (precomputed.py:410 Boruvka,
    :479 Kruskal), from the reference's public API."""
    from fast_hdbscan.hdbscan import compute_minimum_spanning_tree, fast_hdbscan

    for name, (factory, ms, mcs, algo) in PRECOMPUTED_CASES.items():
        if only and name not in only:
            continue
        G = factory()
        t0 = time.time()
        mst, nbrs, core = compute_minimum_spanning_tree(G, min_samples=ms, metric="precomputed",
                                                        algorithm=algo)
        labels, probs = fast_hdbscan(G, min_samples=ms, min_cluster_size=mcs,
                                     metric="precomputed", algorithm=algo)
        coo = G.tocoo()
        out = dict(rows=np.asarray(coo.row, np.int32), cols=np.asarray(coo.col, np.int32),
                   data=np.asarray(coo.data, np.float64), n=np.int64(G.shape[0]),
                   min_samples=np.int64(ms), min_cluster_size=np.int64(mcs),
                   algorithm=np.array(algo), mst=np.asarray(mst, np.float64),
                   neighbors=np.asarray(nbrs, np.int32), core=np.asarray(core, np.float64),
                   labels=np.asarray(labels, np.int64), probabilities=np.asarray(probs))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(f"{name}: n={G.shape[0]} nnz={G.nnz} bridges={int(np.isinf(mst[:, 2]).sum())} "
              f"clusters={len(set(labels.tolist()) - {-1})} {time.time() - t0:.1f}s")


def _flares():
    """Three noisy arms from the origin (a Y) and a separate blob, 2-D."""
    rng = np.random.default_rng(0)
    arms = []
    for ang in (0.0, 2.1, 4.2):
        t = rng.uniform(0, 5, 200)
        arms.append(np.c_[t * np.cos(ang), t * np.sin(ang)] + rng.normal(0, 0.15, (200, 2)))
    X = np.concatenate(arms + [rng.normal((12, 0), 0.5, (150, 2))])
    return X[rng.permutation(len(X))].astype(np.float32)


def _flares_nonfinite():
    X = _flares().astype(np.float64)
    X[[3, 77, 400]] = np.nan
    X[500, 1] = np.inf
    return X


def _blobs_lens():
    rng = np.random.default_rng(5)
    X = np.concatenate([rng.normal(c, 1.0, (250, 2)) for c in ((0, 0), (9, 1), (3, 9))])
    return X[rng.permutation(len(X))].astype(np.float32)


# name -> (data factory, HDBSCAN kwargs, detector, detector kwargs)
SUBCLUSTER_CASES = {
    "sc_branches_flares": (_flares, dict(min_cluster_size=30, min_samples=5), "branch",
                           dict(min_cluster_size=15)),
    "sc_branches_flares_leaf": (_flares, dict(min_cluster_size=30, min_samples=5), "branch",
                                dict(min_cluster_size=10, cluster_selection_method="leaf",
                                     label_sides_as_branches=True)),
    "sc_branches_nonfinite": (_flares_nonfinite, dict(min_cluster_size=30, min_samples=5),
                              "branch", dict(min_cluster_size=15)),
    "sc_lens_x_propagate": (_blobs_lens, dict(min_cluster_size=40, min_samples=8), "lens",
                            dict(min_cluster_size=20, propagate_labels=True)),
}


def subcluster_fixtures(only=None):
    """Sub-cluster and branch detection (sub_clusters.py:245, branches.py:70)
    on fits of the reference's own HDBSCAN, plus the core graph of the first
    cluster (core_graph.py:19) for the host-side check."""
    from fast_hdbscan import HDBSCAN, BranchDetector
    from fast_hdbscan.core_graph import knn_mst_union, flatten_to_csr
    from fast_hdbscan.sub_clusters import SubClusterDetector

    for name, (factory, hkw, kind, dkw) in SUBCLUSTER_CASES.items():
        if only and name not in only:
            continue
        X = factory()
        t0 = time.time()
        c = HDBSCAN(**hkw).fit(X)
        if kind == "branch":
            det = BranchDetector(**dkw).fit(c)
            lens = None
        else:
            lens = np.ascontiguousarray(X[:, 0], dtype=np.float64)
            det = SubClusterDetector(lens_values=lens, **dkw).fit(c)
        prop_labels, prop_sub = det.propagated_labels()
        pts = list(det.cluster_points_)
        out = dict(X=X, hdbscan_kwargs=np.array(repr(hkw)), kind=np.array(kind),
                   detector_kwargs=np.array(repr(dkw)),
                   fit_labels=np.asarray(c.labels_, np.int64),
                   labels=np.asarray(det.labels_, np.int64),
                   probabilities=np.asarray(det.probabilities_, np.float64),
                   sub_labels=np.asarray(det.sub_cluster_labels_, np.int64),
                   sub_probabilities=np.asarray(det.sub_cluster_probabilities_, np.float64),
                   lens_out=np.asarray(det.lens_values_, np.float64),
                   points=np.concatenate(pts).astype(np.int64),
                   points_offsets=np.cumsum([0] + [len(p) for p in pts]).astype(np.int64),
                   prop_labels=np.asarray(prop_labels, np.int64),
                   prop_sub_labels=np.asarray(prop_sub, np.int64))
        if lens is not None:
            out["lens"] = lens
        # the first cluster's core graph, from the reference's own inputs
        points = np.nonzero(det.cluster_labels_ == 0)[0]
        if not np.all(np.isfinite(X)):
            out["core_graph_skipped"] = np.array(True)
        else:
            ids = np.full(X.shape[0], -1, np.int32)
            ids[points] = np.arange(len(points))
            nb = ids[c._neighbors[points, :]]
            core = c._core_distances[points]
            mst = c._min_spanning_tree
            keep = (c.labels_[mst[:, 0].astype(np.int64)] == 0) & \
                   (c.labels_[mst[:, 1].astype(np.int64)] == 0)
            mst = mst[keep].copy()
            mst[:, :2] = ids[mst[:, :2].astype(np.int64)]
            lens0 = np.asarray(det.lens_values_, np.float64)[points]
            g = flatten_to_csr(knn_mst_union(nb, core, mst, lens0))
            out.update(cg_neighbors=nb, cg_core=np.asarray(core), cg_mst=mst, cg_lens=lens0,
                       cg_weights=g.weights, cg_distances=g.distances, cg_indices=g.indices,
                       cg_indptr=g.indptr)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(f"{name}: n={len(X)} clusters={len(pts)} labels={len(np.unique(det.labels_))} "
              f"{time.time() - t0:.1f}s")


def _cg_inputs(seed, n, kind):
    """Random core-graph inputs in in-cluster ids: kNN rows without the point
    itself or repeats (as a fit's neighbours), a random spanning tree over
    part of the points, and lens values (float / integer ties / negative)."""
    rng = np.random.default_rng(seed)
    k = 5
    nb = np.argsort(rng.random((n, n)), axis=1)[:, :k + 1]
    nb = np.array([[c for c in row if c != i][:k] for i, row in enumerate(nb)], np.int32)
    drop = {"sparse": 0.6, "disc": 0.93}.get(kind, 0.1)
    nb[rng.random((n, k)) < drop] = -1
    core = rng.random(n).astype(np.float32)
    perm = rng.permutation(n)
    parents = perm[rng.integers(0, np.arange(1, n))]
    mst = np.c_[parents, perm[1:], rng.random(n - 1)].astype(np.float64)
    if kind in ("sparse", "disc"):
        mst = mst[rng.random(n - 1) < (0.3 if kind == "sparse" else 0.05)]
    lens = {"float": rng.random(n), "int": rng.integers(0, 6, n).astype(np.float64),
            "neg": rng.normal(0, 1, n), "sparse": rng.random(n),
            "disc": rng.integers(0, 3, n).astype(np.float64)}[kind]
    return nb, core, mst, lens


CORE_GRAPH_CASES = {"cg_float_400": (1, 400, "float"), "cg_int_400": (2, 400, "int"),
                    "cg_neg_300": (3, 300, "neg"), "cg_sparse_300": (4, 300, "sparse"),
                    "cg_disconnected_300": (5, 300, "disc")}


def core_graph_fixtures(only=None):
    """The reference's core graph (core_graph.py:19, :47) and its Boruvka forest
    (:198) on random inputs, including empty rows and tied weights.

    sort_by_lens (:70) orders each row with np.argsort; under numba that is
    numba's quicksort, an insertion sort (stable) below 16 elements, while
    numpy's own argsort (which the shim falls back to) may order ties
    differently.  Rows here stay below 16 entries and are ordered with a
    stable argsort, as numba orders them."""
    from fast_hdbscan.core_graph import CoreGraph, boruvka_mst, flatten_to_csr, knn_mst_union

    def sort_rows_as_numba(graph):
        w, d, ix = graph.weights.copy(), graph.distances.copy(), graph.indices.copy()
        for p in range(len(graph.indptr) - 1):
            a, b = graph.indptr[p], graph.indptr[p + 1]
            assert b - a < 16, "row too long for numba's insertion-sort range"
            o = np.argsort(graph.weights[a:b], kind="stable")
            w[a:b], d[a:b], ix[a:b] = graph.weights[a:b][o], graph.distances[a:b][o], \
                graph.indices[a:b][o]
        return CoreGraph(w, d, ix, graph.indptr)

    for name, (seed, n, kind) in CORE_GRAPH_CASES.items():
        if only and name not in only:
            continue
        nb, core, mst, lens = _cg_inputs(seed, n, kind)
        g = sort_rows_as_numba(flatten_to_csr(knn_mst_union(nb, core, mst, lens)))
        nc, comp, edges = boruvka_mst(g)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), nb=nb, core=core, mst=mst,
                            lens=lens, weights=g.weights, distances=g.distances,
                            indices=g.indices, indptr=g.indptr, n_components=np.int64(nc),
                            components=np.asarray(comp, np.int64),
                            edges=np.asarray(edges, np.float64))
        print(f"{name}: n={n} nnz={g.indptr[-1]} components={nc} edges={len(edges)}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--cuts-only", action="store_true",
                    help="only add the DBSCAN-cut fields to existing fixtures")
    ap.add_argument("--kruskal-only", action="store_true",
                    help="only write the kNN-graph Kruskal fixtures")
    ap.add_argument("--precomputed-only", action="store_true",
                    help="only write the metric='precomputed' fixtures")
    ap.add_argument("--subclusters-only", action="store_true",
                    help="only write the sub-cluster / branch detection fixtures")
    args = ap.parse_args()
    sys.path.insert(1, args.reference)
    import fast_hdbscan  # noqa: F401
    if args.kruskal_only:
        kruskal_fixtures(args.only)
        return
    if args.precomputed_only:
        precomputed_fixtures(args.only)
        return
    if args.subclusters_only:
        subcluster_fixtures(args.only)
        core_graph_fixtures(args.only)
        return
    for name, (factory, kwargs) in CASES.items():
        if args.only and name not in args.only:
            continue
        if not args.cuts_only:
            run_case(name, factory, kwargs, args.reference)
        add_cuts(name)
    if not args.only:
        function_fixtures()
        kruskal_fixtures()
        precomputed_fixtures()
        subcluster_fixtures()
        core_graph_fixtures()


if __name__ == "__main__":
    main()
