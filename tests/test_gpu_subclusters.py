"""Sub-cluster and branch detection (sub_clusters.py:245, branches.py:70) on
the GPU engine's fits, against the reference's results on the same inputs
(fixtures written by tests/golden/make_golden.py from the reference's own
HDBSCAN, BranchDetector and SubClusterDetector).  The per-cluster core-graph
forests and cluster hierarchies run on the GPU."""
import ast
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = ["sc_branches_flares", "sc_branches_flares_leaf", "sc_branches_nonfinite",
         "sc_lens_x_propagate"]


def _same_partition(a, b):
    """Equal up to a renaming of the labels (noise -1 kept as noise)."""
    a, b = np.asarray(a), np.asarray(b)
    if not np.array_equal(a == -1, b == -1):
        return False
    pairs = set(zip(a.tolist(), b.tolist()))
    return len(pairs) == len(set(a.tolist())) == len(set(b.tolist()))


@pytest.mark.parametrize("name", CASES)
def test_detector_matches_reference(engine, name):
    from fast_hdbscan_gb300 import HDBSCAN, BranchDetector, SubClusterDetector

    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    hkw = ast.literal_eval(str(g["hdbscan_kwargs"]))
    dkw = ast.literal_eval(str(g["detector_kwargs"]))
    c = HDBSCAN(**hkw).fit(g["X"])
    np.testing.assert_array_equal(c.labels_, g["fit_labels"])
    if str(g["kind"]) == "branch":
        det = BranchDetector(**dkw).fit(c)
    else:
        det = SubClusterDetector(lens_values=g["lens"], **dkw).fit(c)
    pts = [g["points"][a:b] for a, b in zip(g["points_offsets"][:-1], g["points_offsets"][1:])]
    assert len(pts) == len(det.cluster_points_)
    for p, q in zip(pts, det.cluster_points_):
        np.testing.assert_array_equal(p, q)
    np.testing.assert_allclose(det.lens_values_, g["lens_out"], rtol=1e-6)
    np.testing.assert_array_equal(det.labels_, g["labels"])
    np.testing.assert_array_equal(det.sub_cluster_labels_, g["sub_labels"])
    np.testing.assert_allclose(det.probabilities_, g["probabilities"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(det.sub_cluster_probabilities_, g["sub_probabilities"],
                               rtol=1e-5, atol=1e-6)
    prop_labels, prop_sub = det.propagated_labels()
    assert _same_partition(prop_labels, g["prop_labels"])


def test_find_branch_sub_clusters_function(engine):
    from fast_hdbscan_gb300 import HDBSCAN, find_branch_sub_clusters

    g = np.load(os.path.join(GOLDEN, "sc_branches_flares.npz"))
    c = HDBSCAN(**ast.literal_eval(str(g["hdbscan_kwargs"]))).fit(g["X"])
    res = find_branch_sub_clusters(c, min_cluster_size=15)
    np.testing.assert_array_equal(res[0], g["labels"])


def test_detector_input_errors(engine):
    from fast_hdbscan_gb300 import HDBSCAN, BranchDetector

    g = np.load(os.path.join(GOLDEN, "sc_branches_flares.npz"))
    c = HDBSCAN(min_cluster_size=30, min_samples=5).fit(g["X"])
    with pytest.raises(ValueError):
        BranchDetector(min_cluster_size=1).fit(c)
    with pytest.raises(ValueError):
        BranchDetector(cluster_selection_method="other").fit(c)
    with pytest.raises(ValueError):
        BranchDetector().fit(c, labels=np.full(len(g["X"]), -1))


def _random_core_graph_inputs(seed, n, lens_kind):
    rng = np.random.default_rng(seed)
    k = 5
    nb = rng.integers(0, n, size=(n, k)).astype(np.int32)
    nb[rng.random((n, k)) < (0.6 if lens_kind == "sparse" else 0.1)] = -1
    core = rng.random(n).astype(np.float32)
    perm = rng.permutation(n)
    parents = perm[rng.integers(0, np.arange(1, n))]  # a random tree over perm
    mst = np.c_[parents, perm[1:], rng.random(n - 1)].astype(np.float64)
    if lens_kind == "sparse":
        mst = mst[rng.random(n - 1) < 0.3]
    lens = {"float": rng.random(n), "int": rng.integers(0, 6, n).astype(np.float64),
            "neg": rng.normal(0, 1, n), "sparse": rng.random(n)}[lens_kind]
    return nb, core, mst, lens


@pytest.mark.parametrize("seed,kind", [(0, "float"), (1, "int"), (2, "neg"), (3, "sparse")])
def test_core_graph_forest_matches_oracle(engine, seed, kind):
    """The GPU forest equals the restated reference Boruvka edge for edge,
    including its choices among equal weights (integer lens: heavy ties) and
    a disconnected graph."""
    from fast_hdbscan_gb300.core_graph import core_graph_spanning_tree
    from oracle import core_graph_boruvka as CB

    nb, core, mst, lens = _random_core_graph_inputs(seed, 3000, kind)
    nc, comp, forest, graph = core_graph_spanning_tree(nb, core, mst, lens)
    nc_o, comp_o, edges_o = CB.boruvka_mst(graph.weights, graph.indices, graph.indptr)
    assert nc == nc_o
    np.testing.assert_array_equal(forest, edges_o)
    if nc > 1:
        _, ref_labels = np.unique(comp_o, return_inverse=True)
        np.testing.assert_array_equal(comp, ref_labels)


def test_batched_forests_equal_single(engine):
    """Several clusters' graphs in one launch (disjoint blocks, empty rows at
    block ends included) give each graph's own forest."""
    from fast_hdbscan_gb300.core_graph import (core_graph_forests, core_graph_spanning_tree,
                                               knn_mst_union)

    graphs, singles = [], []
    for seed, kind, n in [(5, "float", 700), (6, "sparse", 500), (7, "int", 900), (8, "sparse", 40)]:
        nb, core, mst, lens = _random_core_graph_inputs(seed, n, kind)
        nb[-3:] = -1  # the block's last rows: no kNN children ...
        mst = mst[~np.isin(mst[:, 0], [n - 1, n - 2, n - 3])]  # ... and no MST children
        graphs.append(knn_mst_union(nb, core, mst, lens))
        singles.append(core_graph_spanning_tree(nb, core, mst, lens))
    for (nc, comp, forest), (nc1, comp1, forest1, _) in zip(core_graph_forests(graphs), singles):
        assert nc == nc1
        np.testing.assert_array_equal(forest, forest1)
        np.testing.assert_array_equal(comp, comp1)


def test_gpu_core_graph_layout_equals_host(engine):
    """The block-CSR layout on the GPU (fhg_core_graphs) equals the host
    knn_mst_union row for row (duplicates, self entries, empty rows, tied
    weights), and its forests equal the single forests."""
    from fast_hdbscan_gb300.core_graph import (core_graph_spanning_tree,
                                               core_graphs_and_forests, knn_mst_union)

    inputs = []
    for seed, kind, n in [(9, "float", 800), (10, "int", 600), (11, "sparse", 300),
                          (12, "neg", 1), (13, "int", 2)]:
        nb, core, mst, lens = _random_core_graph_inputs(seed, max(n, 3), kind)
        nb, core, lens = nb[:n], core[:n], lens[:n]
        nb = np.where(nb < n, nb, -1).astype(np.int32)
        mst = mst[(mst[:, 0] < n) & (mst[:, 1] < n)]
        if n > 3:
            nb[-2:] = -1
            mst = mst[~np.isin(mst[:, 0], [n - 1, n - 2])]
        inputs.append((nb, core, mst, lens))
    built = core_graphs_and_forests(inputs)
    for (nb, core, mst, lens), (g, nc, comp, forest) in zip(inputs, built):
        h = knn_mst_union(nb, core, mst, lens)
        np.testing.assert_array_equal(g.indptr, h.indptr)
        np.testing.assert_array_equal(g.indices, h.indices)
        np.testing.assert_array_equal(g.weights, h.weights)
        np.testing.assert_array_equal(g.distances, h.distances)
        nc1, comp1, forest1, _ = core_graph_spanning_tree(nb, core, mst, lens)
        assert nc == nc1
        np.testing.assert_array_equal(forest, forest1)
        np.testing.assert_array_equal(comp, comp1)


@pytest.mark.parametrize("name", ["cg_float_400", "cg_int_400", "cg_neg_300", "cg_sparse_300",
                                  "cg_disconnected_300"])
def test_gpu_forest_matches_reference_fixture(engine, name):
    """The GPU core graph and forest against the reference's (core_graph.py:198)."""
    from fast_hdbscan_gb300.core_graph import core_graph_spanning_tree, core_graphs_and_forests

    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    nc, comp, forest, graph = core_graph_spanning_tree(g["nb"], g["core"], g["mst"], g["lens"])
    assert nc == int(g["n_components"])
    np.testing.assert_array_equal(forest, g["edges"])
    np.testing.assert_array_equal(comp, np.unique(g["components"], return_inverse=True)[1])
    (g2, nc2, comp2, forest2), = core_graphs_and_forests([(g["nb"], g["core"], g["mst"],
                                                           g["lens"])])
    np.testing.assert_array_equal(g2.indices, g["indices"])
    np.testing.assert_array_equal(g2.weights, g["weights"])
    np.testing.assert_array_equal(forest2, g["edges"])


def _reference_sweeps(graph, sub_labels):
    """sub_clusters.py:145-166 restated as the checker: in-place sweeps over the
    noise points in index order, until none is labelled (the reference would
    loop forever on unreachable noise)."""
    import sys

    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_cpu_subclusters import reference_noise_dicts

    lab = np.array(sub_labels).copy()
    und = reference_noise_dicts(graph, lab)
    while True:
        changed = False
        for idx in np.nonzero(lab == -1)[0]:
            cand = {}
            for nb, w in und[idx].items():
                if lab[nb] == -1:
                    continue
                cand[lab[nb]] = cand.get(lab[nb], 0.0) + w
            if not cand:
                continue
            best, bl = -np.inf, -1
            for c, w in cand.items():
                if w > best:
                    best, bl = w, c
            lab[idx] = bl
            changed = True
        if not changed:
            return lab


def _graph(rows, ws):
    from fast_hdbscan_gb300.core_graph import CoreGraph

    indptr = np.cumsum([0] + [len(r) for r in rows]).astype(np.int32)
    return CoreGraph(np.array(sum(ws, []), np.float32), np.zeros(indptr[-1], np.float32),
                     np.array(sum(rows, []), np.int32), indptr)


def test_gpu_label_propagation_small_graph(engine):
    """0 - 1 (w 1), 1 - 2 (w 4), 2 - 3 (w 1), 3 - 4 (w 2); 5 isolated: 1 takes 0's
    label; 2 then weighs 1 (label 0, 1/4) against 3 (label 1, 1/1); 4 follows
    3; 5 stays noise."""
    from fast_hdbscan_gb300.sub_clusters import propagate_sub_cluster_labels

    g = _graph([[1], [2], [3], [4], [], []], [[1.0], [4.0], [1.0], [2.0], [], []])
    sub = np.array([0, -1, -1, 1, -1, -1], dtype=np.int64)
    labels = np.zeros(6, dtype=np.int64)
    propagate_sub_cluster_labels(labels, sub, [g], [np.arange(6)])
    assert sub.tolist() == [0, 0, 1, 1, 1, -1]


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_gpu_label_propagation_matches_sweeps(engine, seed):
    """Several clusters in one launch: every cluster's result equals the
    reference's sequential sweeps; labels are renumbered cluster after
    cluster."""
    from fast_hdbscan_gb300.sub_clusters import propagate_sub_cluster_labels

    rng = np.random.default_rng(seed)
    graphs, subs, pts, at = [], [], [], 0
    for c in range(5):
        n = int(rng.integers(20, 120))
        rows = [sorted(rng.choice(n, rng.integers(0, 5), replace=False).tolist())
                for _ in range(n)]
        ws = [rng.uniform(0.5, 3.0, len(r)).astype(np.float32).tolist() for r in rows]
        graphs.append(_graph(rows, ws))
        subs.append(rng.integers(-1, 3 if c != 2 else 1, n))  # cluster 2: noise + one label
        pts.append(np.arange(at, at + n))
        at += n
    sub = np.concatenate(subs).astype(np.int64)
    want = [_reference_sweeps(g, s) for g, s in zip(graphs, subs)]
    labels = np.zeros(at, dtype=np.int64)
    propagate_sub_cluster_labels(labels, sub, graphs, pts)
    for p, w in zip(pts, want):
        np.testing.assert_array_equal(sub[p], w)
