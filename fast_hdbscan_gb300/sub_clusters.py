"""Sub-cluster detection within fitted clusters (the reference's
sub_clusters.py): every cluster's points get lens values (a callback or an
array), their core graph is clustered on the lens (core_graph.py: the
spanning forests and the cluster hierarchies on the GPU), and the
per-cluster results are merged into one labelling.

All clusters are handled together: one layout pass cuts every cluster's
inputs out of the fit (cluster_layout), one GPU pass builds every core graph
and forest, the label merge is a few vectorised passes over (cluster, label)
pairs, and the optional propagation of labels to noise points runs on the
GPU for every cluster in one launch.  The validation, the returned tuple and
the fitted attributes are the reference's interface."""
import concurrent.futures
import os
import threading

import numpy as np

from . import _native
from .core_graph import _clusters_of_forest, core_graph_to_edge_list, core_graphs_and_forests_block
from .hdbscan import _BaseEstimator as BaseEstimator
from .hdbscan import _check_sample_weight, to_numpy_rec_array
from .hdbscan import _ClusterMixin as ClusterMixin

try:  # scikit-learn is optional, as for the estimator
    from sklearn.exceptions import NotFittedError
except ImportError:  # pragma: no cover - exercised where sklearn is absent
    class NotFittedError(ValueError, AttributeError):
        pass


def check_is_fitted(estimator, attributes, msg):
    """sklearn.utils.validation.check_is_fitted for one attribute name."""
    if not hasattr(estimator, attributes):
        raise NotFittedError(msg)


def cluster_layout(labels, num_clusters, neighbors, min_spanning_tree, device=None):
    """Every cluster's inputs in one pass, clusters back to back.

    Returns (points, bounds, nb_local, mst_local, mst_bounds): the clustered
    points grouped by cluster (cluster c at points[bounds[c]:bounds[c+1]], in
    increasing index order), their kNN neighbours as in-cluster ids (-1 for
    neighbours outside the cluster), and the MST edges with both ends in one
    cluster, grouped by cluster in their original order with in-cluster ids
    (cluster c's at mst_local[mst_bounds[c]:mst_bounds[c+1]]) -- the arrays
    sub_clusters.py:16-61 cuts out for each cluster.  The passes (a stable
    sort of the labels, the gathers) run as torch operations on ``device``
    (the GPU when there is one); the results come back as NumPy arrays."""
    import torch

    if device is None:
        device = "cuda" if torch.cuda.is_available() else "cpu"
    lab = torch.as_tensor(np.ascontiguousarray(labels, dtype=np.int64), device=device)
    n = lab.numel()
    order = torch.sort(lab, stable=True).indices
    marks = torch.arange(num_clusters + 1, dtype=torch.int64, device=device)
    bounds = torch.searchsorted(lab[order].contiguous(), marks)
    points = order[bounds[0]:]
    bounds = bounds - bounds[0]
    sizes = bounds[1:] - bounds[:-1]
    owner = torch.repeat_interleave(marks[:-1], sizes)
    local = torch.full((n,), -1, dtype=torch.int64, device=device)
    local[points] = (torch.arange(points.numel(), dtype=torch.int64, device=device)
                     - torch.repeat_interleave(bounds[:-1], sizes))
    nb = torch.as_tensor(np.ascontiguousarray(neighbors), device=device)[points].long()
    nb_c = nb.clamp(min=0)
    inside = (nb >= 0) & (lab[nb_c] == owner[:, None])
    nb_local = torch.where(inside, local[nb_c], torch.full_like(nb_c, -1)).to(torch.int32)
    mst = torch.as_tensor(np.ascontiguousarray(min_spanning_tree, dtype=np.float64),
                          device=device).reshape(-1, 3)
    pe = lab[mst[:, 0].long()]
    ce = lab[mst[:, 1].long()]
    kept = torch.nonzero((pe == ce) & (pe >= 0)).flatten()
    kept = kept[torch.sort(pe[kept], stable=True).indices]
    mst_bounds = torch.searchsorted(pe[kept].contiguous(), marks)
    mst_local = mst[kept].clone()
    mst_local[:, :2] = local[mst_local[:, :2].long()].double()
    return (points.cpu().numpy(), bounds.cpu().numpy(), nb_local.cpu().numpy(),
            mst_local.cpu().numpy(), mst_bounds.cpu().numpy())


def cluster_lens_values(lens, data, probabilities, points, bounds, nb_local, core, mst_local,
                        mst_bounds):
    """Lens values of every clustered point (clusters back to back): from an
    array over the points, from a callback's all-clusters form in one call,
    or from a per-cluster callback (sub_clusters.py:45) given each cluster's
    slices."""
    if isinstance(lens, np.ndarray):
        return np.asarray(lens)[points]
    all_clusters = getattr(lens, "all_clusters", None)
    if all_clusters is not None:
        return np.asarray(all_clusters(data, probabilities, points, bounds))
    parts = [np.asarray(lens(data, probabilities, nb_local[bounds[c]:bounds[c + 1]],
                             core[bounds[c]:bounds[c + 1]],
                             mst_local[mst_bounds[c]:mst_bounds[c + 1]],
                             points[bounds[c]:bounds[c + 1]]))
             for c in range(len(bounds) - 1)]
    return np.concatenate(parts + [np.zeros(0)])


def compute_sub_clusters_per_cluster(data, labels, probabilities, neighbors, core_distances,
                                     min_spanning_tree, lens_callback, num_clusters,
                                     sample_weights=None, **kwargs):
    """sub_clusters.py:64: every cluster's sub-cluster hierarchy on its lens.
    The clusters' inputs come from one layout pass (cluster_layout), their
    core graphs and spanning forests from one GPU pass each, and their
    hierarchies -- independent, a few short launches each -- run on worker
    threads with a CUDA stream apiece.  Returns, per cluster, (labels,
    probabilities, linkage tree, condensed tree, forest, core graph, lens
    values, points)."""
    points, bounds, nb_local, mst_local, mst_bounds = cluster_layout(
        labels, num_clusters, neighbors, min_spanning_tree)
    core = np.asarray(core_distances)[points]
    lens = cluster_lens_values(lens_callback, data, probabilities, points, bounds, nb_local,
                               core, mst_local, mst_bounds)
    built = core_graphs_and_forests_block(np.diff(bounds), nb_local, lens, core, mst_local,
                                          mst_bounds)

    torch = _native._torch()
    tls = threading.local()

    def hierarchy(c):
        graph, nc, comp, forest = built[c]
        pts = points[bounds[c]:bounds[c + 1]]
        if not hasattr(tls, "stream"):
            tls.stream = torch.cuda.Stream()
        with torch.cuda.stream(tls.stream):
            res = _clusters_of_forest(
                nc, comp, forest, graph,
                sample_weights=(sample_weights[pts] if sample_weights is not None else None),
                **kwargs)
        tls.stream.synchronize()
        return (*res, lens[bounds[c]:bounds[c + 1]], pts)

    torch.cuda.current_stream().synchronize()
    if num_clusters <= 1:
        return [hierarchy(c) for c in range(num_clusters)]
    workers = min(16, os.cpu_count() or 8, num_clusters)
    with concurrent.futures.ThreadPoolExecutor(workers) as ex:
        return list(ex.map(hierarchy, range(num_clusters)))


def _label_counts(sub_labels, points_list):
    """Per cluster: the number of distinct sub-labels and whether -1 is one of
    them, from one np.unique over (cluster, label) pairs.  Also returns the
    clusters' points back to back, each point's cluster and its sub-label."""
    n_cl = len(points_list)
    sizes = np.array([len(p) for p in points_list], dtype=np.int64)
    pts = (np.concatenate([np.asarray(p, dtype=np.int64) for p in points_list])
           if n_cl else np.zeros(0, np.int64))
    owner = np.repeat(np.arange(n_cl), sizes)
    lab = np.asarray(sub_labels)[pts].astype(np.int64)
    span = int(lab.max()) + 2 if lab.size else 1
    pairs = np.unique(owner * span + (lab + 1))
    distinct = np.bincount(pairs // span, minlength=n_cl)
    noise = np.zeros(n_cl, dtype=np.int64)
    noise[(pairs // span)[pairs % span == 0]] = 1
    return distinct, noise, pts, owner, lab


def update_labels(cluster_probabilities, sub_labels_list, sub_probabilities_list,
                  lens_values_list, points_list, data_size):
    """sub_clusters.py:98: one labelling from the per-cluster results.  Labels
    are numbered cluster after cluster, every distinct sub-label (noise
    included) taking one number and noise sharing the cluster's first;
    probabilities are the mean of the cluster and sub-cluster probabilities
    (float32: their sum, halved)."""
    labels = np.full(data_size, -1, dtype=np.int64)
    probabilities = cluster_probabilities.copy()
    sub_labels = np.zeros(data_size, dtype=np.int64)
    sub_probabilities = np.zeros(data_size, dtype=np.float32)
    lens_values = np.zeros(data_size, dtype=np.float32)
    if len(points_list) == 0:
        return labels, probabilities, sub_labels, sub_probabilities, lens_values
    sub_labels[np.concatenate(points_list)] = np.concatenate(sub_labels_list)
    distinct, noise, pts, owner, lab = _label_counts(sub_labels, points_list)
    first = np.concatenate([[0], np.cumsum(distinct)[:-1]])
    labels[pts] = lab + noise[owner] + first[owner]
    sub_probabilities[pts] = np.concatenate(sub_probabilities_list)
    merged = probabilities[pts]
    merged += sub_probabilities[pts]
    merged /= 2
    probabilities[pts] = merged
    lens_values[pts] = np.concatenate(lens_values_list)
    return labels, probabilities, sub_labels, sub_probabilities, lens_values


def _noise_adjacency(graph, sub_labels, base):
    """The neighbours of every noise point of one cluster's core graph, in the
    order the reference's per-point dict (sub_clusters.py:134-142) holds
    them: walking the CSR in row order, an entry (row -> col) first adds row
    to col's dict if col is noise, then col to row's if row is noise; a
    repeated pair keeps its first position and its last value.  Point ids
    are offset by ``base``.  Returns (noise points ascending, their entry
    counts, neighbours, inverse weights)."""
    indptr = np.asarray(graph.indptr, dtype=np.int64)
    n = len(indptr) - 1
    rows = np.repeat(np.arange(n), np.diff(indptr))
    cols = np.asarray(graph.indices, dtype=np.int64)
    inv = 1.0 / np.asarray(graph.weights, dtype=np.float64)
    noise = np.asarray(sub_labels) == -1
    key = np.stack([cols, rows], axis=1).ravel()
    other = np.stack([rows, cols], axis=1).ravel()
    val = np.repeat(inv, 2)
    ok = np.stack([noise[cols], noise[rows]], axis=1).ravel()
    seq = np.nonzero(ok)[0]
    key, other, val = key[seq], other[seq], val[seq]
    pair = key * n + other
    o = np.lexsort((seq, pair))
    head = np.r_[True, pair[o][1:] != pair[o][:-1]]
    tail = np.r_[head[1:], True]
    first_seq = seq[o][head]
    last_val = val[o][tail]
    ukey, uother = key[o][head], other[o][head]
    o2 = np.lexsort((first_seq, ukey))
    noise_pts = np.nonzero(noise)[0]
    counts = np.bincount(ukey[o2], minlength=n)[noise_pts]
    return noise_pts + base, counts, uother[o2] + base, last_val[o2]


def propagate_sub_cluster_labels(labels, sub_labels, graph_list, points_list):
    """sub_clusters.py:170: in every cluster that has both noise and
    sub-clusters, noise points take labels by density-weighted majority votes
    over the core graph, on the GPU for all such clusters in one launch
    (``fhg_propagate_labels``, the reference's in-place sweeps,
    sub_clusters.py:132); then labels are numbered cluster after cluster.
    Noise that no labelled point can reach stays noise (the reference loops
    forever there).  Updates and returns (labels, sub_labels)."""
    if len(points_list) == 0:
        return labels, sub_labels
    distinct, noise, pts, owner, _ = _label_counts(sub_labels, points_list)
    needs = np.nonzero((noise == 1) & (distinct > 1))[0]
    if len(needs):
        torch = _native._torch()
        lab_parts, npt, cnt, adj_o, adj_w, nfirst = [], [], [], [], [], [0]
        base = 0
        for c in needs:
            p = np.asarray(points_list[c], dtype=np.int64)
            sl = np.asarray(sub_labels)[p]
            a, b, o, w = _noise_adjacency(graph_list[c], sl, base)
            lab_parts.append(sl)
            npt.append(a)
            cnt.append(b)
            adj_o.append(o)
            adj_w.append(w)
            nfirst.append(nfirst[-1] + len(a))
            base += len(p)
        T = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).cuda()  # noqa
        d_lab = T(np.concatenate(lab_parts), np.int32)
        counts = np.concatenate(cnt)
        d_first = T(nfirst, np.int32)
        d_pts = T(np.concatenate(npt), np.int32)
        d_ptr = T(np.concatenate([[0], np.cumsum(counts)]), np.int32)
        d_oth = T(np.concatenate(adj_o + [np.zeros(0, np.int64)]), np.int32)
        d_w = T(np.concatenate(adj_w + [np.zeros(0)]), np.float64)
        V = _native.vptr
        _native.check(_native.load().fhg_propagate_labels(
            len(needs), V(d_first), V(d_pts), V(d_ptr), V(d_oth), V(d_w), V(d_lab),
            _native.stream_ptr()))
        new = d_lab.cpu().numpy().astype(np.asarray(sub_labels).dtype)
        at = 0
        for c in needs:
            p = np.asarray(points_list[c], dtype=np.int64)
            sub_labels[p] = new[at:at + len(p)]
            at += len(p)
    widths = distinct - ((noise == 1) & (distinct > 1))
    first = np.concatenate([[0], np.cumsum(widths)[:-1]])
    labels[pts] = np.asarray(sub_labels)[pts] + first[owner]
    return labels, sub_labels


def remap_results(labels, probabilities, cluster_labels, cluster_probabilities, sub_labels,
                  sub_probabilities, lens_values, points, finite_index, num_points):
    """sub_clusters.py:188: back to the caller's rows when non-finite rows were
    dropped before the fit."""
    def widen(a, fill):
        out = np.full(num_points, fill, dtype=a.dtype)
        out[finite_index] = a
        return out

    labels = widen(labels, -1)
    probabilities = widen(probabilities, 0.0)
    cluster_labels = widen(cluster_labels, -1)
    cluster_probabilities = widen(cluster_probabilities, 0.0)
    sub_labels = widen(sub_labels, 0)
    sub_probabilities = widen(sub_probabilities, 1.0)
    lens_values = widen(lens_values, 0.0)
    for pts in points:
        pts[:] = finite_index[pts]
    return (labels, probabilities, cluster_labels, cluster_probabilities, sub_labels,
            sub_probabilities, lens_values, points)


def find_sub_clusters(clusterer, cluster_labels=None, cluster_probabilities=None,
                      sample_weights=None, lens_callback=None, *, min_cluster_size=None,
                      max_cluster_size=None, allow_single_cluster=None,
                      cluster_selection_method=None, cluster_selection_epsilon=0.0,
                      cluster_selection_persistence=0.0, propagate_labels=False):
    """sub_clusters.py:245, with the same validation and return tuple."""
    if getattr(clusterer, "metric", "euclidean") == "precomputed":
        raise NotImplementedError(
            "SubClusterDetector and BranchDetector are not supported for models fitted with "
            "metric='precomputed'. These detectors require raw feature vectors to compute "
            "lens values.")
    if getattr(clusterer, "_raw_data", None) is None:
        raise ValueError(
            "SubClusterDetector and BranchDetector require the clusterer to have stored "
            "_raw_data during fit. Ensure the model was fitted with raw feature vectors.")
    check_is_fitted(clusterer, "_min_spanning_tree",
                    msg="You first need to fit the HDBSCAN model before detecting sub clusters.")
    if cluster_labels is None:
        cluster_labels = clusterer.labels_
    elif cluster_probabilities is None:
        cluster_probabilities = np.ones(cluster_labels.shape[0], dtype=np.float32)
    if cluster_probabilities is None:
        cluster_probabilities = clusterer.probabilities_
    if sample_weights is not None:
        sample_weights = _check_sample_weight(sample_weights, clusterer._raw_data,
                                              dtype=np.float32)
    if min_cluster_size is None:
        min_cluster_size = clusterer.min_cluster_size
    if max_cluster_size is None:
        max_cluster_size = clusterer.max_cluster_size
    if allow_single_cluster is None:
        allow_single_cluster = clusterer.allow_single_cluster
    if cluster_selection_method is None:
        cluster_selection_method = clusterer.cluster_selection_method
    if not (np.issubdtype(type(min_cluster_size), np.integer) and min_cluster_size >= 2):
        raise ValueError(f"min_cluster_size must be an integer greater or equal "
                         f"to 2,  {min_cluster_size} given.")
    if max_cluster_size <= 0:
        raise ValueError(f"max_cluster_size must be greater 0, {max_cluster_size} given.")
    if not (np.issubdtype(type(cluster_selection_persistence), np.floating)
            and cluster_selection_persistence >= 0.0):
        raise ValueError(f"cluster_selection_persistence must be a float greater or equal to "
                         f"0.0, {cluster_selection_persistence} given.")
    if not (np.issubdtype(type(cluster_selection_epsilon), np.floating)
            and cluster_selection_epsilon >= 0.0):
        raise ValueError(f"cluster_selection_epsilon must be a float greater or equal to "
                         f"0.0, {cluster_selection_epsilon} given.")
    if cluster_selection_method not in ("eom", "leaf"):
        raise ValueError(f"Invalid cluster_selection_method: {cluster_selection_method}\n"
                         f'Should be one of: "eom", "leaf"\n')
    if np.all(cluster_labels == -1):
        raise ValueError("Input contains only noise points.")

    # the rows the fit kept (non-finite rows are the condensed tree's lambda-0 children)
    data = clusterer._raw_data
    num_points = data.shape[0]
    last_outlier = np.searchsorted(clusterer._condensed_tree["lambda_val"], 0.0, side="right")
    if last_outlier > 0:
        finite_index = np.setdiff1d(np.arange(data.shape[0]),
                                    clusterer._condensed_tree["child"][:last_outlier])
        data = data[finite_index]
        cluster_labels = cluster_labels[finite_index]
        cluster_probabilities = cluster_probabilities[finite_index]
        sample_weights = sample_weights[finite_index] if sample_weights is not None else None

    if isinstance(lens_callback, np.ndarray):
        if len(lens_callback) != num_points:
            raise ValueError(
                "when providing values as lens_callback, they must have"
                f"the same length as the data, {len(lens_callback)} != {data.shape[0]}")
        lens_callback = np.asarray(lens_callback[finite_index] if last_outlier > 0
                                   else lens_callback)

    num_clusters = np.max(cluster_labels) + 1
    (sub_labels, sub_probabilities, linkage_trees, condensed_trees, spanning_trees,
     core_graphs, lens_values, points) = zip(*compute_sub_clusters_per_cluster(
         data, cluster_labels, cluster_probabilities, clusterer._neighbors,
         clusterer._core_distances, clusterer._min_spanning_tree, lens_callback, num_clusters,
         min_cluster_size=min_cluster_size, max_cluster_size=max_cluster_size,
         allow_single_cluster=allow_single_cluster,
         cluster_selection_method=cluster_selection_method,
         cluster_selection_epsilon=cluster_selection_epsilon,
         cluster_selection_persistence=cluster_selection_persistence,
         sample_weights=sample_weights))

    condensed_trees = [to_numpy_rec_array(tree) if tree.parent.shape[0] > 0 else None
                       for tree in condensed_trees]
    linkage_trees = [tree if tree.shape[0] > 0 else None for tree in linkage_trees]
    labels, probabilities, sub_labels, sub_probabilities, lens_values = update_labels(
        cluster_probabilities, sub_labels, sub_probabilities, lens_values, points,
        data.shape[0])
    if propagate_labels:
        labels, sub_labels = propagate_sub_cluster_labels(labels, sub_labels, core_graphs,
                                                          points)
    if last_outlier > 0:
        (labels, probabilities, cluster_labels, cluster_probabilities, sub_labels,
         sub_probabilities, lens_values, points) = remap_results(
             labels, probabilities, cluster_labels, cluster_probabilities, sub_labels,
             sub_probabilities, lens_values, points, finite_index, clusterer._raw_data.shape[0])
    return (labels, probabilities, cluster_labels, cluster_probabilities, sub_labels,
            sub_probabilities, core_graphs, condensed_trees, linkage_trees, spanning_trees,
            lens_values, points)


class SubClusterDetector(ClusterMixin, BaseEstimator):
    """sub_clusters.py:458: lens-value sub-cluster detection on a fitted
    HDBSCAN clusterer."""

    def __init__(self, *, lens_values=None, min_cluster_size=None, max_cluster_size=None,
                 allow_single_cluster=False, cluster_selection_method="eom",
                 cluster_selection_epsilon=0.0, cluster_selection_persistence=0.0,
                 propagate_labels=False):
        self.lens_values = lens_values
        self.min_cluster_size = min_cluster_size
        self.max_cluster_size = max_cluster_size
        self.allow_single_cluster = allow_single_cluster
        self.cluster_selection_method = cluster_selection_method
        self.cluster_selection_epsilon = cluster_selection_epsilon
        self.cluster_selection_persistence = cluster_selection_persistence
        self.propagate_labels = propagate_labels

    def fit(self, clusterer, labels=None, probabilities=None, sample_weight=None,
            lens_callback=None):
        """labels and probabilities override the clusterer's values."""
        (self.labels_, self.probabilities_, self.cluster_labels_, self.cluster_probabilities_,
         self.sub_cluster_labels_, self.sub_cluster_probabilities_, self._approximation_graphs,
         self._condensed_trees, self._linkage_trees, self._spanning_trees, self.lens_values_,
         self.cluster_points_) = find_sub_clusters(
             clusterer, labels, probabilities, sample_weight,
             self.lens_values if lens_callback is None else lens_callback,
             min_cluster_size=self.min_cluster_size, max_cluster_size=self.max_cluster_size,
             allow_single_cluster=self.allow_single_cluster,
             cluster_selection_method=self.cluster_selection_method,
             cluster_selection_epsilon=self.cluster_selection_epsilon,
             cluster_selection_persistence=self.cluster_selection_persistence,
             propagate_labels=self.propagate_labels)
        self._raw_data = clusterer._raw_data
        self._core_distances = clusterer._core_distances
        return self

    def propagated_labels(self):
        """Sub-cluster labels propagated to noise points."""
        check_is_fitted(self, "labels_", msg="You first need to fit the SubClusterDetector "
                                             "model before propagating the labels.")
        return propagate_sub_cluster_labels(self.labels_.copy(), self.sub_cluster_labels_.copy(),
                                            self._approximation_graphs, self.cluster_points_)

    @property
    def approximation_graph_(self):
        return self._make_approximation_graph()

    def _make_approximation_graph(self, lens_name=None, sub_cluster_name=None):
        from hdbscan.plots import ApproximationGraph  # the reference's optional dependency

        check_is_fitted(self, "_approximation_graphs", msg="You first need to fit the "
                        "BranchDetector model before accessing the approximation graphs")
        edge_lists = []
        for graph, points in zip(self._approximation_graphs, self.cluster_points_):
            edges = core_graph_to_edge_list(graph)
            edges[:, 0] = points[edges[:, 0].astype(np.int64)]
            edges[:, 1] = points[edges[:, 1].astype(np.int64)]
            edge_lists.append(edges)
        return ApproximationGraph(edge_lists, self.labels_, self.probabilities_,
                                  self.lens_values_, self.cluster_labels_,
                                  self.cluster_probabilities_, self.sub_cluster_labels_,
                                  self.sub_cluster_probabilities_, lens_name=lens_name,
                                  sub_cluster_name=sub_cluster_name, raw_data=self._raw_data)

    @property
    def condensed_trees_(self):
        from hdbscan.plots import CondensedTree

        check_is_fitted(self, "_condensed_trees", msg="You first need to fit the "
                        "BranchDetector model before accessing the condensed trees")
        return [CondensedTree(tree, self.sub_cluster_labels_[points]) if tree is not None
                else None for tree, points in zip(self._condensed_trees, self.cluster_points_)]

    @property
    def linkage_trees_(self):
        from hdbscan.plots import SingleLinkageTree

        check_is_fitted(self, "_linkage_trees", msg="You first need to fit the "
                        "BranchDetector model before accessing the linkage trees")
        return [SingleLinkageTree(tree) if tree is not None else None
                for tree in self._linkage_trees]

    @property
    def spanning_trees_(self):
        from hdbscan.plots import MinimumSpanningTree

        check_is_fitted(self, "_spanning_trees", msg="You first need to fit the "
                        "BranchDetector model before accessing the linkage trees")
        return [MinimumSpanningTree(tree, self._raw_data) for tree in self._spanning_trees]
