"""Sub-cluster detection within fitted clusters (sub_clusters.py of the
reference): every cluster's points get lens values (a callback or an array),
their core graph is clustered on the lens (core_graph.py, the spanning forest
and cluster hierarchy on the GPU), and the per-cluster results are merged
into one labelling.  The host side -- the per-cluster loop, label merging,
noise propagation and non-finite remapping -- follows the reference step for
step."""
import concurrent.futures
import threading

import numpy as np

from . import _native
from .core_graph import (_clusters_of_forest, core_graph_clusters, core_graph_to_edge_list,
                         core_graphs_and_forests)
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


def compute_sub_clusters_in_cluster(cluster, data, labels, probabilities, neighbors,
                                    core_distances, min_spanning_tree, parent_labels,
                                    child_labels, lens_callback, sample_weights=None,
                                    **kwargs):
    """sub_clusters.py:16: one cluster's sub-clusters, in in-cluster ids."""
    points = np.nonzero(labels == cluster)[0]
    in_cluster_ids = np.full(data.shape[0], -1, dtype=np.int32)
    in_cluster_ids[points] = np.arange(len(points))
    neighbors = in_cluster_ids[neighbors[points, :]]
    core_distances = core_distances[points]
    min_spanning_tree = min_spanning_tree[(parent_labels == cluster) & (child_labels == cluster)]
    min_spanning_tree[:, :2] = in_cluster_ids[min_spanning_tree[:, :2].astype(np.int64)]
    lens_values = lens_callback(data, probabilities, neighbors, core_distances,
                                min_spanning_tree, points)
    return (*core_graph_clusters(
        lens_values, neighbors, core_distances, min_spanning_tree,
        sample_weights=(sample_weights[points] if sample_weights is not None else None),
        **kwargs), lens_values, points)


def compute_sub_clusters_per_cluster(data, labels, probabilities, neighbors, core_distances,
                                     min_spanning_tree, lens_callback, num_clusters,
                                     sample_weights=None, **kwargs):
    """sub_clusters.py:64: compute_sub_clusters_in_cluster for every cluster.
    The per-cluster inputs come from one grouping pass (points and in-cluster
    MST edges in their original order, in-cluster ids in one array) instead
    of a scan of all points and edges per cluster; they are the same arrays."""
    labels = np.asarray(labels)
    parent_labels = labels[min_spanning_tree[:, 0].astype(np.int64)]
    child_labels = labels[min_spanning_tree[:, 1].astype(np.int64)]
    order = np.argsort(labels, kind="stable")
    bounds = np.searchsorted(labels[order], np.arange(num_clusters + 1))
    same = parent_labels == child_labels
    e_idx = np.nonzero(same)[0]
    e_order = e_idx[np.argsort(parent_labels[e_idx], kind="stable")]
    e_bounds = np.searchsorted(parent_labels[e_order], np.arange(num_clusters + 1))
    local = np.empty(len(labels), dtype=np.int32)
    for cluster in range(num_clusters):
        pts = order[bounds[cluster]:bounds[cluster + 1]]
        local[pts] = np.arange(len(pts), dtype=np.int32)
    per = []
    for cluster in range(num_clusters):
        points = order[bounds[cluster]:bounds[cluster + 1]]
        nb = neighbors[points, :]
        cl_nb = np.where(nb >= 0, labels[np.maximum(nb, 0)], -2) == cluster
        nb_local = np.where(cl_nb, local[np.maximum(nb, 0)], -1).astype(np.int32)
        mst = min_spanning_tree[e_order[e_bounds[cluster]:e_bounds[cluster + 1]]].copy()
        mst[:, :2] = local[mst[:, :2].astype(np.int64)]
        core = core_distances[points]
        lens_values = lens_callback(data, probabilities, nb_local, core, mst, points)
        per.append((points, lens_values, (nb_local, core, mst, lens_values)))
    # every cluster's core graph and forest on the GPU in one pass each, then
    # each cluster's hierarchy
    built = core_graphs_and_forests([inp for _, _, inp in per])

    # the clusters' hierarchies are independent: worker threads, each on its
    # own CUDA stream, overlap their short launches and copies
    torch = _native._torch()
    tls = threading.local()

    def hierarchy(i):
        (points, lens_values, _), (graph, nc, comp, forest) = per[i], built[i]
        if not hasattr(tls, "stream"):
            tls.stream = torch.cuda.Stream()
        with torch.cuda.stream(tls.stream):
            res = _clusters_of_forest(
                nc, comp, forest, graph,
                sample_weights=(sample_weights[points] if sample_weights is not None else None),
                **kwargs)
        tls.stream.synchronize()
        return (*res, lens_values, points)

    torch.cuda.current_stream().synchronize()
    if len(per) <= 1:
        return [hierarchy(i) for i in range(len(per))]
    with concurrent.futures.ThreadPoolExecutor(min(8, len(per))) as ex:
        return list(ex.map(hierarchy, range(len(per))))


def update_labels(cluster_probabilities, sub_labels_list, sub_probabilities_list,
                  lens_values_list, points_list, data_size):
    """sub_clusters.py:98: one labelling from the per-cluster results."""
    labels = np.full(data_size, -1, dtype=np.int64)
    probabilities = cluster_probabilities.copy()
    sub_labels = np.zeros(data_size, dtype=np.int64)
    sub_probabilities = np.zeros(data_size, dtype=np.float32)
    lens_values = np.zeros(data_size, dtype=np.float32)
    running_id = 0
    for points, _labels, _probs, _lens in zip(points_list, sub_labels_list,
                                              sub_probabilities_list, lens_values_list):
        unique_labels = np.unique(_labels)
        labels[points] = _labels + int(unique_labels[0] == -1) + running_id
        sub_labels[points] = _labels
        sub_probabilities[points] = _probs
        probabilities[points] += _probs
        probabilities[points] /= 2
        lens_values[points] = _lens
        running_id += len(unique_labels)
    return labels, probabilities, sub_labels, sub_probabilities, lens_values


def propagate_labels_per_cluster(graph, sub_labels):
    """sub_clusters.py:132: noise points take the label of greatest summed
    inverse lens weight among their labelled core-graph neighbours, repeated
    until every point that can be reached is labelled."""
    n = len(sub_labels)
    undirected = [dict() for _ in range(n)]
    for idx in range(n):
        for i in range(graph.indptr[idx], graph.indptr[idx + 1]):
            neighbor = int(graph.indices[i])
            w = 1.0 / float(graph.weights[i])
            if sub_labels[neighbor] == -1:
                undirected[neighbor][idx] = w
            if sub_labels[idx] == -1:
                undirected[idx][neighbor] = w
    while True:
        noise_idx = np.nonzero(sub_labels == -1)[0]
        if noise_idx.shape[0] == 0:
            break
        changed = False
        for idx in noise_idx:
            candidates = {}
            for neighbor_idx, weight in undirected[idx].items():
                label = sub_labels[neighbor_idx]
                if label == -1:
                    continue
                candidates[label] = candidates.get(label, 0.0) + weight
            if not candidates:
                continue
            max_weight, max_candidate = -np.inf, -1
            for candidate, weight in candidates.items():
                if weight > max_weight:
                    max_weight, max_candidate = weight, candidate
            sub_labels[idx] = max_candidate
            changed = True
        if not changed:  # unreachable noise stays noise (the reference loops forever)
            break
    return sub_labels


def propagate_sub_cluster_labels(labels, sub_labels, graph_list, points_list):
    """sub_clusters.py:170."""
    running_id = 0
    for points, core_graph in zip(points_list, graph_list):
        unique_sub_labels = np.unique(sub_labels[points])
        has_noise = unique_sub_labels[0] == -1 and len(unique_sub_labels) > 1
        if has_noise:
            sub_labels[points] = propagate_labels_per_cluster(core_graph, sub_labels[points])
        labels[points] = sub_labels[points] + running_id
        running_id += len(unique_sub_labels) - int(has_noise)
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
        lens_array = lens_callback[finite_index] if last_outlier > 0 else lens_callback
        lens_callback = lambda a, b, c, d, e, pts: lens_array[pts]  # noqa: E731

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
