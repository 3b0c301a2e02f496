"""Branch detection within clusters (the reference's FLASC post-processing,
branches.py): sub-cluster detection on the lens "centrality" -- the inverse
distance of a point to its cluster's probability-weighted centroid -- and
then the branch-count rule that folds clusters with too few branches back
into one label.

Both steps run over all clusters at once: the centralities of every
clustered point in one pass over the cluster layout the sub-cluster driver
already builds (one centroid per cluster, then every point's distance
together), and the branch rule from one ``np.unique`` over (cluster, branch)
pairs.
"""
import numpy as np

from .sub_clusters import SubClusterDetector, find_sub_clusters


def _centroids(data, probabilities, points, bounds):
    """Probability-weighted centroid of every cluster (cluster c holds
    points[bounds[c]:bounds[c+1]]).  Each is np.average over the cluster's rows
    in index order, the lens's definition (branches.py:5-11), so the float32
    rounding is the reference's."""
    dt = np.result_type(data.dtype, probabilities.dtype)
    out = np.zeros((len(bounds) - 1, data.shape[1]), dtype=dt)
    for c in np.nonzero(np.diff(bounds) > 0)[0]:
        rows = points[bounds[c]:bounds[c + 1]]
        out[c] = np.average(data[rows], weights=probabilities[rows], axis=0)
    return out


def centralities(data, probabilities, points, bounds):
    """Centrality of every clustered point, clusters back to back as in
    ``points`` (cluster c at points[bounds[c]:bounds[c+1]]): 1 / the Euclidean
    distance to the cluster's weighted centroid (+inf at the centroid)."""
    data = np.asarray(data)
    probabilities = np.asarray(probabilities)
    points = np.asarray(points, dtype=np.int64)
    bounds = np.asarray(bounds, dtype=np.int64)
    cen = _centroids(data, probabilities, points, bounds)
    owner = np.repeat(np.arange(len(bounds) - 1), np.diff(bounds))
    offset = data[points] - cen[owner]
    with np.errstate(divide="ignore"):
        return 1 / np.linalg.norm(offset, axis=1)


def compute_centrality(data, probabilities, *args):
    """The centrality lens callback (branches.py:5) for one cluster: its
    points are the callback's last argument."""
    points = np.asarray(args[-1])
    return centralities(data, probabilities, points, np.array([0, len(points)]))


# the sub-cluster driver evaluates this lens for all clusters in one call
compute_centrality.all_clusters = centralities


def apply_branch_threshold(labels, branch_labels, probabilities, cluster_probabilities,
                           cluster_points, linkage_trees, label_sides_as_branches=False):
    """branches.py:14: a cluster that has a linkage tree but at most one
    branch (two, unless sides count as branches; noise not counted) keeps a
    single label and its cluster probabilities; any other cluster takes one
    label per branch, and its noise one more.  Labels are numbered cluster
    after cluster in ``cluster_points`` order.  Updates labels and
    probabilities in place."""
    n_cl = len(cluster_points)
    if n_cl == 0:
        return
    sizes = np.array([len(p) for p in cluster_points], dtype=np.int64)
    pts = np.concatenate([np.asarray(p, dtype=np.int64) for p in cluster_points])
    owner = np.repeat(np.arange(n_cl), sizes)
    br = np.asarray(branch_labels)[pts].astype(np.int64)
    # distinct (cluster, branch) pairs: how many branches, and whether noise
    span = int(br.max()) + 2
    pairs = np.unique(owner * span + (br + 1))
    pc, pb = pairs // span, pairs % span - 1
    distinct = np.bincount(pc, minlength=n_cl)
    noise = np.zeros(n_cl, dtype=np.int64)
    noise[pc[pb == -1]] = 1
    branches = distinct - noise
    has_tree = np.array([t is not None for t in linkage_trees], dtype=bool)
    keep_one = (branches <= (1 if label_sides_as_branches else 2)) & has_tree
    width = np.where(keep_one, 1, branches + noise)
    first = np.concatenate([[0], np.cumsum(width)[:-1]])
    one = keep_one[owner]
    labels[pts] = np.where(one, first[owner], br + noise[owner] + first[owner])
    probabilities[pts] = np.where(one, np.asarray(cluster_probabilities)[pts],
                                  probabilities[pts])


def find_branch_sub_clusters(clusterer, cluster_labels=None, cluster_probabilities=None,
                             label_sides_as_branches=False, min_cluster_size=None,
                             max_cluster_size=None, allow_single_cluster=None,
                             cluster_selection_method=None, cluster_selection_epsilon=0.0,
                             cluster_selection_persistence=0.0):
    """branches.py:37: sub-clusters on the centrality lens, then the branch
    rule; returns find_sub_clusters' tuple with labels and probabilities
    after the rule.  (The reference's own call leaves out the linkage trees
    the rule needs and raises a TypeError; they are passed here.)"""
    result = find_sub_clusters(
        clusterer, cluster_labels, cluster_probabilities, lens_callback=compute_centrality,
        min_cluster_size=min_cluster_size, max_cluster_size=max_cluster_size,
        allow_single_cluster=allow_single_cluster,
        cluster_selection_method=cluster_selection_method,
        cluster_selection_epsilon=cluster_selection_epsilon,
        cluster_selection_persistence=cluster_selection_persistence)
    (labels, probabilities, _, cluster_probs, branch_labels, _, _, _, linkage_trees, _, _,
     points) = result
    apply_branch_threshold(labels, branch_labels, probabilities, cluster_probs, points,
                           linkage_trees, label_sides_as_branches=label_sides_as_branches)
    return result


class BranchDetector(SubClusterDetector):
    """branches.py:70: flare (branch) detection within the clusters of a
    fitted HDBSCAN model; the parameters and fitted attributes of the
    reference's detector (branch_labels_, branch_probabilities_,
    centralities_ beside the sub-cluster attributes)."""

    def __init__(self, min_cluster_size=None, max_cluster_size=None, allow_single_cluster=None,
                 cluster_selection_method=None, cluster_selection_epsilon=0.0,
                 cluster_selection_persistence=0.0, propagate_labels=False,
                 label_sides_as_branches=False):
        super().__init__(min_cluster_size=min_cluster_size, max_cluster_size=max_cluster_size,
                         allow_single_cluster=allow_single_cluster,
                         cluster_selection_method=cluster_selection_method,
                         cluster_selection_epsilon=cluster_selection_epsilon,
                         cluster_selection_persistence=cluster_selection_persistence,
                         propagate_labels=propagate_labels)
        self.label_sides_as_branches = label_sides_as_branches

    def fit(self, clusterer, labels=None, probabilities=None, sample_weight=None):
        super().fit(clusterer, labels, probabilities, sample_weight, compute_centrality)
        apply_branch_threshold(self.labels_, self.sub_cluster_labels_, self.probabilities_,
                               self.cluster_probabilities_, self.cluster_points_,
                               self._linkage_trees,
                               label_sides_as_branches=self.label_sides_as_branches)
        self.branch_labels_ = self.sub_cluster_labels_
        self.branch_probabilities_ = self.sub_cluster_probabilities_
        self.centralities_ = self.lens_values_
        return self

    def propagated_labels(self, label_sides_as_branches=None):
        """Branch labels propagated to the noise points inside clusters, then
        the branch rule (probabilities are not returned, so zeros stand in)."""
        sides = (self.label_sides_as_branches if label_sides_as_branches is None
                 else label_sides_as_branches)
        labels, branch_labels = super().propagated_labels()
        scratch = np.zeros_like(self.probabilities_)
        apply_branch_threshold(labels, branch_labels, scratch, scratch, self.cluster_points_,
                               self._linkage_trees, label_sides_as_branches=sides)
        return labels, branch_labels

    @property
    def approximation_graph_(self):
        return super()._make_approximation_graph(lens_name="centrality",
                                                 sub_cluster_name="branch")
