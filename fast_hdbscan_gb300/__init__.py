"""GB300-native HDBSCAN engine behind fast_hdbscan's API (Euclidean fit path).

    from fast_hdbscan_gb300 import HDBSCAN
    labels = HDBSCAN(min_cluster_size=50, min_samples=10).fit_predict(X)

Every stage (spatial index, kNN core distances, Boruvka MST, linkage tree,
condensed tree, cluster selection, labels) runs as hand-written sm_103a CUDA
kernels in libfhg.so, called through the C ABI of include/fhg.h -- as do the
reference's other back-ends behind the same API: algorithm="kruskal" with a
kNN graph, metric="precomputed" sparse graphs, the kNN-graph route for data
above 30 dimensions (an exact tensor-core kNN), and sub-cluster / branch
detection (SubClusterDetector, BranchDetector).  batch.fit_many runs many
independent fits at once; radius.RadiusModel is an optional learned kNN
search radius that leaves every result unchanged.
"""
from .branches import BranchDetector, find_branch_sub_clusters  # noqa: F401
from .hdbscan import HDBSCAN, fast_hdbscan  # noqa: F401
from .sub_clusters import SubClusterDetector, find_sub_clusters  # noqa: F401

__all__ = ["HDBSCAN", "fast_hdbscan", "BranchDetector", "find_branch_sub_clusters",
           "SubClusterDetector", "find_sub_clusters"]
