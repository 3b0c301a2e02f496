"""GB300-native HDBSCAN engine behind fast_hdbscan's API (Euclidean fit path).

    from fast_hdbscan_gb300 import HDBSCAN
    labels = HDBSCAN(min_cluster_size=50, min_samples=10).fit_predict(X)

Every stage (spatial index, kNN core distances, Boruvka MST, linkage tree,
condensed tree, cluster selection, labels) runs as hand-written sm_103a CUDA
kernels in libfhg.so, called through the C ABI of include/fhg.h.
"""
from .branches import BranchDetector, find_branch_sub_clusters  # noqa: F401
from .hdbscan import HDBSCAN, fast_hdbscan  # noqa: F401
from .sub_clusters import SubClusterDetector, find_sub_clusters  # noqa: F401

__all__ = ["HDBSCAN", "fast_hdbscan", "BranchDetector", "find_branch_sub_clusters",
           "SubClusterDetector", "find_sub_clusters"]
