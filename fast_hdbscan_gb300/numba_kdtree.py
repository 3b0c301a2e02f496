"""GPU spatial index behind the reference's KD-tree entry points.

Mirrors fast_hdbscan/numba_kdtree.py: ``build_kdtree`` returns a tree object
whose ``data`` attribute is the float32 copy of the input (the only field the
fit path reads), and ``parallel_tree_query`` returns the k nearest neighbours
of every point, itself included.  The index itself is a Morton-ordered bucket
tree on the GPU (see include/fhg.h).
"""
import numpy as np

from . import _native


class GpuKDTree:
    """Stand-in for the reference's NumbaKDTree namedtuple (numba_kdtree.py:7)."""

    def __init__(self, data):
        self.data = np.ascontiguousarray(data, dtype=np.float32)
        if self.data.ndim != 2:
            raise ValueError("data must be a 2-D array")
        self._X = _native.to_device(self.data, np.float32)
        self._index = _native.Index(self._X)

    @property
    def index(self):
        return self._index


def build_kdtree(data, leaf_size=40):
    """numba_kdtree.py:478 build_kdtree (leaf_size is accepted for signature
    compatibility; the GPU index always uses buckets of 32 points)."""
    if leaf_size < 1:
        raise ValueError("leaf_size must be greater than or equal to 1")
    return GpuKDTree(data)


def parallel_tree_query(tree, data, k=10, output_rdist=False):
    """numba_kdtree.py:765 parallel_tree_query for data == tree.data."""
    torch = _native._torch()
    if data is not tree.data and not np.array_equal(np.asarray(data, np.float32), tree.data):
        raise NotImplementedError("queries must be the indexed points (tree.data)")
    n = tree.data.shape[0]
    rd = torch.empty((n, k), dtype=torch.float32, device="cuda")
    ix = torch.empty((n, k), dtype=torch.int32, device="cuda")
    lib = _native.load()
    _native.check(lib.fhg_index_knn(tree.index.handle, int(k), _native.dptr(rd),
                                    _native.dptr(ix), _native.stream_ptr()))
    rd_h, ix_h = rd.cpu().numpy(), ix.cpu().numpy()
    if not output_rdist:
        rd_h = np.sqrt(rd_h)
    return rd_h, ix_h


class ReferenceKDTree:
    """The reference's NumbaKDTree fields (numba_kdtree.py:7): data,
    idx_array, idx_start, idx_end, radius, is_leaf, node_bounds."""

    def __init__(self, data, idx_array, idx_start, idx_end, radius, is_leaf, node_bounds):
        self.data = data
        self.idx_array = idx_array
        self.idx_start = idx_start
        self.idx_end = idx_end
        self.radius = radius
        self.is_leaf = is_leaf
        self.node_bounds = node_bounds


def node_ranges(n, levels):
    """idx_start, idx_end and is_leaf of the reference's tree over n points
    with `levels` levels (numba_kdtree.py:478-509): every node's range is
    halved, the left child taking the smaller half; a node is a leaf in the
    last level or below 2 points, and nodes under a leaf stay zero."""
    nodes = 2 ** levels - 1
    start = np.zeros(nodes, dtype=np.intp)
    end = np.zeros(nodes, dtype=np.intp)
    leaf = np.zeros(nodes, dtype=np.bool_)
    level = np.array([0], dtype=np.int64)
    s, e = np.array([0], dtype=np.int64), np.array([n], dtype=np.int64)
    while level.size:
        start[level], end[level] = s, e
        is_leaf = (2 * level + 1 >= nodes) | (e - s < 2)
        leaf[level] = is_leaf
        keep = ~is_leaf
        level, s, e = level[keep], s[keep], e[keep]
        mid = s + (e - s) // 2
        level = np.concatenate([2 * level + 1, 2 * level + 2])
        s, e = np.concatenate([s, mid]), np.concatenate([mid, e])
    return start, end, leaf


def build_reference_kdtree(data, leaf_size=40):
    """numba_kdtree.py:478 build_kdtree exactly -- the reference's own
    median-split KD-tree, built on the GPU (fhg_reference_kdtree), every
    partition of its build reproduced, so that idx_array and node_bounds are
    the reference's arrays.  Only leaf_size=40 (the reference's default, the
    one its fit uses) is supported."""
    if leaf_size != 40:
        raise NotImplementedError("build_reference_kdtree supports leaf_size=40 only")
    data = np.ascontiguousarray(data, dtype=np.float32)
    if data.ndim != 2:
        raise ValueError("data must be a 2-D array")
    n, d = data.shape
    torch = _native._torch()
    lib = _native.load()
    levels = int(lib.fhg_reference_kdtree_levels(n))
    nodes = 2 ** levels - 1
    X = _native.to_device(data, np.float32)
    idx = torch.empty(n, dtype=torch.int32, device="cuda")
    bounds = torch.empty((2, nodes, d), dtype=torch.float32, device="cuda")
    _native.check(lib.fhg_reference_kdtree(_native.dptr(X), n, d, _native.dptr(idx),
                                           _native.dptr(bounds), _native.stream_ptr()))
    start, end, leaf = node_ranges(n, levels)
    node_bounds = bounds.cpu().numpy()
    visited = end > start
    # _init_node's radius: half the box diagonal, float32 (numba_kdtree.py:101-111)
    half = np.abs(node_bounds[1] - node_bounds[0]) * np.float32(0.5)
    radius = np.zeros(nodes, dtype=np.float32)
    acc = np.zeros(nodes, dtype=np.float32)
    for j in range(d):
        acc = acc + half[:, j] * half[:, j]
    radius[visited] = np.sqrt(acc[visited])
    node_bounds[:, ~visited] = 0.0
    return ReferenceKDTree(data, idx.cpu().numpy().astype(np.intp), start, end, radius, leaf,
                           node_bounds)
