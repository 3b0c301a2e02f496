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
