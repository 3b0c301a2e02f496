"""Learned kNN search radius for the core-distance kNN.

A network 11 -> 64 -> 64 -> 1 (ReLU, bfloat16 operands, float32 accumulation)
predicts each point's log core distance from 11 features of the spatial
index: the first three coordinates scaled to the bounding box, and the log
point density of the point's 32-point bucket and of the 7 tree nodes above
it.  It is trained on the GPU by the engine's own forward, backward and Adam
kernels on the core distances that the plain kNN itself produces.

With a model in use, the kNN of the fit (the core distances of
boruvka.py:561-585 / parallel_tree_query) starts every query with the
predicted radius times ``margin`` as its search bound and certifies the
result: a query with fewer than k points inside its radius is searched again
without a bound.  Every output -- neighbours, core distances, the MST, labels
-- is therefore identical to the plain search's; the model only decides how
early the search can prune.

    model = RadiusModel.train(X_train, min_samples=15)
    with model.active():
        labels = HDBSCAN(min_samples=15).fit(X).labels_
    model.last_fallbacks()      # queries the certified search redid
"""
import contextlib
import ctypes

import numpy as np

from . import _native

N_FEATURES = 11
HIDDEN = 64


def param_count():
    return int(_native.load().fhg_radius_param_count())


def _layout():
    """Offsets of the float32 parameter block (W1, b1, W2, b2, w3, b3, mu,
    sigma) as the kernels read it."""
    sizes = [("W1", HIDDEN * N_FEATURES), ("b1", HIDDEN), ("W2", HIDDEN * HIDDEN),
             ("b2", HIDDEN), ("w3", HIDDEN), ("b3", 1), ("mu", N_FEATURES),
             ("sigma", N_FEATURES)]
    out, off = {}, 0
    for name, sz in sizes:
        out[name] = (off, off + sz)
        off += sz
    return out, off


LAYOUT, N_PARAMS = _layout()
N_TRAINED = LAYOUT["mu"][0]


def unpack(params):
    """numpy parameter block -> dict of arrays (W1 64x11, W2 64x64, ...)."""
    p = np.asarray(params, dtype=np.float32)
    d = {k: p[a:b] for k, (a, b) in LAYOUT.items()}
    d["W1"] = d["W1"].reshape(HIDDEN, N_FEATURES)
    d["W2"] = d["W2"].reshape(HIDDEN, HIDDEN)
    d["b3"] = d["b3"][0]
    return d


def _index_of(X):
    from .numba_kdtree import build_kdtree
    return build_kdtree(np.ascontiguousarray(X, dtype=np.float32))


def features(X=None, tree=None):
    """The 11 features of every point of X (caller order), as a CUDA tensor."""
    torch = _native._torch()
    tree = tree if tree is not None else _index_of(X)
    n = tree.data.shape[0]
    f = torch.empty((n, N_FEATURES), dtype=torch.float32, device="cuda")
    _native.check(_native.load().fhg_radius_features(tree.index.handle, _native.vptr(f),
                                                      _native.stream_ptr()))
    return f


def log_core_targets(tree, min_samples):
    """log of every point's core distance for ``min_samples`` (the distance to
    its min_samples-th neighbour, itself excluded -- the k-th entry of the
    fit's kNN with k = min_samples + 1)."""
    torch = _native._torch()
    n = tree.data.shape[0]
    t = torch.empty((n,), dtype=torch.float32, device="cuda")
    k = int(min_samples) + 1 if min_samples > 1 else 2
    _native.check(_native.load().fhg_radius_targets(tree.index.handle, min(k, n),
                                                     _native.vptr(t), _native.stream_ptr()))
    return t


class RadiusModel:
    """A trained radius network (parameters on the GPU) and its margin."""

    def __init__(self, params, margin=1.0, min_samples=None, loss_curve=None):
        torch = _native._torch()
        self.params = torch.as_tensor(np.asarray(params, np.float32)).cuda().contiguous() \
            if not (hasattr(params, "is_cuda") and params.is_cuda) else params.contiguous()
        if self.params.numel() != N_PARAMS:
            raise ValueError(f"a radius model has {N_PARAMS} parameters")
        self.margin = float(margin)
        self.min_samples = min_samples
        self.loss_curve = loss_curve

    # ------------------------------------------------------------ training
    @classmethod
    def train(cls, X, min_samples=15, steps=1500, batch=4096, lr=3e-3, seed=0,
              quantile=0.99):
        """Train on the core distances of X (the plain kNN's own output) and
        set the margin to the ``quantile`` of exp(target - prediction) over
        the training points, so that about that share of queries certify."""
        torch = _native._torch()
        tree = _index_of(X)
        n = tree.data.shape[0]
        feat = features(tree=tree)
        tgt = log_core_targets(tree, min_samples)
        lib = _native.load()
        params = torch.empty((N_PARAMS,), dtype=torch.float32, device="cuda")
        s = _native.stream_ptr()
        _native.check(lib.fhg_radius_init(_native.vptr(params), _native.vptr(feat),
                                          _native.vptr(tgt), n, int(seed), s))
        curve = torch.zeros((int(steps),), dtype=torch.float32, device="cuda")
        _native.check(lib.fhg_radius_train(_native.vptr(params), _native.vptr(feat),
                                           _native.vptr(tgt), n, int(steps), int(batch),
                                           float(lr), int(seed), _native.vptr(curve), s))
        model = cls(params, 1.0, min_samples, curve.cpu().numpy())
        y = model.predict_log(feat=feat)
        resid = tgt.cpu().numpy() - y
        model.margin = float(np.exp(max(np.quantile(resid, quantile), 0.0)))
        model.train_rmse = float(np.sqrt(np.mean(resid.astype(np.float64) ** 2)))
        return model

    # ------------------------------------------------------------ inference
    def predict_log(self, X=None, feat=None):
        """Predicted log core distance of every point (numpy float32)."""
        torch = _native._torch()
        if feat is None:
            feat = features(X)
        n = feat.shape[0]
        y = torch.empty((n,), dtype=torch.float32, device="cuda")
        _native.check(_native.load().fhg_radius_forward(
            _native.vptr(self.params), _native.vptr(feat), n, _native.vptr(y),
            _native.stream_ptr()))
        return y.cpu().numpy()

    def knn(self, tree, k):
        """parallel_tree_query(tree, tree.data, k, output_rdist=True) through
        the certified radius search: (rdist, indices, fallbacks)."""
        torch = _native._torch()
        n = tree.data.shape[0]
        rd = torch.empty((n, k), dtype=torch.float32, device="cuda")
        ix = torch.empty((n, k), dtype=torch.int32, device="cuda")
        fb = ctypes.c_int64(0)
        _native.check(_native.load().fhg_index_knn_radius(
            tree.index.handle, int(k), _native.vptr(self.params), ctypes.c_float(self.margin),
            _native.vptr(rd), _native.vptr(ix), ctypes.byref(fb), _native.stream_ptr()))
        return rd.cpu().numpy(), ix.cpu().numpy(), int(fb.value)

    @contextlib.contextmanager
    def active(self):
        """Fits made by this thread inside the block search their kNN with
        this model."""
        lib = _native.load()
        _native.check(lib.fhg_radius_use(_native.vptr(self.params), ctypes.c_float(self.margin)))
        try:
            yield self
        finally:
            lib.fhg_radius_use(None, ctypes.c_float(1.0))

    @staticmethod
    def last_fallbacks():
        """Queries the calling thread's last radius search searched again."""
        c = ctypes.c_int64(0)
        _native.check(_native.load().fhg_radius_fallbacks(ctypes.byref(c),
                                                          _native.stream_ptr()))
        return int(c.value)

    def gradient(self, feat, target, rows):
        """(grad of the trained parameters, loss) of the mean squared error
        over feature rows ``rows`` -- the backward kernels' output."""
        torch = _native._torch()
        r = torch.as_tensor(np.asarray(rows, np.int32)).cuda()
        g = torch.empty((N_TRAINED,), dtype=torch.float32, device="cuda")
        loss = torch.empty((1,), dtype=torch.float32, device="cuda")
        _native.check(_native.load().fhg_radius_backward(
            _native.vptr(self.params), _native.vptr(feat), _native.vptr(target), _native.vptr(r),
            int(r.numel()), _native.vptr(g), _native.vptr(loss), _native.stream_ptr()))
        return g.cpu().numpy(), float(loss.cpu().numpy()[0])
