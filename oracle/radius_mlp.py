"""numpy restatement of the learned-radius network -- TEST INFRASTRUCTURE ONLY.

Only the tests use this module, as the checker of the GPU forward and
backward kernels; the product library never imports it.  The network has no
counterpart in the reference (it proposes search radii for the kNN of
boruvka.py:561-585 / numba_kdtree.py:765 parallel_tree_query, whose results
it never changes); its definition is the engine's own:

    x  = bf16((f - mu) / sigma)
    h1 = bf16(relu(bf16(W1) x + b1))
    h2 = relu(bf16(W2) h1 + b2)
    y  = bf16(w3) . h2 + b3
    loss = mean((y - target)^2)

with float32 master weights and gradients that pass through the bfloat16
roundings unchanged.  ``bf=False`` drops the roundings (the exact network the
finite-difference check differentiates).
"""
import numpy as np

N_FEATURES, HIDDEN = 11, 64


def _layout():
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


def bf16(x):
    """Round float32 values to the nearest bfloat16 (ties to even), returned
    as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).reshape(a.shape)
    return np.where(np.isnan(a), a, out)


def _split(params, dtype):
    p = np.asarray(params, dtype=np.float32)
    d = {k: p[a:b] for k, (a, b) in LAYOUT.items()}
    W1 = d["W1"].reshape(HIDDEN, N_FEATURES)
    W2 = d["W2"].reshape(HIDDEN, HIDDEN)
    return W1, d["b1"], W2, d["b2"], d["w3"], d["b3"][0], d["mu"], d["sigma"]


def forward(params, feat, bf=True):
    """(y float64[n], cache) of the network on feature rows ``feat``."""
    r = bf16 if bf else (lambda v: np.asarray(v, np.float32))
    W1, b1, W2, b2, w3, b3, mu, sg = _split(params, np.float32)
    f = np.asarray(feat, np.float32)
    x = r(((f - mu) / sg).astype(np.float32)).astype(np.float64)
    W1r, W2r, w3r = (r(W1).astype(np.float64), r(W2).astype(np.float64),
                     r(w3).astype(np.float64))
    z1 = (x @ W1r.T + b1).astype(np.float32)
    h1 = r(np.maximum(z1, 0.0)).astype(np.float64)
    z2 = h1 @ W2r.T + b2
    h2 = np.maximum(z2, 0.0)
    y = h2 @ w3r + float(b3)
    return y, (x, h1, h2, W2r, w3r)


def gradient(params, feat, target, rows, bf=True):
    """(gradient of the trained parameters float64[N_TRAINED], loss) of the
    mean squared error over feature rows ``rows``."""
    rows = np.asarray(rows)
    y, (x, h1, h2, W2r, w3r) = forward(params, np.asarray(feat)[rows], bf)
    t = np.asarray(target, np.float64)[rows]
    B = len(rows)
    e = y - t
    dy = 2.0 * e / B
    d2 = np.where(h2 > 0, dy[:, None] * w3r[None, :], 0.0)
    d1 = np.where(h1 > 0, d2 @ W2r, 0.0)
    g = np.concatenate([
        (d1.T @ x).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0), dy @ h2, [dy.sum()]])
    assert g.size == N_TRAINED
    return g, float(np.mean(e * e))
