"""The certificate of the high-dimensional kNN (highd.cu) restated in numpy:
for every pair, the lower bound the kernel derives from a bfloat16 split
estimate never exceeds the pair's true squared distance.  The estimate is
formed as the kernel forms it -- centred float32 coordinates split into two
bfloat16 terms, float32 norms in dimension order, a float32 dot product over
the 3 dp concatenated terms -- and the bound uses the kernel's constants."""
import numpy as np
import pytest

from oracle.radius_mlp import bf16

U = 2.0 ** -24


def _estimate(X):
    n, d = X.shape
    dp = 32 if d <= 32 else (64 if d <= 64 else 96)
    mu = X.astype(np.float64).mean(0).astype(np.float32)
    c = (X - mu).astype(np.float32)
    hi = bf16(c)
    lo = bf16((c - hi).astype(np.float32))
    y = (hi + lo).astype(np.float32)
    ny = np.zeros(n, np.float32)
    for k in range(d):  # dimension order, float32 at every step
        ny = (ny + y[:, k] * y[:, k]).astype(np.float32)
    A = np.concatenate([hi, hi, lo], axis=1).astype(np.float32)
    B = np.concatenate([hi, lo, hi], axis=1).astype(np.float32)
    dot = np.zeros((n, n), np.float32)
    for k in range(A.shape[1]):  # float32 accumulation over the 3 d terms
        dot = (dot + np.outer(A[:, k], B[:, k]).astype(np.float32)).astype(np.float32)
    Dt = np.maximum((ny[:, None] + ny[None, :]).astype(np.float32) - (2 * dot).astype(np.float32),
                    0).astype(np.float32)
    cn = np.sqrt((c.astype(np.float64) ** 2).sum(1)).astype(np.float32)
    return Dt, ny, cn, dp


@pytest.mark.parametrize("d,offset,scale", [(40, 0.0, 1.0), (64, 50.0, 3.0), (96, -7.0, 0.01)])
def test_certificate_lower_bound_is_sound(d, offset, scale):
    rng = np.random.default_rng(d)
    X = (offset + scale * rng.normal(size=(160, d))).astype(np.float32)
    Dt, ny, cn, dp = _estimate(X)
    kw = 3 * dp
    ymax, cmax = np.sqrt(ny.max()), cn.max()
    yq = np.sqrt(ny)
    eta = ((2 * kw + 4 * dp + 16) * U * (yq + ymax) ** 2 * 1.0001
           + 2.0 ** -15 * cn * cmax * 1.0001)
    E = (2.0 ** -16 + 2.0 ** -23) * (cn + cmax) * 1.0001
    a2 = Dt - eta[:, None]
    lb = np.where(a2 > 0, np.sqrt(np.maximum(a2, 0)) * (1 - 2.0 ** -20), 0) - E[:, None]
    lb = np.maximum(lb, 0)
    Xd = X.astype(np.float64)
    true = ((Xd[:, None, :] - Xd[None, :, :]) ** 2).sum(-1)
    # every non-candidate's float32 distance is at least lb^2 (1 - (d + 8) 2^-23)
    assert np.all(lb ** 2 * (1 - (d + 8) * 2.0 ** -23) <= true * (1 + 1e-12) + 1e-30)
    # and the bound is useful: close to the truth for most pairs
    off = ~np.eye(len(X), dtype=bool)
    rel = np.sqrt(lb[off] ** 2 / true[off])
    assert np.median(rel) > 0.99
