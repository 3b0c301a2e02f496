"""Seeded synthetic point clouds with the shapes of the HDBSCAN benchmark
workloads.  All generators return C-contiguous float32 arrays and are fully
determined by (n, seed).

* ``blobs_2d``       - 2-D, 10 isotropic Gaussian blobs (std 1.0, centres
                       U[-10,10]^2), 95 % blob points + 5 % uniform noise over
                       the bounding box.
* ``umap_like``      - 5-D, 40 blobs with std log-uniform in [0.2, 2.0],
                       Dirichlet(1) weights, centres U[-20,20]^5, 90 % blob
                       points + 10 % uniform noise.
* ``aniso_highdim``  - 64-D, 50 anisotropic Gaussians (covariance A A^T with
                       A_ij ~ N(0, 0.3^2)), centres N(0, 4 I).
* ``varying_density``- 3-D, 200 Gaussians with std log-normal(0, 1) and
                       centres U[-100,100]^3 (widely varying density).
* ``batch_instances``- many small mixtures of uneven size (3-12 blobs + 5 %
                       noise, d in 2..8).
"""
import numpy as np


def blobs_2d(n=20000, seed=0):
    rng = np.random.default_rng(seed)
    n_noise = int(round(0.05 * n))
    n_blob = n - n_noise
    centers = rng.uniform(-10.0, 10.0, size=(10, 2))
    which = rng.integers(0, 10, size=n_blob)
    pts = centers[which] + rng.normal(0.0, 1.0, size=(n_blob, 2))
    lo, hi = pts.min(axis=0), pts.max(axis=0)
    noise = rng.uniform(lo, hi, size=(n_noise, 2))
    X = np.concatenate([pts, noise])
    X = X[rng.permutation(n)]
    return np.ascontiguousarray(X, dtype=np.float32)


def umap_like(n=2_000_000, seed=1, dim=5, n_blobs=40):
    rng = np.random.default_rng(seed)
    n_noise = int(round(0.10 * n))
    n_blob = n - n_noise
    centers = rng.uniform(-20.0, 20.0, size=(n_blobs, dim))
    stds = np.exp(rng.uniform(np.log(0.2), np.log(2.0), size=n_blobs))
    weights = rng.dirichlet(np.ones(n_blobs))
    which = rng.choice(n_blobs, size=n_blob, p=weights)
    pts = centers[which] + rng.normal(0.0, 1.0, size=(n_blob, dim)) * stds[which, None]
    lo, hi = pts.min(axis=0), pts.max(axis=0)
    noise = rng.uniform(lo, hi, size=(n_noise, dim))
    X = np.concatenate([pts, noise])
    X = X[rng.permutation(n)]
    return np.ascontiguousarray(X, dtype=np.float32)


def aniso_highdim(n=1_000_000, seed=2, dim=64, n_comp=50):
    rng = np.random.default_rng(seed)
    centers = rng.normal(0.0, 2.0, size=(n_comp, dim))
    which = rng.integers(0, n_comp, size=n)
    X = np.empty((n, dim), dtype=np.float64)
    for c in range(n_comp):
        idx = np.nonzero(which == c)[0]
        A = rng.normal(0.0, 0.3, size=(dim, dim))
        X[idx] = centers[c] + rng.normal(0.0, 1.0, size=(idx.size, dim)) @ A.T
    return np.ascontiguousarray(X, dtype=np.float32)


def varying_density(n=10_000_000, seed=3, dim=3, n_comp=200):
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-100.0, 100.0, size=(n_comp, dim))
    stds = rng.lognormal(0.0, 1.0, size=n_comp)
    which = rng.integers(0, n_comp, size=n)
    X = centers[which] + rng.normal(0.0, 1.0, size=(n, dim)) * stds[which, None]
    return np.ascontiguousarray(X, dtype=np.float32)


def batch_instances(n_instances=4096, seed=4, n_min=200, n_max=200_000):
    """Returns a list of (X, min_samples, min_cluster_size) tuples."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_instances):
        n = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        d = int(rng.integers(2, 9))
        k = int(rng.integers(3, 13))
        n_noise = int(round(0.05 * n))
        n_blob = n - n_noise
        centers = rng.uniform(-10.0, 10.0, size=(k, d))
        which = rng.integers(0, k, size=n_blob)
        pts = centers[which] + rng.normal(0.0, 1.0, size=(n_blob, d))
        lo, hi = pts.min(axis=0), pts.max(axis=0)
        noise = rng.uniform(lo, hi, size=(n_noise, d))
        X = np.concatenate([pts, noise])[rng.permutation(n)]
        ms = int(rng.choice([5, 10, 20]))
        mcs = max(10, n // 100)
        out.append((np.ascontiguousarray(X, dtype=np.float32), ms, mcs))
    return out


WORKLOADS = {
    "blobs_2d": dict(gen=blobs_2d, n=20_000, min_samples=10, min_cluster_size=50),
    "umap_like": dict(gen=umap_like, n=2_000_000, min_samples=10, min_cluster_size=500),
    "aniso_highdim": dict(gen=aniso_highdim, n=1_000_000, min_samples=10,
                          min_cluster_size=500),
    "varying_density": dict(gen=varying_density, n=10_000_000, min_samples=15,
                            min_cluster_size=500),
}
