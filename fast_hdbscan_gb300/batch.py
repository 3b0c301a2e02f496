"""Many independent HDBSCAN fits in one call (fhg_hdbscan_fit_batch).

    from fast_hdbscan_gb300.batch import fit_many
    results = fit_many([X0, X1, ...], min_samples=[5, 10, ...], min_cluster_size=[...])

Every instance gets exactly the labels and probabilities of a single fit
(fast_hdbscan(X, min_samples, min_cluster_size)); the fits run concurrently on
a pool of worker streams inside the engine.  The number of streams can be
tuned per batch size signature (autotune_workers, fit_many(workers="auto")).
"""
import ctypes
import time

import numpy as np

from . import _native


def _per_instance(v, count, name):
    if np.ndim(v) == 0:
        return [v] * count
    v = list(v)
    if len(v) != count:
        raise ValueError(f"{name} needs one value per instance ({count}), got {len(v)}")
    return v


WORKER_CANDIDATES = (4, 8, 16, 32, 64)
_TUNED = {}  # size signature -> worker count


def _signature(instances):
    """Size bucket of a batch: log2 of its median instance size and of its
    instance count."""
    sizes = np.array([np.shape(X)[0] for X in instances], dtype=np.float64)
    return (int(np.log2(max(np.median(sizes), 1.0))), int(np.log2(max(len(sizes), 1))))


def autotune_workers(instances, min_samples=10, min_cluster_size=10, candidates=None,
                     sample=256, seed=0, **kwargs):
    """Pick the number of worker streams for batches like ``instances``: time
    fit_many on a random sample of them (a warm-up pass, then one timed pass
    per candidate) and keep the fastest for the batch's size signature.
    Returns ``(workers, {candidate: seconds})``."""
    torch = _native._torch()
    count = len(instances)
    ms = _per_instance(min_samples, count, "min_samples")
    mcs = _per_instance(min_cluster_size, count, "min_cluster_size")
    rng = np.random.default_rng(seed)
    pick = np.sort(rng.choice(count, min(sample, count), replace=False))
    Xs, m1, m2 = [instances[i] for i in pick], [ms[i] for i in pick], [mcs[i] for i in pick]
    candidates = tuple(candidates or WORKER_CANDIDATES)
    fit_many(Xs, m1, m2, workers=max(candidates), **kwargs)
    times = {}
    for w in candidates:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fit_many(Xs, m1, m2, workers=w, **kwargs)
        torch.cuda.synchronize()
        times[w] = time.perf_counter() - t0
    best = min(times, key=times.get)
    _TUNED[_signature(instances)] = best
    return best, times


def fit_many(instances, min_samples=10, min_cluster_size=10, cluster_selection_method="eom",
             max_cluster_size=np.inf, allow_single_cluster=False, workers=16):
    """Returns [(labels intp[n_i], probabilities float32[n_i]), ...].

    ``min_samples`` / ``min_cluster_size``: one value, or one per instance
    (min_samples None means min_cluster_size, as in fast_hdbscan).
    ``workers="auto"``: the count autotune_workers found for batches of this
    size signature (tuned on a sample of this batch when there is none)."""
    torch = _native._torch()
    count = len(instances)
    if workers == "auto":
        sig = _signature(instances)
        if sig not in _TUNED:
            autotune_workers(instances, min_samples, min_cluster_size,
                             cluster_selection_method=cluster_selection_method,
                             max_cluster_size=max_cluster_size,
                             allow_single_cluster=allow_single_cluster)
        workers = _TUNED[sig]
    ms = _per_instance(min_samples, count, "min_samples")
    mcs = _per_instance(min_cluster_size, count, "min_cluster_size")
    method = {"eom": 0, "leaf": 1}.get(cluster_selection_method)
    if method is None:
        raise ValueError(f"Invalid cluster_selection_method {cluster_selection_method}")
    Xs = [np.asarray(X) for X in instances]
    bad = "every instance must be a finite n x d array with d <= 30"
    for X in Xs:
        if X.ndim != 2 or X.shape[1] > 30:
            raise ValueError(bad)
    results = [None] * count
    run = [i for i in range(count) if Xs[i].shape[0] >= 2]
    for i in range(count):
        if Xs[i].shape[0] < 2:  # hdbscan.py:278-304
            if not np.all(np.isfinite(Xs[i])):
                raise ValueError(bad)
            results[i] = (np.full(Xs[i].shape[0], -1, dtype=np.intp),
                          np.zeros(Xs[i].shape[0], dtype=np.float32))
    if not run:
        return results
    sizes = np.array([Xs[i].size for i in run], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    npts = np.array([Xs[i].shape[0] for i in run], dtype=np.int64)
    poffs = np.concatenate([[0], np.cumsum(npts)])
    # every instance written once, as float32, straight into pinned memory;
    # the finite check runs on the GPU
    flat = torch.empty(int(offs[-1]), dtype=torch.float32, pin_memory=True)
    fv = flat.numpy()
    for j, i in enumerate(run):
        fv[offs[j]:offs[j + 1]] = Xs[i].reshape(-1)
    d_x = flat.to("cuda", non_blocking=True)
    if not bool(torch.isfinite(d_x).all()):
        raise ValueError(bad)
    d_lab = torch.empty(int(poffs[-1]), dtype=torch.int64, device="cuda")
    d_prob = torch.empty(int(poffs[-1]), dtype=torch.float32, device="cuda")
    m = len(run)
    P = ctypes.c_void_p
    xp = (P * m)(*[d_x.data_ptr() + 4 * int(offs[j]) for j in range(m)])
    lp = (P * m)(*[d_lab.data_ptr() + 8 * int(poffs[j]) for j in range(m)])
    pp = (P * m)(*[d_prob.data_ptr() + 4 * int(poffs[j]) for j in range(m)])
    nn = (ctypes.c_int64 * m)(*[int(v) for v in npts])
    dd = (ctypes.c_int32 * m)(*[Xs[i].shape[1] for i in run])
    msa = (ctypes.c_int32 * m)(*[int(mcs[i] if ms[i] is None else ms[i]) for i in run])
    mcsa = (ctypes.c_int64 * m)(*[int(mcs[i]) for i in run])
    status = (ctypes.c_int32 * m)()
    _native.check(_native.load().fhg_hdbscan_fit_batch(
        m, ctypes.cast(xp, P), ctypes.cast(nn, P), ctypes.cast(dd, P), ctypes.cast(msa, P),
        ctypes.cast(mcsa, P), method, float(max_cluster_size), int(bool(allow_single_cluster)),
        ctypes.cast(lp, P), ctypes.cast(pp, P), int(workers), ctypes.cast(status, P),
        _native.stream_ptr()))
    lab = torch.empty(d_lab.shape, dtype=torch.int64, pin_memory=True)
    prob = torch.empty(d_prob.shape, dtype=torch.float32, pin_memory=True)
    lab.copy_(d_lab, non_blocking=True)
    prob.copy_(d_prob, non_blocking=True)
    torch.cuda.current_stream().synchronize()
    # one copy out of pinned memory; each instance's results are views of it
    lab, prob = lab.numpy().astype(np.intp, copy=True), prob.numpy().copy()
    for j, i in enumerate(run):
        a, b = int(poffs[j]), int(poffs[j + 1])
        results[i] = (lab[a:b], prob[a:b])
    return results
