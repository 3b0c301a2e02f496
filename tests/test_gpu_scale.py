"""Parity at the benchmark's own scale: the 2M x 5-D UMAP-like input
(min_samples 10, min_cluster_size 500) and the 10M x 3-D varying-density
input (min_samples 15, min_cluster_size 500).

* Against the oracle in canonical tie mode (the engine's default rules):
  every output bit for bit.
* Against the oracle in the reference's tie mode (mode 2: the reference's
  sequential rules, evaluated in parallel): the MST weight multiset is
  identical, every differing label or probability lies on a tie-broken edge;
  the adjusted Rand index and the differing points are printed.
* With reproducible=True (the engine's reference tie mode): the MST, labels
  and probabilities equal the oracle's mode 2 bit for bit.
"""
import time

import numpy as np
import pytest

from fast_hdbscan_gb300 import synthetic
from parity import tie_report

pytestmark = pytest.mark.gpu

SCALE = [("umap_like", 2_000_000, 10, 500, 1), ("varying_density", 10_000_000, 15, 500, 3)]


@pytest.mark.parametrize("gen,n,ms,mcs,seed", SCALE)
def test_benchmark_scale_parity(engine, gen, n, ms, mcs, seed):
    import os

    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree, fast_hdbscan
    from oracle import oracle as O

    X = getattr(synthetic, gen)(n, seed=seed)
    t0 = time.perf_counter()
    labels, probs, linkage, ct, smst, nbrs, core = fast_hdbscan(
        X, min_samples=ms, min_cluster_size=mcs, return_trees=True)
    t_gpu = time.perf_counter() - t0
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    orc = O.fit(X, ms, mcs, mode=1, nthreads=cores)
    t_orc = time.perf_counter() - t0
    np.testing.assert_array_equal(core, orc.core)
    np.testing.assert_array_equal(nbrs, orc.neighbors)
    np.testing.assert_array_equal(smst, orc.sorted_mst)
    np.testing.assert_array_equal(linkage, orc.linkage)
    for a, b in zip(ct, orc.condensed):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(labels, orc.labels)
    np.testing.assert_array_equal(probs, orc.probabilities)
    canon_mst = orc.mst
    del orc
    ref = O.fit(X, ms, mcs, mode=2, nthreads=cores)
    np.testing.assert_array_equal(core, ref.core)
    ari, bad_l, bad_p, ties = tie_report(labels, probs, canon_mst, ref.labels,
                                         ref.probabilities, ref.mst)
    print(f"\n{gen} n={n}: GPU fit {t_gpu:.2f} s (incl. host copies), oracle {t_orc:.1f} s; "
          f"vs the reference's tie rules: ARI {ari:.8f}, labels differ at {bad_l} points, "
          f"probabilities at {bad_p}, {ties} points on tie-broken edges")
    # the reference tie mode: the reference's own tree, labels and probabilities
    mst_r, _, _ = compute_minimum_spanning_tree(X, min_samples=ms, reproducible=True)
    np.testing.assert_array_equal(mst_r, ref.mst)
    labels_r, probs_r = fast_hdbscan(X, min_samples=ms, min_cluster_size=mcs, reproducible=True)
    np.testing.assert_array_equal(labels_r, ref.labels)
    np.testing.assert_array_equal(probs_r, ref.probabilities)
    print(f"{gen} n={n}, reproducible=True: MST, labels and probabilities equal the "
          f"reference's tie rules bit for bit (ARI 1)")
