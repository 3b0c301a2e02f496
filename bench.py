#!/usr/bin/env python
"""HDBSCAN fit throughput on GB300: points/s for one full fit.

Workload: the 10M x 3-D varying-density set (200 Gaussians, std
log-normal(0, 1), centres U[-100, 100]^3), min_samples=15,
min_cluster_size=500, seeded synthetic data.  A step is one complete fit
(spatial index, kNN core distances, Boruvka MST, linkage tree, condensed
tree, EOM selection, labels and membership strengths).

  value  device-resident: X already in HBM, every output left in HBM.
  e2e    HDBSCAN(...).fit(X) from pinned host memory, all fitted attributes
         (labels_, probabilities_, trees, neighbours, core distances) read
         back to host inside the timed region.

--impl reference times the CPU restatement of the reference algorithm
(oracle/, OpenMP over the reference's parallel loops) on all host cores, each
step one fit of the same seeded 10M-point input (about half a minute on 16
cores); cpu_baseline in the default line is one such fit.

Multi-GPU: one process per GPU, each fitting its own independent dataset
(the fit does not shard without a per-round exchange): weak scaling,
replicas only.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "HDBSCAN fit points/s at 10M x 3-D (varying density, min_samples=15)"
WORKLOAD = dict(workload="varying_density_10M_3d", n=10_000_000, d=3, min_samples=15,
                min_cluster_size=500, seed=3,
                generator="200 Gaussians, std lognormal(0,1), centres U[-100,100]^3")
# Other configurations of the benchmark family, for reports (--workload):
# the 2M x 5-D UMAP-like input (40 blobs, std log-uniform [0.2, 2], Dirichlet
# weights, centres U[-20, 20]^5, 10 % noise).
OTHER_WORKLOADS = {
    "umap2m": dict(workload="umap_like_2M_5d", n=2_000_000, d=5, min_samples=10,
                   min_cluster_size=500, seed=1,
                   generator="40 blobs, std logU[0.2,2], Dirichlet weights, centres "
                             "U[-20,20]^5, 10% noise"),
    # a 15-NN distance graph of 1M points of the metric's generator, metric="precomputed"
    "precomputed1m": dict(workload="knn15_graph_1M_3d_precomputed", n=1_000_000, d=3,
                          min_samples=10, min_cluster_size=100, seed=3, metric="precomputed",
                          graph_k=15, algorithm="kruskal",
                          generator="15-NN float64 distance graph (scipy sparse) of 200 "
                                    "Gaussians, std lognormal(0,1), centres U[-100,100]^3"),
    # the metric's data through the algorithm="kruskal" back-end (kNN graph, knn_k=16)
    "kruskal10m": dict(workload="varying_density_10M_3d_kruskal_knn16", n=10_000_000, d=3,
                       min_samples=15, min_cluster_size=500, seed=3, algorithm="kruskal",
                       knn_k=16,
                       generator="200 Gaussians, std lognormal(0,1), centres U[-100,100]^3"),
    # the high-dimensional route (d > 30 without weights: the kNN-graph
    # back-end, nndescent.py:179) on the exact tensor-core kNN, knn_k = 30
    "highd1m": dict(workload="aniso_highdim_1M_64d_knn_graph", n=1_000_000, d=64,
                    min_samples=10, min_cluster_size=500, seed=2, algorithm="knn_graph",
                    knn_k=30, cpu_sample=30_000,
                    generator="50 anisotropic Gaussians (covariance A A^T, A_ij ~ N(0, 0.3^2)),"
                              " centres N(0, 4 I)"),
}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=WORKLOAD["n"], help="points (testing only)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-radius", action="store_true", help="skip the learned-radius arm")
    ap.add_argument("--no-ref-ties", action="store_true",
                    help="skip the reference-tie-mode arm (reproducible=True)")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched-instances figure of the default line")
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="points per CPU fit (default: the workload's own size)")
    ap.add_argument("--workload", default="fit", choices=["fit", "batched", *OTHER_WORKLOADS],
                    help="fit: the metric's 10M x 3-D fit; batched: many independent fits; "
                         "umap2m: the 2M x 5-D fit; kruskal10m: the 10M x 3-D fit on the "
                         "kNN-graph Kruskal back-end; highd1m: the 1M x 64-D fit on the "
                         "kNN-graph route with the tensor-core kNN")
    ap.add_argument("--instances", type=int, default=4096, help="batched workload size")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value, device):
    """The largest value over all ranks (the slowest rank's step time)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_data(n, seed):
    from fast_hdbscan_gb300 import synthetic

    if WORKLOAD["workload"].startswith("umap_like"):
        return synthetic.umap_like(n, seed=seed, dim=WORKLOAD["d"])
    if WORKLOAD["workload"].startswith("aniso_highdim"):
        return synthetic.aniso_highdim(n, seed=seed, dim=WORKLOAD["d"])
    return synthetic.varying_density(n, seed=seed)


# --------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- gb300 arm
def tree_nodes(n):
    """Nodes of the bucket tree: a complete binary tree over the 32-point
    buckets, its leaf level padded to a power of two."""
    leaves = (n + 31) // 32
    slots = 1
    while slots < leaves:
        slots *= 2
    return 2 * slots - 1


def algorithmic_bytes(kernel, n, k, d_pad):
    """Least HBM bytes one launch of a timed kernel must move, counted narrowly
    (every other access of the walk is a cache-resident re-read).  Reported as
    a second, labelled figure beside the stage-level formulas below."""
    if kernel == "knn_kernel":
        # read every point once (padded coordinates + caller index); write the
        # Morton-order rows (squared distance + position), the caller-order
        # neighbour matrix (k - 1 columns) and the one-byte boundary-tie flag
        return n * (4 * d_pad + 4) + n * k * 8 + n * (k - 1) * 4 + n
    if kernel == "search_kernel":
        # per pass: each point's component, core distance, candidate (weight
        # + position), k-th distance and tie flag; each tree node's
        # (component, least core) word
        return n * (4 + 4 + 8 + 4 + 1) + tree_nodes(n) * 8
    return None


def boruvka_round_bytes(n, k, d, components):
    """Algorithmic HBM bytes of one Boruvka round (fixed formula): per point
    its k kNN edges (destination i32 + weight f32 + the destination's gathered
    component i32), its coordinates, core distance, component and packed
    candidate (4d + 4 + 4 + 8), the relabel read + write (8); per component
    its packed best edge (8)."""
    return n * k * 12 + n * (4 * d + 16) + 8 * components + n * 8


def knn_stage_bytes(n, k, d):
    """Algorithmic HBM bytes of the kNN / core-distance stage (fixed formula):
    read X (4d per point), the spatial sort's write + read of the permuted
    points and keys ((4d + 8) x 2), the kNN rows written (distance + index, 8
    per neighbour) and the core distance (4)."""
    return n * 4 * d + n * (4 * d + 8) * 2 + n * k * 8 + n * 4


# The high-dimensional candidate kernel: GEMM depth per point pair and the
# instruction path (kept beside the algorithmic 2 n^2 d count).
HD_KERNEL_NOTE = ("tcgen05.mma 128x128x16 bf16 into tensor memory, TMA operand tiles, "
                  "two-term split (hi, lo): depth 3 x padded d rounded up to 64")


def hd_kernel_depth(d):
    if d <= 64:  # the tcgen05 pipeline's rows: whole 64-element segments
        return -(-3 * (32 if d <= 32 else 64) // 64) * 64
    return 3 * 96


def traffic_per_point(kernel):
    """DRAM bytes per point and launch measured by ncu, from the committed
    summary (profiles/ncu_traffic_per_point.txt: '<kernel> <bytes>' lines)."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic_per_point.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) == 2 and parts[0] == kernel:
                return float(parts[1])
    except OSError:
        pass
    return None


def run_gb300(args):
    import torch
    import torch.distributed as dist

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from fast_hdbscan_gb300 import _native, build as engine_build
    from fast_hdbscan_gb300.hdbscan import HDBSCAN

    engine_build.build()
    lib = _native.load()
    lib.fhg_launch_count.restype = ctypes.c_uint64
    lib.fhg_profile_enable.argtypes = [ctypes.c_int]
    lib.fhg_profile_report.argtypes = [ctypes.c_char_p, ctypes.c_int64]

    n = args.n
    ms, mcs = WORKLOAD["min_samples"], WORKLOAD["min_cluster_size"]
    pre = WORKLOAD.get("metric") == "precomputed"
    kruskal = WORKLOAD.get("algorithm") == "kruskal" and not pre
    kgraph = WORKLOAD.get("algorithm") == "knn_graph"
    knn_k = WORKLOAD.get("knn_k", 0)
    Xh = make_data(n, WORKLOAD["seed"] + rank)
    d = Xh.shape[1]
    Xd = torch.from_numpy(Xh).cuda()
    if pre:  # the input graph: every point's graph_k nearest points, float64 distances
        from fast_hdbscan_gb300.numba_kdtree import build_kdtree, parallel_tree_query

        gk = WORKLOAD["graph_k"]
        rd, gi = parallel_tree_query(build_kdtree(Xh), Xh, k=gk + 1, output_rdist=True)
        g_rows = torch.arange(n, dtype=torch.int32).repeat_interleave(gk).cuda()
        g_cols = torch.from_numpy(np.ascontiguousarray(gi[:, 1:])).reshape(-1).cuda()
        g_data = torch.from_numpy(np.sqrt(rd[:, 1:].astype(np.float64))).reshape(-1).cuda()
        nnz = n * gk
    E = _native.empty
    labels, probs = E(n, np.int64), E(n, np.float32)
    mst, linkage = E((n - 1, 3), np.float64), E((n - 1, 4), np.float64)
    ctp, ctc, ctl, cts = (E(2 * n, np.int64), E(2 * n, np.int64), E(2 * n, np.float32),
                          E(2 * n, np.float32))
    nbrs, sel = E((n, ms), np.int32), E(n, np.int64)
    core = E(n, np.float64 if (kruskal or pre or kgraph) else np.float32)
    rows, nsel = ctypes.c_int64(0), ctypes.c_int64(0)
    V = _native.vptr
    stream = torch.cuda.current_stream()

    def step():
        if pre:
            _native.check(lib.fhg_hdbscan_fit_precomputed(
                V(g_rows), V(g_cols), V(g_data), nnz, n, ms, 1, mcs, 0, float("inf"), 0, 0.0,
                0.0, V(labels), V(probs), V(mst), V(linkage), V(ctp), V(ctc), V(ctl), V(cts),
                ctypes.byref(rows), V(nbrs), V(core), V(sel), ctypes.byref(nsel),
                _native.stream_ptr()))
            return
        if kgraph:
            _native.check(lib.fhg_hdbscan_fit_knn_graph(
                V(Xd), n, d, ms, knn_k, mcs, 0, float("inf"), 0, 0.0, 0.0, V(labels), V(probs),
                V(mst), V(linkage), V(ctp), V(ctc), V(ctl), V(cts), ctypes.byref(rows),
                V(nbrs), V(core), V(sel), ctypes.byref(nsel), _native.stream_ptr()))
            return
        if kruskal:
            _native.check(lib.fhg_hdbscan_fit_kruskal(
                V(Xd), n, d, ms, knn_k, max(knn_k, ms) + 1, mcs, 0, float("inf"), 0, 0.0, 0.0,
                None, V(labels), V(probs), V(mst), V(linkage), V(ctp), V(ctc), V(ctl), V(cts),
                ctypes.byref(rows), V(nbrs), V(core), V(sel), ctypes.byref(nsel),
                _native.stream_ptr()))
            return
        _native.check(lib.fhg_hdbscan_fit(
            V(Xd), n, d, ms, mcs, 0, float("inf"), 0, 0.0, 0.0, None, 0, V(labels), V(probs), V(mst),
            V(linkage), V(ctp), V(ctc), V(ctl), V(cts), ctypes.byref(rows), V(nbrs), V(core),
            V(sel), ctypes.byref(nsel), _native.stream_ptr()))

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    lib.fhg_profile_report(None, 0)  # drop warm-up records
    lib.fhg_profile_enable(1)
    launches0 = lib.fhg_launch_count()
    with ClockSampler(local) as clocks:
        barrier()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        barrier()
    launches = lib.fhg_launch_count() - launches0
    lib.fhg_profile_enable(0)
    buf = ctypes.create_string_buffer(1 << 16)
    lib.fhg_profile_report(buf, len(buf))
    stages = json.loads(buf.value.decode() or "{}")
    ms_step = ev0.elapsed_time(ev1) / args.steps
    ms_step_max = max_over_ranks(ms_step, torch.device("cuda", local))
    value = n * world / (ms_step_max / 1e3)
    clock_info = clocks.summary()

    # per-stage share and the dominant kernel's roofline
    # kernel records nest inside the stage records: shares are over stages
    nested = ("knn_kernel", "search_kernel", "hd_cand_kernel", "hd_rerank_kernel",
              "hd_exact_kernel", "highd_knn", "boruvka_components")
    total_stage = sum(v[0] for k, v in stages.items() if k not in nested) or 1.0
    kernel_stages = {k: v for k, v in stages.items()
                     if k in ("knn_kernel", "search_kernel", "hd_cand_kernel")}
    dom = max(kernel_stages, key=lambda k: kernel_stages[k][0]) if kernel_stages else None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        peak, peak_src = 6800.0, "fallback"
    roofline = None
    rounds = stages.get("boruvka_components", [0, 0])[1] // max(args.steps, 1)
    if dom == "hd_cand_kernel":
        # tensor-bound: 2 n^2 K flops per launch, K = 3 x 64 (two-term bf16
        # split) for d = 64; against the measured cuBLAS bf16 burst peak
        tot_ms, cnt = kernel_stages[dom]
        per_launch_ms = tot_ms / cnt
        # the candidate GEMM's algorithmic count, 2 n^2 d; the kernel's own
        # depth (padding and a two-term split) is reported beside it
        flops = 2.0 * n * n * d
        kdepth = hd_kernel_depth(d)
        achieved = flops / (per_launch_ms / 1e3) / 1e12
        try:
            tpeak, tsrc = float(peaks["bf16_tflops"]), "measured cuBLAS bf16 burst"
        except (KeyError, ValueError, TypeError):
            tpeak, tsrc = 1900.0, "fallback"
        roofline = {"bound": "tensor", "kernel": dom, "achieved": round(achieved, 2),
                    "peak": tpeak, "peak_source": tsrc, "unit": "TFLOP/s",
                    "frac": round(achieved / tpeak, 5), "traffic": None,
                    "algorithmic_flops_per_launch": flops,
                    "kernel_depth": kdepth,
                    "issued_tflops": round(2.0 * n * n * kdepth / (per_launch_ms / 1e3) / 1e12,
                                           2),
                    "launches_per_step": cnt // max(args.steps, 1),
                    "ms_per_launch": round(per_launch_ms, 4),
                    "kernel_share_of_stage_time": round(tot_ms / total_stage, 4),
                    "note": HD_KERNEL_NOTE if d <= 64 and knn_k + 1 <= 32 else
                    "mma.sync m16n8k16 bf16, two-term split (hi, lo): depth 3 x padded d"}
    elif dom:
        kq = (max(knn_k, ms) if kruskal else ms) + 1
        comps = stages.get("boruvka_components")
        bor_ms = sum(stages.get(k, [0.0])[0] for k in
                     ("boruvka_search", "boruvka_merge", "boruvka_nodes")) / args.steps
        if comps and comps[1] > 0 and bor_ms > 0 and not kruskal:
            # the Boruvka stage: every round's seed, search, merge and node
            # passes, against the per-round formula summed over the rounds
            rounds_f = comps[1] / args.steps
            total = (rounds_f * boruvka_round_bytes(n, kq, d, 0)
                     + 8 * comps[0] / args.steps)
            achieved = total / (bor_ms / 1e3) / 1e9
            tpp = traffic_per_point("boruvka_stage")
            s_tot, s_cnt = kernel_stages.get("search_kernel", (0.0, 0))
            s_alg = algorithmic_bytes("search_kernel", n, kq, 4 if d <= 4 else 8)
            roofline = {
                "bound": "hbm", "kernel": "boruvka_round (seed + search + merge + node passes)",
                "achieved": round(achieved, 2), "peak": peak, "peak_source": peak_src,
                "unit": "GB/s", "frac": round(achieved / peak, 5),
                "traffic": round(tpp * n * rounds_f) if tpp is not None else None,
                "traffic_note": "DRAM bytes of all kernels of the Boruvka rounds, per fit, "
                                "scaled from an ncu capture on a 4M-point fit",
                "algorithmic_bytes_per_fit": round(total),
                "formula": "sum over rounds of n*k*12 + n*(4d+16) + 8*C_r + 8n",
                "rounds_per_step": round(rounds_f, 2),
                "components_per_step": round(comps[0] / args.steps),
                "ms_per_step": round(bor_ms, 4),
                "ms_per_round": round(bor_ms / max(rounds_f, 1), 4),
                "stage_share": round(bor_ms * args.steps / total_stage, 4),
                "search_kernel_narrow": None if not s_cnt else {
                    "algorithmic_bytes_per_launch": s_alg,
                    "ms_per_launch": round(s_tot / s_cnt, 4),
                    "achieved": round(s_alg / (s_tot / s_cnt / 1e3) / 1e9, 2),
                    "launches_per_step": s_cnt // max(args.steps, 1),
                    "traffic": (round(traffic_per_point("search_kernel") * n)
                                if traffic_per_point("search_kernel") else None)},
            }
        else:
            tot_ms, cnt = kernel_stages[dom]
            per_launch_ms = tot_ms / cnt
            alg = algorithmic_bytes(dom, n, kq, 4 if d <= 4 else 8)
            achieved = alg / (per_launch_ms / 1e3) / 1e9
            # the ncu traffic per point was measured for the Boruvka fit's kNN (k = 16)
            tpp = None if kruskal else traffic_per_point(dom)
            traffic = round(tpp * n) if tpp is not None else None
            roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 2),
                        "peak": peak, "peak_source": peak_src, "unit": "GB/s",
                        "frac": round(achieved / peak, 5), "traffic": traffic,
                        "algorithmic_bytes_per_launch": alg,
                        "launches_per_step": cnt // max(args.steps, 1),
                        "ms_per_launch": round(per_launch_ms, 4),
                        "kernel_share_of_stage_time": round(tot_ms / total_stage, 4)}
        knn_ms = stages.get("knn", [0.0])[0] / args.steps
        if knn_ms > 0 and not kruskal:
            kb = knn_stage_bytes(n, kq, d)
            roofline["knn_stage"] = {
                "algorithmic_bytes_per_fit": kb, "ms_per_step": round(knn_ms, 4),
                "achieved": round(kb / (knn_ms / 1e3) / 1e9, 2),
                "frac": round(kb / (knn_ms / 1e3) / 1e9 / peak, 5),
                "formula": "n*4d + n*(4d+8)*2 + n*k*8 + n*4",
                "note": "issue-bound (list insertion and box tests), not HBM-bound"}

    # e2e through the public estimator, pinned host input, outputs to host
    e2e = None
    if not args.no_e2e:
        Xp = torch.from_numpy(Xh).pin_memory()
        if pre:  # the caller's scipy graph on the host
            import scipy.sparse

            Xp = scipy.sparse.csr_matrix(
                (g_data.cpu().numpy(), g_cols.cpu().numpy(),
                 np.arange(0, nnz + 1, WORKLOAD["graph_k"], dtype=np.int64)), shape=(n, n))
            est = HDBSCAN(min_cluster_size=mcs, min_samples=ms, metric="precomputed",
                          algorithm=WORKLOAD["algorithm"])
        elif kruskal:
            est = HDBSCAN(min_cluster_size=mcs, min_samples=ms, algorithm="kruskal",
                          knn_k=knn_k)
        else:
            est = HDBSCAN(min_cluster_size=mcs, min_samples=ms)
        # warm-up fits: the estimator holds one fit's outputs while the next
        # runs, so the pinned host buffers reach their steady state (two sets
        # in PyTorch's caching host allocator) before the timed fits
        for _ in range(max(args.warmup, 2)):
            est.fit(Xp)
        barrier()
        t0 = time.perf_counter()
        step_s = []
        for _ in range(args.steps):
            ts = time.perf_counter()
            est.fit(Xp)  # returns with the outputs on the host (it synchronises)
            step_s.append(time.perf_counter() - ts)
        barrier()
        e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps,
                               torch.device("cuda", local))
        rows_out = est._condensed_tree.shape[0]
        # labels i64, probabilities f32, sorted MST (n-1) x 3 f64, linkage (n-1) x 4 f64,
        # condensed tree 28 B/row, neighbours n x ms i32, core distances f32 (Kruskal: f64)
        d2h = (n * 8 + n * 4 + (n - 1) * 24 + (n - 1) * 32 + rows_out * 28 + n * ms * 4
               + n * (8 if (kruskal or pre or kgraph) else 4))
        # CSR graph: row pointers (int64), column indices (int32), weights (float64)
        h2d = 8 * (n + 1) + 12 * n * WORKLOAD["graph_k"] if pre else n * d * 4
        e2e = {"value": round(n * world / e2e_s, 1), "unit": "points/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "s_per_step": round(e2e_s, 4),
               "step_ms": {"min": round(1e3 * min(step_s), 2),
                           "median": round(1e3 * float(np.median(step_s)), 2),
                           "max": round(1e3 * max(step_s), 2)}}

    # the learned-radius arm (after the e2e arm, so that its training
    # leaves no trace in the end-to-end timing): the same fit with the kNN radius proposed by a
    # network trained on a 2M-point draw of the generator with another seed
    # (training untimed), labels checked identical to the plain fit's
    learned = None
    if not (pre or kruskal or kgraph or args.no_radius):
        from fast_hdbscan_gb300.radius import RadiusModel

        step()  # the plain fit's outputs, to compare against
        lab_plain, prob_plain = labels.clone(), probs.clone()
        t0 = time.perf_counter()
        model = RadiusModel.train(make_data(2_000_000, WORKLOAD["seed"] + 100), min_samples=ms,
                                  steps=1500, batch=4096, seed=7)
        train_s = time.perf_counter() - t0
        with model.active():
            for _ in range(args.warmup):
                step()
            barrier()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                step()
            e1.record(stream)
            barrier()
            fallbacks = model.last_fallbacks()
        ms_learned = max_over_ranks(e0.elapsed_time(e1) / args.steps,
                                    torch.device("cuda", local))
        learned = {"value": round(n * world / (ms_learned / 1e3), 1), "unit": "points/s",
                   "ms_per_step": round(ms_learned, 3),
                   "vs_plain": round(ms_step_max / ms_learned, 4),
                   "fallback_rate": round(fallbacks / n, 6), "margin": round(model.margin, 4),
                   "train_s": round(train_s, 3), "train_points": 2_000_000,
                   "train_rmse_log": round(model.train_rmse, 4),
                   "identical_labels": bool(torch.equal(labels, lab_plain)
                                            and torch.equal(probs, prob_plain))}

    # the reference tie mode (reproducible=True): the same fit making the
    # reference's own choices among equal-weight edges (its KD-tree built
    # exactly on the GPU, a tie walk per component and round); the tests
    # check its output against the reference's rules bit for bit
    ref_ties = None
    if not (pre or kruskal or kgraph or args.no_ref_ties):
        old_rule = lib.fhg_set_tie_rule(1)
        try:
            for _ in range(args.warmup):
                step()
            barrier()
            lib.fhg_profile_report(None, 0)
            lib.fhg_profile_enable(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                step()
            e1.record(stream)
            barrier()
            lib.fhg_profile_enable(0)
            rbuf = ctypes.create_string_buffer(1 << 16)
            lib.fhg_profile_report(rbuf, len(rbuf))
            rst = json.loads(rbuf.value.decode() or "{}")
        finally:
            lib.fhg_set_tie_rule(old_rule)
        ms_ref = max_over_ranks(e0.elapsed_time(e1) / args.steps, torch.device("cuda", local))
        ref_ties = {"value": round(n * world / (ms_ref / 1e3), 1), "unit": "points/s",
                    "ms_per_step": round(ms_ref, 3), "vs_plain": round(ms_step_max / ms_ref, 4),
                    "stages_ms_per_step": {k: round(v[0] / args.steps, 3)
                                           for k, v in rst.items()
                                           if k.startswith(("ref_tree", "ref_knn", "tie_walk", "boruvka"))}}

    # many independent fits of uneven size in one call (the batched
    # executor), on the benchmark family's 4,096-instance batch
    batched = None
    if rank == 0 and not (pre or kruskal or kgraph or args.no_batched):
        batched = batched_summary()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(_cpu_sample_n(args))

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 1), "unit": "points/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step_max, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator of the benchmark workload)",
            "config": {**{k: v for k, v in WORKLOAD.items() if k != "n"}, "n": n,
                       "parallelism": f"replicas x{world}",
                       "l2": "inputs and working set (several GB) larger than the 129 MB L2"},
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "gpu_launches": int(launches),
            "clocks": clock_info,
            "stages_ms_per_step": {k: round(v[0] / args.steps, 3) for k, v in stages.items()
                                   if k != "boruvka_components"},
            "stage_share": {k: round(v[0] / total_stage, 4) for k, v in stages.items()
                            if k not in nested},
            "boruvka_rounds": rounds,
            "learned_radius": learned,
            "reference_ties": ref_ties,
            "batched": batched,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------- CPU baseline
def _oracle_fit_time(X, nthreads):
    """Wall time of one fit of X by the oracle (the C/OpenMP restatement of
    the reference's path), the reference's tie behaviour (mode 0)."""
    from oracle import oracle as O

    n = X.shape[0]
    t0 = time.perf_counter()
    if WORKLOAD.get("metric") == "precomputed":  # hdbscan.py:306 on the kNN graph
        import scipy.sparse

        gk = WORKLOAD["graph_k"]
        rd, gi = O.tree_query(O.build_kdtree(X), gk + 1, 0, nthreads)
        G = scipy.sparse.csr_matrix(
            (np.sqrt(rd[:, 1:].astype(np.float64)).ravel(), gi[:, 1:].ravel(),
             np.arange(0, n * gk + 1, gk)), shape=(n, n))
        t0 = time.perf_counter()
        mst, _, _ = O.precomputed_kruskal(G, WORKLOAD["min_samples"])
        O.clusters_from_spanning_tree(mst, WORKLOAD["min_cluster_size"])
    elif WORKLOAD.get("algorithm") == "knn_graph":  # hdbscan.py:446 -> nndescent.py:179
        mst, _, _ = O.kruskal_knn(O.build_kdtree(X), WORKLOAD["min_samples"], WORKLOAD["knn_k"],
                                  mode=0, nthreads=nthreads)
        O.clusters_from_spanning_tree(mst, WORKLOAD["min_cluster_size"])
    elif WORKLOAD.get("algorithm") == "kruskal":  # hdbscan.py:306 with algorithm="kruskal"
        mst, _, _ = O.kruskal_knn(O.build_kdtree(X), WORKLOAD["min_samples"], WORKLOAD["knn_k"],
                                  mode=0, nthreads=nthreads)
        O.clusters_from_spanning_tree(mst, WORKLOAD["min_cluster_size"])
    else:
        O.fit(X, WORKLOAD["min_samples"], WORKLOAD["min_cluster_size"], mode=0,
              nthreads=nthreads)
    return time.perf_counter() - t0


def _cpu_sample_n(args):
    """Points per CPU fit: the workload's own size unless a workload's
    brute-force reference path (the kNN-graph route, O(n^2)) needs a sample."""
    if args.cpu_sample:
        return args.cpu_sample
    return WORKLOAD.get("cpu_sample", args.n)


def cpu_baseline_sample(n_sample):
    cores = os.cpu_count() or 1
    X = make_data(n_sample, WORKLOAD["seed"])
    t = _oracle_fit_time(X, cores)
    whole = n_sample == WORKLOAD["n"]
    return {"value": round(n_sample / t, 1), "unit": "points/s", "cores": cores, "kind": "port",
            "sample": (f"the full workload ({n_sample} points, the same seeded input), one fit, "
                       f"{t:.2f} s" if whole else
                       f"{n_sample} points of the same generator, one fit, {t:.2f} s"),
            "same_config": whole,
            "what": "C/OpenMP restatement of the reference fit path (oracle/), reference "
                    "tie mode; numba is not installed on this machine"}


def run_reference(args):
    """The reference's algorithm (the oracle's restatement, numba being absent
    on the GPU host) on all host cores.  Each timed step fits the workload's
    own input (the same seeded points as the GPU arm).  The untimed warm-up
    steps fit a 1M-point draw of the generator: a compiled CPU path has no JIT
    to warm, and a full-size warm-up would only double the run time."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    n_fit = _cpu_sample_n(args)
    X = make_data(n_fit, WORKLOAD["seed"])
    Xw = make_data(min(n_fit, 1_000_000), WORKLOAD["seed"] + 1)
    for _ in range(args.warmup):
        _oracle_fit_time(Xw, cores)
    times = [_oracle_fit_time(X, cores) for _ in range(args.steps)]
    s = sum(times) / len(times)
    value = n_fit / s
    whole = n_fit == WORKLOAD["n"]
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": "points/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(s * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator of the benchmark workload)",
        "config": {**{k: v for k, v in WORKLOAD.items() if k != "n"}, "n": n_fit,
                   **({} if whole else {"sample_of_n": WORKLOAD["n"]})},
        "cpu_baseline": {"value": round(value, 1), "unit": "points/s", "cores": cores,
                         "kind": "port", "same_config": whole,
                         "sample": ("the full workload per step (the GPU arm's seeded input); "
                                    "warm-up steps on a 1M-point draw" if whole else
                                    f"{n_fit}-point sample of the workload per step")},
        "e2e": {"value": round(value, 1), "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------ batched independent fits
def batched_summary(instances=4096):
    """One timed pass of fit_many over the 4,096-instance batch (sizes
    log-uniform 200..200k, d 2..8, min_samples in {5, 10, 20},
    min_cluster_size = max(10, n / 100)) after a warm-up on its first 64
    instances; host arrays in, host labels and probabilities out."""
    import torch
    from fast_hdbscan_gb300 import synthetic
    from fast_hdbscan_gb300.batch import fit_many

    inst = synthetic.batch_instances(instances, seed=4)
    Xs = [X for X, _, _ in inst]
    ms = [m for _, m, _ in inst]
    mcs = [c for _, _, c in inst]
    total = sum(X.shape[0] for X in Xs)
    fit_many(Xs[:64], ms[:64], mcs[:64], workers=16)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fit_many(Xs, ms, mcs, workers=16)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    return {"value": round(len(Xs) / t, 2), "unit": "instances/s",
            "points_per_s": round(total / t, 1), "s_total": round(t, 3),
            "instances": len(Xs), "points": total, "workers": 16,
            "workload": "batched_uneven_instances (bench.py --workload batched for the full "
                        "report)"}


def run_batched(args):
    """Many independent fits of uneven size (log-uniform 200..200k points, d
    2..8, 3-12 Gaussian blobs + 5 % noise, min_samples in {5, 10, 20},
    min_cluster_size = max(10, n/100)): instances/s and points/s through
    fit_many (worker streams), beside the same instances one at a time and
    the CPU oracle on a bounded sample of them."""
    import torch
    from fast_hdbscan_gb300 import build as engine_build
    from fast_hdbscan_gb300.batch import fit_many

    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    from fast_hdbscan_gb300 import synthetic

    engine_build.build()
    inst = synthetic.batch_instances(args.instances, seed=4)
    Xs = [X for X, _, _ in inst]
    ms = [m for _, m, _ in inst]
    mcs = [c for _, _, c in inst]
    total = sum(X.shape[0] for X in Xs)
    warm = min(64, len(Xs))
    fit_many(Xs[:warm], ms[:warm], mcs[:warm], workers=16)

    def timed(workers):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fit_many(Xs, ms, mcs, workers=workers)
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    from fast_hdbscan_gb300.batch import autotune_workers

    best, tune_times = autotune_workers(Xs, ms, mcs, sample=256)
    with ClockSampler(local) as clocks:
        t_batch = timed(best)
    t_16 = timed(16)
    t_one = timed(1)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O

        cores = os.cpu_count() or 1
        sample = list(range(0, len(Xs), max(1, len(Xs) // 48)))
        t0 = time.perf_counter()
        for i in sample:
            O.fit(Xs[i], ms[i], mcs[i], mode=0, nthreads=cores)
        tc = time.perf_counter() - t0
        pts = sum(Xs[i].shape[0] for i in sample)
        cpu = {"value": round(len(sample) / tc, 2), "unit": "instances/s", "cores": cores,
               "kind": "port", "points_per_s": round(pts / tc, 1),
               "sample": f"{len(sample)} of the instances (every {len(Xs) // len(sample)}th), "
                         f"one oracle fit each, {tc:.1f} s"}
    line = {
        "metric": "batched independent HDBSCAN fits, instances/s", "value":
            round(len(Xs) / t_batch, 2), "unit": "instances/s", "n_gpus": 1,
        "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded generator)",
        "config": {"workload": "batched_uneven_instances", "instances": len(Xs),
                   "points": total, "sizes": "log-uniform 200..200000", "d": "2..8",
                   "min_samples": "{5,10,20}", "min_cluster_size": "max(10, n/100)",
                   "workers": best, "workers_source": "autotune_workers on 256 sampled "
                   "instances", "autotune_s": {str(k): round(v, 3) for k, v in tune_times.items()}},
        "points_per_s": round(total / t_batch, 1), "s_total": round(t_batch, 3),
        "one_at_a_time": {"value": round(len(Xs) / t_one, 2), "unit": "instances/s",
                          "s_total": round(t_one, 3)},
        "speedup_vs_one_at_a_time": round(t_one / t_batch, 2),
        "workers_16": {"value": round(len(Xs) / t_16, 2), "unit": "instances/s",
                       "s_total": round(t_16, 3)},
        "cpu_baseline": cpu, "clocks": clocks.summary(),
        "e2e_note": "host arrays in, host labels/probabilities out (fit_many)",
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.workload in OTHER_WORKLOADS:
        WORKLOAD.clear()
        WORKLOAD.update(OTHER_WORKLOADS[args.workload])
        if args.n == 10_000_000:
            args.n = WORKLOAD["n"]
        global METRIC
        METRIC = f"HDBSCAN fit points/s at {WORKLOAD['n'] // 1_000_000}M x {WORKLOAD['d']}-D"
        if WORKLOAD.get("metric") == "precomputed":
            METRIC += (f" (metric='precomputed', {WORKLOAD['graph_k']}-NN graph, "
                       f"algorithm='{WORKLOAD['algorithm']}')")
        elif WORKLOAD.get("algorithm") == "kruskal":
            METRIC += f" (algorithm='kruskal', knn_k={WORKLOAD['knn_k']})"
        elif WORKLOAD.get("algorithm") == "knn_graph":
            METRIC += f" (kNN-graph route, exact tensor-core kNN, knn_k={WORKLOAD['knn_k']})"
        args.workload = "fit"
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
