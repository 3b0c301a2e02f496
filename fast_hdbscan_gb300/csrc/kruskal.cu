// kNN-graph Kruskal MST (kruskal.py:950 _kruskal_mst_knn, the
// algorithm="kruskal" back-end with an integer knn_k, without cannot-link
// constraints).
//
// The reference lists the mutual-reachability edges of every point's kNN list
// (kruskal.py:456), drops self-loops and infinite weights, orders them by a
// stable argsort of their float64 weights and runs Kruskal's union-find; a
// disconnected kNN graph is then joined by +inf bridges between the smallest
// points of its components (kruskal.py:723, precomputed.py:308).
//
// Here: the spatial index's kNN (rows in caller order), one thread per edge
// for the weights, a stable LSD radix sort of the valid edges, and -- in place
// of the sequential scan -- Boruvka rounds over the sorted ranks: every
// component takes its lowest-rank outgoing edge, the picked edges are hooked
// with a lock-free union-find and edges inside one component leave the active
// list.  Ranks are distinct, so the forest is the one Kruskal accepts (the
// minimum spanning forest of a strict order is unique); compacting the picked
// ranks gives Kruskal's acceptance order.  The union-find keeps every root the
// smallest point of its component, so the bridges join the roots in index
// order.
//
// Every float64 weight is a monotone image of one float32 value -- without
// sample weights sqrt(double(max(core2_i, core2_j, rdist_ij))) (core2 the
// squared core distance, a kNN rdist entry), with them
// double(max(core_i, core_j, sqrtf(rdist_ij))) -- and distinct float32 values
// give distinct weights (a correctly rounded double square root keeps the
// strict order of float32 inputs), so the sort runs on the 32-bit pattern of
// that value (non-negative floats order like their bits).
#include <memory>

#include "highd.cuh"
#include "index.cuh"
#include "mst.cuh"
#include "primitives.cuh"
#include "uf.cuh"

namespace fhg {
namespace {

#define LAUNCH(kernel, count, ...)                                        \
    do {                                                                  \
        if ((count) > 0) {                                                \
            ::fhg::note_launch();                                         \
            kernel<<<grid_for((count), 256), 256, 0, s>>>(__VA_ARGS__);   \
            FHG_CUDA(cudaGetLastError());                                 \
        }                                                                 \
    } while (0)

// kruskal.py:995-1015: float64 core distances from the kNN lists (rows of kq,
// the point itself first; min_samples <= 1: zero) and the float32 value the
// edge keys take the maximum of (the squared core distance).
__global__ void kr_core_kernel(int64_t n, int kq, int ms, const float* __restrict__ rd,
                               double* __restrict__ core, float* __restrict__ ck) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float c2 = ms > 1 ? rd[i * kq + ms] : 0.0f;
    core[i] = ms > 1 ? __dsqrt_rn((double)c2) : 0.0;
    ck[i] = c2;
}
// kruskal.py:981-990 with boruvka.py:528 sample_weight_core_distance: the
// first list position at which the running float64 weight (the point's own
// first) reaches min_samples; index -1 (padding) reads the last weight.  The
// distances are the float32 square roots the reference's tree query returns.
__global__ void kr_core_w_kernel(int64_t n, int kq, int ms, const float* __restrict__ rd,
                                 const int32_t* __restrict__ ix, const float* __restrict__ w,
                                 double* __restrict__ core, float* __restrict__ ck) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double total = 0.0;
    int j = 0;
    while (total < (double)ms && j < kq) {
        const int32_t q = ix[i * kq + j];
        total += (double)w[q >= 0 ? q : n - 1];
        ++j;
    }
    const float c = __fsqrt_rn(rd[i * kq + (j > 0 ? j - 1 : 0)]);
    core[i] = (double)c;
    ck[i] = c;
}
// kruskal.py:456 _build_mrd_edges_knn and the filter of :1022, as each edge's
// float32 key.  Edge e is the (e % kk)-th neighbour of point e / kk
// (kk = kq - 1).
__global__ void kr_edges_kernel(int64_t n, int kq, int weighted, const float* __restrict__ rd,
                                const int32_t* __restrict__ ix, const float* __restrict__ ck,
                                uint32_t* __restrict__ key, uint32_t* __restrict__ flag) {
    const int64_t kk = kq - 1;
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * kk) return;
    const int64_t i = e / kk, jp = e - i * kk;
    const int32_t j = ix[i * kq + jp + 1];
    float v = INFINITY;
    if (j >= 0) {
        const float r = rd[i * kq + jp + 1];
        v = fmaxf(fmaxf(ck[i], ck[j]), weighted ? __fsqrt_rn(r) : r);
    }
    key[e] = __float_as_uint(v);
    flag[e] = (j >= 0 && j != (int32_t)i && isfinite(v)) ? 1u : 0u;
}
__global__ void kr_compact_kernel(int64_t E, const uint32_t* __restrict__ flag,
                                  const uint32_t* __restrict__ pos, const uint32_t* __restrict__ k0,
                                  uint32_t* __restrict__ key, int32_t* __restrict__ eid) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E || !flag[e]) return;
    key[pos[e]] = k0[e];
    eid[pos[e]] = (int32_t)e;
}
// Endpoints of every sorted edge, and the initial active list (all ranks).
__global__ void kr_ends_kernel(int64_t m, int kq, const int32_t* __restrict__ eid,
                               const int32_t* __restrict__ ix, int2* __restrict__ uv,
                               int32_t* __restrict__ act, int2* __restrict__ act_uv) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    const int64_t kk = kq - 1, e = eid[r], i = e / kk;
    const int2 p = make_int2((int32_t)i, ix[i * kq + (e - i * kk) + 1]);
    uv[r] = p;
    act[r] = (int32_t)r;
    act_uv[r] = p;
}
__global__ void kr_iota_kernel(int32_t* a, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = (int32_t)i;
}
__global__ void kr_fill_u32_kernel(uint32_t* a, int64_t n, uint32_t v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}
// One Boruvka round, step 1: every component's lowest outgoing rank.  Active
// ranks come in increasing order, so a component's best is mostly set by its
// first edge and later ones only read it.
__global__ void kr_best_kernel(int64_t na, const int32_t* __restrict__ act,
                               const int2* __restrict__ act_uv, int32_t* par,
                               uint32_t* __restrict__ best) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= na) return;
    const uint32_t r = (uint32_t)act[t];
    const int2 p = act_uv[t];
    const int32_t cu = uf_find(par, p.x), cv = uf_find(par, p.y);
    if (cu == cv) return;
    if (r < *(volatile uint32_t*)&best[cu]) atomicMin(&best[cu], r);
    if (r < *(volatile uint32_t*)&best[cv]) atomicMin(&best[cv], r);
}
// Step 2 (no union yet, so the roots are those of step 1): an edge picked by
// either of its components is marked with the round.
__global__ void kr_pick_kernel(int64_t na, const int32_t* __restrict__ act,
                               const int2* __restrict__ act_uv, int32_t* par,
                               const uint32_t* __restrict__ best, int32_t* __restrict__ mark,
                               int round, uint32_t* __restrict__ picked) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= na) return;
    const uint32_t r = (uint32_t)act[t];
    const int2 p = act_uv[t];
    const int32_t cu = uf_find(par, p.x), cv = uf_find(par, p.y);
    if (cu != cv && (best[cu] == r || best[cv] == r)) {
        mark[r] = round;
        atomicAdd(picked, 1u);
    }
}
// Step 3: hook the picked edges.
__global__ void kr_hook_kernel(int64_t na, const int32_t* __restrict__ act,
                               const int2* __restrict__ act_uv, int32_t* par,
                               const int32_t* __restrict__ mark, int round) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= na) return;
    if (mark[act[t]] != round) return;
    const int2 p = act_uv[t];
    uf_union(par, p.x, p.y);
}
// Step 4: edges now inside one component leave the list.
__global__ void kr_keep_kernel(int64_t na, const int2* __restrict__ act_uv, int32_t* par,
                               uint32_t* __restrict__ keep) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= na) return;
    const int2 p = act_uv[t];
    keep[t] = uf_find(par, p.x) != uf_find(par, p.y) ? 1u : 0u;
}
__global__ void kr_scatter_active_kernel(int64_t na, const int32_t* __restrict__ act,
                                         const int2* __restrict__ act_uv,
                                         const uint32_t* __restrict__ keep,
                                         const uint32_t* __restrict__ pos,
                                         int32_t* __restrict__ act2, int2* __restrict__ act_uv2) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= na || !keep[t]) return;
    act2[pos[t]] = act[t];
    act_uv2[pos[t]] = act_uv[t];
}
__global__ void kr_mark_flags_kernel(int64_t m, const int32_t* __restrict__ mark,
                                     uint32_t* __restrict__ flag) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < m) flag[r] = mark[r] > 0 ? 1u : 0u;
}
// kruskal.py:104-107: picked edges in rank order as (row point, neighbour,
// float64 weight); the weight is the rank's float32 key (kNN graph) or its
// float64 weight.
__global__ void kr_emit_kernel(int64_t m, int weighted, const uint32_t* __restrict__ flag,
                               const uint32_t* __restrict__ pos, const int2* __restrict__ uv,
                               const uint32_t* __restrict__ key, const double* __restrict__ w64,
                               double* __restrict__ edges) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m || !flag[r]) return;
    const int64_t o = pos[r];
    edges[3 * o + 0] = (double)uv[r].x;
    edges[3 * o + 1] = (double)uv[r].y;
    if (w64) {
        edges[3 * o + 2] = w64[r];
    } else {
        const float v = __uint_as_float(key[r]);
        edges[3 * o + 2] = weighted ? (double)v : __dsqrt_rn((double)v);
    }
}
__global__ void kr_root_flags_kernel(int64_t n, int32_t* par, uint32_t* __restrict__ flag) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flag[i] = uf_find(par, (int32_t)i) == (int32_t)i ? 1u : 0u;
}
// kruskal.py:723 / precomputed.py:308: +inf bridges between consecutive
// component representatives (the roots, each its component's smallest point).
__global__ void kr_bridge_kernel(int64_t n, int64_t nc, const uint32_t* __restrict__ flag,
                                 const uint32_t* __restrict__ pos, int64_t base,
                                 double* __restrict__ edges) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    const int64_t c = pos[i];  // this root's place among the roots
    if (c > 0) {               // bridge c - 1 ends here
        edges[3 * (base + c - 1) + 1] = (double)i;
        edges[3 * (base + c - 1) + 2] = INFINITY;
    }
    if (c + 1 < nc) edges[3 * (base + c) + 0] = (double)i;  // bridge c starts here
}
__global__ void kr_neighbors_kernel(int64_t n, int kq, int cols, const int32_t* __restrict__ ix,
                                    int32_t* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * cols) return;
    const int64_t i = t / cols, c = t - i * cols;
    out[t] = ix[i * kq + c + 1];
}

}  // namespace

int kruskal_knn_mst(const fhg_index& index, int min_samples, int query_k, const float* weights,
                    double* edges, int32_t* neighbors, double* core, int64_t* n_components,
                    cudaStream_t s) {
    return kruskal_mst_of_lists(index.n, min_samples, query_k, weights, &index, nullptr, 0,
                                edges, neighbors, core, n_components, s);
}

int kruskal_mst_of_lists(int64_t n, int min_samples, int query_k, const float* weights,
                         const fhg_index* index, const float* X, int d, double* edges,
                         int32_t* neighbors, double* core, int64_t* n_components,
                         cudaStream_t s) {
    const int kq = query_k;
    const int64_t kk = kq - 1;
    // the spatial index's kNN takes lists of up to kKnnMaxK; the
    // high-dimensional kNN graph is used here with lists of up to 64
    const int kq_max = index ? kKnnMaxK : 64;
    if (kq < 2 || kq > kq_max) {
        set_error("kruskal: the kNN query size must be in [2, %d] (got %d)", kq_max, kq);
        return kq > kq_max ? FHG_ERR_UNSUPPORTED : FHG_ERR_INVALID;
    }
    if (n * kk > 0x7fffffffLL) {
        set_error("kruskal: %lld kNN edges exceed the int32 edge index", (long long)(n * kk));
        return FHG_ERR_UNSUPPORTED;
    }
    if (!weights && min_samples > 1 && min_samples >= kq) {
        set_error("kruskal: the kNN query size %d must exceed min_samples %d", kq, min_samples);
        return FHG_ERR_INVALID;
    }
    *n_components = n > 0 ? 1 : 0;
    if (n < 2) {
        if (n == 1) FHG_CUDA(cudaMemsetAsync(core, 0, sizeof(double), s));
        return FHG_OK;
    }
    Stage stage(s, "kruskal_knn");
    Workspace ws(s);
    float *rd, *ck;
    int32_t* ix;
    FHG_TRY(ws.alloc(&rd, (size_t)(n * kq)));
    FHG_TRY(ws.alloc(&ix, (size_t)(n * kq)));
    FHG_TRY(ws.alloc(&ck, (size_t)n));
    if (index) FHG_TRY(index_knn(*index, kq, nullptr, nullptr, rd, ix, s));
    else FHG_TRY(highd_knn(X, n, d, kq, rd, ix, nullptr, s));
    if (weights) LAUNCH(kr_core_w_kernel, n, n, kq, min_samples, rd, ix, weights, core, ck);
    else LAUNCH(kr_core_kernel, n, n, kq, min_samples, rd, core, ck);
    if (neighbors) {
        const int cols = weights ? kq - 1 : (min_samples > 1 ? min_samples : 1);
        LAUNCH(kr_neighbors_kernel, n * cols, n, kq, cols, ix, neighbors);
    }

    // ---- valid edges, stably sorted by weight
    std::unique_ptr<Stage> sub(new Stage(s, "kruskal_edges"));
    const int64_t E = n * kk;
    uint32_t *k0, *flag, *pos, *cnt;
    FHG_TRY(ws.alloc(&k0, (size_t)E));
    FHG_TRY(ws.alloc(&flag, (size_t)E));
    FHG_TRY(ws.alloc(&pos, (size_t)E));
    FHG_TRY(ws.alloc(&cnt, 2));
    LAUNCH(kr_edges_kernel, E, n, kq, weights ? 1 : 0, rd, ix, ck, k0, flag);
    FHG_TRY(scan_exclusive_u32(ws, flag, pos, E, cnt));
    uint32_t h_m = 0;
    FHG_CUDA(cudaMemcpyAsync(&h_m, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    const int64_t m = h_m;
    const size_t mm = (size_t)(m > 0 ? m : 1);
    uint32_t* key;
    int32_t* eid;
    FHG_TRY(ws.alloc(&key, mm));
    FHG_TRY(ws.alloc(&eid, mm));
    LAUNCH(kr_compact_kernel, E, E, flag, pos, k0, key, eid);
    sub.reset(new Stage(s, "kruskal_sort"));
    if (m > 1) {
        Workspace tmp(s);
        FHG_TRY(radix_sort_u32(tmp, key, eid, m, 0, 32));
    }

    sub.reset();
    FHG_TRY(sorted_forest_edges(ws, n, m, kq, eid, ix, nullptr, key, weights ? 1 : 0, edges,
                                n_components));
    return FHG_OK;
}

int sorted_forest_edges(Workspace& ws, int64_t n, int64_t m, int kq, const int32_t* eid,
                        const int32_t* ix, const int2* uv_in, const uint32_t* key32,
                        int key_weighted, double* edges, int64_t* n_components,
                        const double* w64) {
    cudaStream_t s = ws.stream();
    const size_t mm = (size_t)(m > 0 ? m : 1);
    // ---- minimum spanning forest: Boruvka rounds over the ranks
    std::unique_ptr<Stage> sub(new Stage(s, "kruskal_forest"));
    int32_t *par, *act, *act2, *mark;
    int2 *uv, *act_uv, *act_uv2;
    uint32_t *best, *keep, *picked, *pos, *cnt;
    FHG_TRY(ws.alloc(&par, (size_t)n));
    FHG_TRY(ws.alloc(&best, (size_t)n));
    FHG_TRY(ws.alloc(&uv, mm));
    FHG_TRY(ws.alloc(&act, mm));
    FHG_TRY(ws.alloc(&act2, mm));
    FHG_TRY(ws.alloc(&act_uv, mm));
    FHG_TRY(ws.alloc(&act_uv2, mm));
    FHG_TRY(ws.alloc(&keep, mm));
    FHG_TRY(ws.alloc(&pos, mm));
    FHG_TRY(ws.alloc(&mark, mm));
    FHG_TRY(ws.alloc(&picked, 1));
    FHG_TRY(ws.alloc(&cnt, 2));
    LAUNCH(kr_iota_kernel, n, par, n);
    if (uv_in) {
        FHG_CUDA(cudaMemcpyAsync(uv, uv_in, sizeof(int2) * m, cudaMemcpyDeviceToDevice, s));
        FHG_CUDA(cudaMemcpyAsync(act_uv, uv_in, sizeof(int2) * m, cudaMemcpyDeviceToDevice, s));
        LAUNCH(kr_iota_kernel, m, act, m);
    } else {
        LAUNCH(kr_ends_kernel, m, m, kq, eid, ix, uv, act, act_uv);
    }
    if (m > 0) FHG_CUDA(cudaMemsetAsync(mark, 0, sizeof(int32_t) * m, s));
    int64_t na = m;
    for (int round = 1; na > 0; ++round) {
        if (round > 64) {  // each round at least halves the components
            set_error("kruskal: the spanning forest did not converge");
            return FHG_ERR_NO_CONVERGENCE;
        }
        LAUNCH(kr_fill_u32_kernel, n, best, n, 0xffffffffu);
        FHG_CUDA(cudaMemsetAsync(picked, 0, sizeof(uint32_t), s));
        LAUNCH(kr_best_kernel, na, na, act, act_uv, par, best);
        LAUNCH(kr_pick_kernel, na, na, act, act_uv, par, best, mark, round, picked);
        LAUNCH(kr_hook_kernel, na, na, act, act_uv, par, mark, round);
        LAUNCH(kr_keep_kernel, na, na, act_uv, par, keep);
        FHG_TRY(scan_exclusive_u32(ws, keep, pos, na, cnt));
        LAUNCH(kr_scatter_active_kernel, na, na, act, act_uv, keep, pos, act2, act_uv2);
        uint32_t h[2] = {0, 0};
        FHG_CUDA(cudaMemcpyAsync(&h[0], picked, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        FHG_CUDA(cudaMemcpyAsync(&h[1], cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        FHG_CUDA(cudaStreamSynchronize(s));
        std::swap(act, act2);
        std::swap(act_uv, act_uv2);
        na = h[0] == 0 ? 0 : (int64_t)h[1];
    }

    // ---- the forest in Kruskal's acceptance order, then the bridges
    sub.reset(new Stage(s, "kruskal_emit"));
    uint32_t *flag, *rflag, *rpos;
    FHG_TRY(ws.alloc(&flag, mm));
    FHG_TRY(ws.alloc(&rflag, (size_t)n));
    FHG_TRY(ws.alloc(&rpos, (size_t)n));
    uint32_t h_f = 0, h_c = 0;
    if (m > 0) {
        LAUNCH(kr_mark_flags_kernel, m, m, mark, flag);
        FHG_TRY(scan_exclusive_u32(ws, flag, pos, m, cnt));
        FHG_CUDA(cudaMemcpyAsync(&h_f, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    }
    LAUNCH(kr_root_flags_kernel, n, n, par, rflag);
    FHG_TRY(scan_exclusive_u32(ws, rflag, rpos, n, cnt + 1));
    FHG_CUDA(cudaMemcpyAsync(&h_c, cnt + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    const int64_t nf = h_f, nc = h_c;
    if (nc < 1 || nf + nc != n) {  // a forest over n points in nc components
        set_error("kruskal: %lld forest edges for %lld points in %lld components", (long long)nf,
                  (long long)n, (long long)nc);
        return FHG_ERR_NO_CONVERGENCE;
    }
    if (m > 0) LAUNCH(kr_emit_kernel, m, m, key_weighted, flag, pos, uv, key32, w64, edges);
    if (nc > 1) LAUNCH(kr_bridge_kernel, n, n, nc, rflag, rpos, nf, edges);
    *n_components = nc;
    return FHG_OK;
}

}  // namespace fhg
