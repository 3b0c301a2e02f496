// Cluster selection, labels and membership strengths over the condensed tree.
//
//   stabilities   cluster_trees.py:656 score_condensed_tree_nodes -- float32,
//                 accumulated in row order.  Rows are stably sorted by parent,
//                 then each cluster sums its own rows in order, so every
//                 rounding step matches the reference.
//   EOM           cluster_trees.py:694 eom_recursion / :724
//                 extract_eom_clusters -- evaluated bottom-up over the (small)
//                 cluster tree, one depth level at a time in a single block;
//                 child totals are float64 sums in row order.
//   leaf          cluster_trees.py:369 cluster_tree_leaves.
//   labels        cluster_trees.py:944 get_cluster_label_vector -- the
//                 reference's union-find over unselected rows gives every
//                 point the nearest selected cluster above its row's parent,
//                 computed here by pointer doubling over clusters.
//   probabilities cluster_trees.py:999-1031.
#include "primitives.cuh"
#include "trees.cuh"

namespace fhg {
namespace {

constexpr int kEomThreads = 1024;

__global__ void parent_keys_kernel(int64_t rows, int64_t n, const int32_t* __restrict__ parent,
                                   uint32_t* __restrict__ key, int32_t* __restrict__ cnt) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    int32_t c = parent[r] - (int32_t)n;
    key[r] = (uint32_t)c;
    // rows of one parent come in runs: one atomic per parent per warp
    const unsigned peers = __match_any_sync(__activemask(), c);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&cnt[c], __popc(peers));
}
__global__ void row_of_child_kernel(int64_t rows, int64_t n, const int32_t* __restrict__ child,
                                    int32_t* __restrict__ row_of_cluster,
                                    int32_t* __restrict__ row_of_point) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    int32_t c = child[r];
    if (c >= n) row_of_cluster[c - n] = (int32_t)r;
    else if (row_of_point) row_of_point[c] = (int32_t)r;
}
// lambda * size of every row, in parent-grouped row order (contiguous per
// cluster), so that each cluster's sequential sum below streams its addends.
__global__ void products_kernel(int64_t rows, const int32_t* __restrict__ order,
                                const float* __restrict__ lam, const float* __restrict__ csize,
                                float* __restrict__ prod) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= rows) return;
    int32_t r = order[j];
    prod[j] = __fmul_rn(lam[r], csize[r]);
}
// One thread per cluster: the float32 sum of its rows' products, strictly in
// row order (a float32 sum is not associative, so the order is the result).
// Clusters of kBigRows rows or more are summed by score_big_kernel.
constexpr int32_t kBigRows = 8192;
__device__ __forceinline__ float score_start(int64_t c, const int32_t* __restrict__ row_of_cluster,
                                             const float* __restrict__ lam,
                                             const float* __restrict__ csize) {
    float s = 0.0f;
    if (c > 0) {
        int32_t r = row_of_cluster[c];
        if (r >= 0 && csize[r] > 1.0f) s = __fmul_rn(-lam[r], csize[r]);
    }
    return s;
}
__global__ void score_kernel(int64_t C, const int64_t* __restrict__ start,
                             const int32_t* __restrict__ cnt, const float* __restrict__ prod,
                             const int32_t* __restrict__ row_of_cluster,
                             const float* __restrict__ lam, const float* __restrict__ csize,
                             float* __restrict__ score) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C || cnt[c] >= kBigRows) return;
    float s = score_start(c, row_of_cluster, lam, csize);
    const int64_t b = start[c], e = b + cnt[c];
    int64_t j = b;
    for (; j + 8 <= e; j += 8) {
        float v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = __ldg(prod + j + u);
#pragma unroll
        for (int u = 0; u < 8; ++u) s = __fadd_rn(s, v[u]);
    }
    for (; j < e; ++j) s = __fadd_rn(s, __ldg(prod + j));
    score[c] = s;
}
// One block per cluster of kBigRows rows or more: the same sequential sum by
// one thread, fed from shared memory -- the other warps stage the next chunk
// of products while the current one is summed, so that the chain of
// dependent additions never waits for memory.
constexpr int kScoreThreads = 256;
constexpr int kScoreChunk = 4096;
__global__ void __launch_bounds__(kScoreThreads) score_big_kernel(
    int64_t C, const int64_t* __restrict__ start, const int32_t* __restrict__ cnt,
    const float* __restrict__ prod, const int32_t* __restrict__ row_of_cluster,
    const float* __restrict__ lam, const float* __restrict__ csize, float* __restrict__ score) {
    __shared__ float buf[2][kScoreChunk];
    for (int64_t c = blockIdx.x; c < C; c += gridDim.x) {
        if (cnt[c] < kBigRows) continue;  // uniform over the block
        const int64_t b = start[c], len = cnt[c];
        const int64_t chunks = (len + kScoreChunk - 1) / kScoreChunk;
        for (int64_t j = threadIdx.x; j < kScoreChunk && j < len; j += blockDim.x)
            buf[0][j] = __ldg(prod + b + j);
        __syncthreads();
        float s = threadIdx.x == 0 ? score_start(c, row_of_cluster, lam, csize) : 0.0f;
        for (int64_t k = 0; k < chunks; ++k) {
            const int cur = (int)(k & 1);
            const int64_t base = k * kScoreChunk;
            const int cl = (int)(len - base < kScoreChunk ? len - base : kScoreChunk);
            if (threadIdx.x >= 32) {  // warps 1.. stage chunk k + 1
                const int64_t nb = base + kScoreChunk;
                for (int64_t j = threadIdx.x - 32; j < kScoreChunk && nb + j < len;
                     j += blockDim.x - 32)
                    buf[cur ^ 1][j] = __ldg(prod + b + nb + j);
            } else if (threadIdx.x == 0) {
                const float* v = buf[cur];
                int t = 0;
                for (; t + 8 <= cl; t += 8) {
                    float x[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) x[u] = v[t + u];
#pragma unroll
                    for (int u = 0; u < 8; ++u) s = __fadd_rn(s, x[u]);
                }
                for (; t < cl; ++t) s = __fadd_rn(s, v[t]);
            }
            __syncthreads();  // chunk k summed, chunk k + 1 staged
        }
        if (threadIdx.x == 0) score[c] = s;
    }
}

// Cluster rows (child_size > 1) of every parent, kept in row order.
__global__ void cluster_row_flags_kernel(int64_t rows, const int32_t* __restrict__ order,
                                         const float* __restrict__ csize,
                                         uint32_t* __restrict__ flag) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < rows) flag[j] = csize[order[j]] > 1.0f ? 1u : 0u;
}
__global__ void cluster_row_compact_kernel(int64_t rows, const int32_t* __restrict__ order,
                                           const uint32_t* __restrict__ flag,
                                           const uint32_t* __restrict__ pos,
                                           int32_t* __restrict__ corder) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < rows && flag[j]) corder[pos[j]] = order[j];
}
__global__ void cluster_row_ranges_kernel(int64_t C, int64_t rows, const int64_t* __restrict__ start,
                                          const int32_t* __restrict__ cnt,
                                          const uint32_t* __restrict__ pos,
                                          const uint32_t* __restrict__ total,
                                          int64_t* __restrict__ cstart, int32_t* __restrict__ ccnt) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    int64_t b = start[c], e = b + cnt[c];
    uint32_t pb = b < rows ? pos[b] : *total, pe = e < rows ? pos[e] : *total;
    cstart[c] = pb;
    ccnt[c] = (int32_t)(pe - pb);
}

// Cluster-tree structure: parent cluster (local id) and size of each cluster.
__global__ void cluster_info_kernel(int64_t C, int64_t n, const int32_t* __restrict__ row_of_cluster,
                                    const int32_t* __restrict__ parent,
                                    const float* __restrict__ csize, int32_t* __restrict__ cpar,
                                    float* __restrict__ nsize, int8_t* __restrict__ in_tree) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    if (c == 0) {
        cpar[0] = -1;
        nsize[0] = (float)(n - 1);
        in_tree[0] = 1;
        return;
    }
    int32_t r = row_of_cluster[c];
    bool ok = r >= 0 && csize[r] > 1.0f;
    cpar[c] = ok ? parent[r] - (int32_t)n : -1;
    nsize[c] = ok ? csize[r] : 0.0f;
    in_tree[c] = ok ? 1 : 0;
}

__device__ void block_scan_excl(int32_t* a, int64_t len, int32_t* tmp_total) {
    // simple single-block exclusive scan over global memory (len small)
    __shared__ int32_t part[kEomThreads];
    const int t = threadIdx.x;
    int64_t per = (len + blockDim.x - 1) / blockDim.x;
    int64_t b = t * per, e = b + per < len ? b + per : len;
    int32_t s = 0;
    for (int64_t i = b; i < e; ++i) s += a[i];
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        int32_t run = 0;
        for (int i = 0; i < (int)blockDim.x; ++i) {
            int32_t v = part[i];
            part[i] = run;
            run += v;
        }
        *tmp_total = run;
    }
    __syncthreads();
    int32_t run = part[t];
    for (int64_t i = b; i < e; ++i) {
        int32_t v = a[i];
        a[i] = run;
        run += v;
    }
    __syncthreads();
}

// Single-block EOM.  Scratch arrays are C entries each.
__global__ void __launch_bounds__(kEomThreads) eom_kernel(
    int64_t C, const int32_t* __restrict__ cpar, const float* __restrict__ nsize,
    const int8_t* __restrict__ in_tree, const float* __restrict__ score,
    const int64_t* __restrict__ start, const int32_t* __restrict__ cnt,
    const int32_t* __restrict__ order, const float* __restrict__ csize,
    const int32_t* __restrict__ child, int64_t n, double max_cs, int allow_single,
    int32_t* depth, int32_t* depth2, int32_t* jmp, int32_t* jmp2, int32_t* dcount, int32_t* byd,
    double* ret, int8_t* chose, int8_t* blocked, int32_t* flags, int32_t* sel, int64_t* n_sel) {
    const int t = threadIdx.x;
    __shared__ int32_t s_maxd, s_total;
    // depth of every cluster by pointer doubling (root = 0)
    for (int64_t c = t; c < C; c += blockDim.x) {
        const bool inner = c != 0 && in_tree[c];
        depth[c] = inner ? 1 : 0;
        jmp[c] = inner ? cpar[c] : 0;
    }
    __syncthreads();
    int rounds = 1;
    while (((int64_t)1 << rounds) < C + 1) ++rounds;
    for (int r = 0; r <= rounds; ++r) {
        for (int64_t c = t; c < C; c += blockDim.x) {
            const int32_t a = jmp[c];
            depth2[c] = depth[c] + depth[a];
            jmp2[c] = jmp[a];
        }
        __syncthreads();
        int32_t* tp = depth; depth = depth2; depth2 = tp;
        tp = jmp; jmp = jmp2; jmp2 = tp;
    }
    if (t == 0) s_maxd = 0;
    __syncthreads();
    for (int64_t c = t; c < C; c += blockDim.x)
        if (in_tree[c]) atomicMax(&s_maxd, depth[c]);
    __syncthreads();
    const int32_t maxd = s_maxd;
    // bucket clusters by depth (counting sort)
    for (int64_t d = t; d <= maxd + 1; d += blockDim.x) dcount[d] = 0;
    __syncthreads();
    for (int64_t c = t; c < C; c += blockDim.x)
        if (in_tree[c]) atomicAdd(&dcount[depth[c]], 1);
    __syncthreads();
    block_scan_excl(dcount, maxd + 2, &s_total);
    for (int64_t c = t; c < C; c += blockDim.x)
        if (in_tree[c]) byd[atomicAdd(&dcount[depth[c]], 1)] = (int32_t)c;
    __syncthreads();
    // dcount[d] is now the end of level d; level d spans [end(d-1), end(d))
    for (int32_t d = maxd; d >= 0; --d) {
        const int32_t b = d == 0 ? 0 : dcount[d - 1], e = dcount[d];
        for (int32_t j = b + t; j < e; j += blockDim.x) {
            const int32_t c = byd[j];
            chose[c] = 0;
            if (c == 0 && !allow_single) {
                ret[c] = 0.0;
                continue;
            }
            const double cur = (double)score[c] > 0.0 ? (double)score[c] : 0.0;
            double tot = 0.0;
            for (int64_t q = start[c]; q < start[c] + cnt[c]; ++q) tot += ret[child[order[q]] - n];
            if (tot > cur || (double)nsize[c] > max_cs) {
                ret[c] = tot;
            } else {
                ret[c] = cur;
                chose[c] = 1;
            }
        }
        __syncthreads();
    }
    for (int32_t d = 0; d <= maxd; ++d) {
        const int32_t b = d == 0 ? 0 : dcount[d - 1], e = dcount[d];
        for (int32_t j = b + t; j < e; j += blockDim.x) {
            const int32_t c = byd[j];
            if (c == 0) {
                blocked[c] = 0;
                continue;
            }
            const int32_t p = cpar[c];
            blocked[c] = blocked[p] || (chose[p] && (p != 0 || allow_single));
        }
        __syncthreads();
    }
    // selected ids in label order (the reference dict's insertion order)
    for (int64_t c = t; c < C; c += blockDim.x)
        flags[c] = (in_tree[c] && chose[c] && !blocked[c]) ? 1 : 0;
    __syncthreads();
    block_scan_excl(flags, C, &s_total);
    for (int64_t c = t; c < C; c += blockDim.x) {
        const bool on = in_tree[c] && chose[c] && !blocked[c];
        if (on) sel[flags[c]] = (int32_t)(n + c);
    }
    if (t == 0) *n_sel = s_total;
}

__global__ void __launch_bounds__(kEomThreads) leaf_kernel(
    int64_t C, int64_t n, const int32_t* __restrict__ cpar, const int8_t* __restrict__ in_tree,
    int32_t* __restrict__ flags, int32_t* sel, int64_t* n_sel) {
    const int t = threadIdx.x;
    __shared__ int32_t s_max, s_total;
    if (t == 0) s_max = -1;
    for (int64_t c = t; c < C; c += blockDim.x) flags[c] = 1;
    __syncthreads();
    for (int64_t c = t; c < C; c += blockDim.x)
        if (in_tree[c] && c > 0) {
            flags[cpar[c]] = 0;
            atomicMax(&s_max, (int32_t)c);
        }
    __syncthreads();
    // labels n .. n + max cluster-row child that never appear as a parent
    for (int64_t c = t; c < C; c += blockDim.x)
        if (c > s_max) flags[c] = 0;
    __syncthreads();
    block_scan_excl(flags, C, &s_total);
    for (int64_t c = t; c < C; c += blockDim.x) {
        bool on = c <= s_max && (c + 1 < C ? flags[c + 1] - flags[c] : s_total - flags[c]) == 1;
        if (on) sel[flags[c]] = (int32_t)(n + c);
    }
    if (t == 0) *n_sel = s_max < 0 ? 0 : s_total;
}

// ---------------------------------------------------------------- labels
__global__ void sel_flags_kernel(int64_t n_sel, int64_t n, int64_t C, const int32_t* __restrict__ sel,
                                 int8_t* __restrict__ is_sel, uint32_t* __restrict__ key,
                                 int32_t* __restrict__ val) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_sel) return;
    int32_t c = sel[i] - (int32_t)n;
    if (c >= 0 && c < C) is_sel[c] = 1;
    key[i] = (uint32_t)sel[i];
    val[i] = (int32_t)i;
}
__global__ void label_map_kernel(int64_t n_sel, int64_t n, int64_t C,
                                 const uint32_t* __restrict__ sorted_ids,
                                 int32_t* __restrict__ label_of, int32_t* __restrict__ by_label) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_sel) return;
    int32_t c = (int32_t)sorted_ids[j] - (int32_t)n;
    by_label[j] = c;
    if (c >= 0 && c < C) atomicMax(&label_of[c], (int32_t)j);  // last position wins
}
__global__ void anc_init_kernel(int64_t C, const int32_t* __restrict__ cpar,
                                const int8_t* __restrict__ is_sel, int32_t* __restrict__ jmp,
                                int32_t* __restrict__ sa) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    jmp[c] = c == 0 ? 0 : (cpar[c] < 0 ? 0 : cpar[c]);
    sa[c] = (is_sel[c] || c == 0) ? (int32_t)c : -1;
}
__global__ void anc_step_kernel(int64_t C, const int32_t* __restrict__ jmp,
                                const int32_t* __restrict__ sa, int32_t* __restrict__ jmp2,
                                int32_t* __restrict__ sa2) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    int32_t a = jmp[c];
    jmp2[c] = jmp[a];
    sa2[c] = sa[c] != -1 ? sa[c] : sa[a];
}
__global__ void root_stats_kernel(int64_t rows, int64_t n, const int32_t* __restrict__ parent,
                                  const float* __restrict__ lam, const float* __restrict__ csize,
                                  unsigned int* __restrict__ root_max, unsigned int* __restrict__ death) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    int32_t c = parent[r] - (int32_t)n;
    unsigned int b = __float_as_uint(lam[r]);
    const int lane = threadIdx.x & 31;
    const unsigned act = __activemask();
    // non-negative floats order like their bits; lanes combine first, then one
    // atomic per target per warp
    const unsigned roots = __ballot_sync(act, c == 0);
    if (c == 0) {
        const unsigned m = __reduce_max_sync(roots, b);
        if (lane == __ffs(roots) - 1) atomicMax(root_max, m);
    }
    const bool pt = csize[r] == 1.0f;
    const unsigned pts = __ballot_sync(act, pt);
    if (pt) {
        const unsigned peers = __match_any_sync(pts, c);
        const unsigned m = __reduce_max_sync(peers, b);
        if (lane == __ffs(peers) - 1) atomicMax(&death[c], m);
    }
}
__global__ void point_labels_kernel(int64_t n, int64_t n_distinct, double eps,
                                    const int32_t* __restrict__ row_of_point,
                                    const int32_t* __restrict__ parent,
                                    const float* __restrict__ lam, const int32_t* __restrict__ sa,
                                    const int8_t* __restrict__ is_sel,
                                    const int32_t* __restrict__ label_of,
                                    const unsigned int* __restrict__ root_max,
                                    int64_t* __restrict__ labels, int* __restrict__ err) {
    int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    int32_t r = row_of_point[x];
    int64_t lab = -1;
    if (r >= 0 && lam[r] != 0.0f) {
        int32_t a = sa[parent[r] - (int32_t)n];
        if (a != 0) {
            lab = label_of[a];
        } else if (n_distinct == 1) {
            float lx = lam[r];
            bool take = eps > 0.0 ? ((double)lx >= 1.0 / eps) : (lx >= __uint_as_float(*root_max));
            if (take) {
                if (is_sel[0]) lab = label_of[0];
                else atomicOr(err, 1);
            }
        }
    }
    labels[x] = lab;
}
__global__ void probs_kernel(int64_t rows, int64_t n, const int32_t* __restrict__ child,
                             const float* __restrict__ lam, const int64_t* __restrict__ labels,
                             const int32_t* __restrict__ by_label,
                             const unsigned int* __restrict__ death, float* __restrict__ probs) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    int32_t x = child[r];
    if (x >= n) return;
    int64_t lab = labels[x];
    if (lab < 0) return;
    int32_t c = by_label[lab];
    double ml = (double)__uint_as_float(death[c]);
    float lx = lam[r];
    if (ml == 0.0 || !isfinite(lx)) {
        probs[x] = 1.0f;
    } else {
        double lv = (double)lx < ml ? (double)lx : ml;
        probs[x] = (float)(lv / ml);
    }
}
__global__ void widen_kernel(int64_t C, const int32_t* __restrict__ a, int64_t* __restrict__ b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < C) b[i] = a[i];
}
__global__ void fill_i64_kernel(int64_t* a, int64_t n, int64_t v) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}
__global__ void fill_i32_kernel(int32_t* a, int64_t n, int32_t v) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

#define LAUNCH(kernel, count, ...)                                          \
    do {                                                                    \
        if ((count) > 0) {                                                  \
            ::fhg::note_launch(); \
            kernel<<<grid_for((count), 256), 256, 0, s>>>(__VA_ARGS__);     \
            FHG_CUDA(cudaGetLastError());                                   \
        }                                                                   \
    } while (0)

// Shared preparation: rows grouped by parent, scores, cluster tree.
//
// The scores are one sequential float32 sum per cluster, so a large cluster's
// sum is a long chain of dependent additions on a single thread.  They are
// computed on a side stream while the stream goes on with the work that does
// not read them; join() (also run by the destructor) orders the stream after
// them.  Every buffer the side stream touches belongs to the caller's
// Workspace, which outlives the join.
struct Prepared {
    int64_t C = 0;
    int32_t *order = nullptr, *cnt = nullptr, *row_of_cluster = nullptr, *cpar = nullptr;
    int32_t *corder = nullptr, *ccnt = nullptr;
    int64_t *start = nullptr, *cstart = nullptr;
    float *score = nullptr, *nsize = nullptr, *prod = nullptr;
    int8_t* in_tree = nullptr;
    cudaStream_t main = nullptr, side = nullptr;
    cudaEvent_t done = nullptr;

    Prepared() = default;
    Prepared(const Prepared&) = delete;
    Prepared& operator=(const Prepared&) = delete;
    ~Prepared() { join(); }
    void join() {
        if (!side) return;
        cudaStreamWaitEvent(main, done, 0);
        cudaEventDestroy(done);
        cudaStreamDestroy(side);  // released once its work has completed
        side = nullptr;
        done = nullptr;
    }
};

int prepare(Workspace& ws, const Condensed& ct, Prepared* P) {
    cudaStream_t s = ws.stream();
    const int64_t C = ct.n_clusters, rows = ct.rows, n = ct.n;
    P->C = C;
    uint32_t* key;
    FHG_TRY(ws.alloc(&P->order, (size_t)rows));
    FHG_TRY(ws.alloc(&P->cnt, (size_t)C));
    FHG_TRY(ws.alloc(&P->start, (size_t)C));
    FHG_TRY(ws.alloc(&P->row_of_cluster, (size_t)C));
    FHG_TRY(ws.alloc(&P->score, (size_t)C));
    FHG_TRY(ws.alloc(&P->cpar, (size_t)C));
    FHG_TRY(ws.alloc(&P->nsize, (size_t)C));
    FHG_TRY(ws.alloc(&P->in_tree, (size_t)C));
    FHG_CUDA(cudaMemsetAsync(P->cnt, 0, sizeof(int32_t) * C, s));
    LAUNCH(fill_i32_kernel, C, P->row_of_cluster, C, -1);
    LAUNCH(row_of_child_kernel, rows, rows, n, ct.child, P->row_of_cluster, (int32_t*)nullptr);
    {
        Workspace tmp(s);
        FHG_TRY(tmp.alloc(&key, (size_t)rows));
        int64_t* cnt64;
        FHG_TRY(tmp.alloc(&cnt64, (size_t)C));
        LAUNCH(parent_keys_kernel, rows, rows, n, ct.parent, key, P->cnt);
        FHG_TRY(fill_iota_i32(P->order, rows, s));
        FHG_TRY(radix_sort_u32(tmp, key, P->order, rows, 0, bits_for(C)));
        // start = exclusive scan of counts
        LAUNCH(widen_kernel, C, C, P->cnt, cnt64);
        FHG_TRY(scan_exclusive_i64(tmp, cnt64, P->start, C, nullptr));
    }
    FHG_TRY(ws.alloc(&P->prod, (size_t)rows));
    LAUNCH(products_kernel, rows, rows, P->order, ct.lambda, ct.csize, P->prod);
    {
        // the scores on a side stream (on the stream itself if none can be made)
        cudaStream_t ss = s;
        cudaEvent_t fork = nullptr;
        if (cudaStreamCreateWithFlags(&P->side, cudaStreamNonBlocking) == cudaSuccess) {
            if (cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) == cudaSuccess &&
                cudaEventCreateWithFlags(&P->done, cudaEventDisableTiming) == cudaSuccess &&
                cudaEventRecord(fork, s) == cudaSuccess &&
                cudaStreamWaitEvent(P->side, fork, 0) == cudaSuccess) {
                ss = P->side;
                P->main = s;
            } else {
                if (P->done) cudaEventDestroy(P->done);
                P->done = nullptr;
                cudaStreamDestroy(P->side);
                P->side = nullptr;
            }
            if (fork) cudaEventDestroy(fork);
        } else {
            P->side = nullptr;
            cudaGetLastError();
        }
        if (C > 0) {
            ::fhg::note_launch();
            score_big_kernel<<<(unsigned)(C < 1024 ? C : 1024), kScoreThreads, 0, ss>>>(
                C, P->start, P->cnt, P->prod, P->row_of_cluster, ct.lambda, ct.csize, P->score);
            FHG_CUDA(cudaGetLastError());
            ::fhg::note_launch();
            score_kernel<<<grid_for(C, 256), 256, 0, ss>>>(C, P->start, P->cnt, P->prod,
                                                           P->row_of_cluster, ct.lambda,
                                                           ct.csize, P->score);
            FHG_CUDA(cudaGetLastError());
        }
        if (P->side) FHG_CUDA(cudaEventRecord(P->done, P->side));
    }
    FHG_TRY(ws.alloc(&P->corder, (size_t)rows));
    FHG_TRY(ws.alloc(&P->cstart, (size_t)C));
    FHG_TRY(ws.alloc(&P->ccnt, (size_t)C));
    {
        Workspace tmp(s);
        uint32_t *flag, *pos, *total;
        FHG_TRY(tmp.alloc(&flag, (size_t)rows));
        FHG_TRY(tmp.alloc(&pos, (size_t)rows));
        FHG_TRY(tmp.alloc(&total, 1));
        LAUNCH(cluster_row_flags_kernel, rows, rows, P->order, ct.csize, flag);
        FHG_TRY(scan_exclusive_u32(tmp, flag, pos, rows, total));
        LAUNCH(cluster_row_compact_kernel, rows, rows, P->order, flag, pos, P->corder);
        LAUNCH(cluster_row_ranges_kernel, C, C, rows, P->start, P->cnt, pos, total, P->cstart,
               P->ccnt);
    }
    LAUNCH(cluster_info_kernel, C, C, n, P->row_of_cluster, ct.parent, ct.csize, P->cpar, P->nsize,
           P->in_tree);
    return FHG_OK;
}

}  // namespace

namespace {
__global__ void narrow_rows_kernel(int64_t rows, const int64_t* __restrict__ p,
                                   const int64_t* __restrict__ c, int32_t* __restrict__ op,
                                   int32_t* __restrict__ oc, unsigned long long* __restrict__ mx) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    op[r] = (int32_t)p[r];
    oc[r] = (int32_t)c[r];
    // labels fit 32 bits: combine the warp first, then one atomic per warp
    const unsigned act = __activemask();
    const unsigned m = __reduce_max_sync(act, (unsigned)max(p[r], c[r]));
    if ((int)(threadIdx.x & 31) == __ffs(act) - 1) atomicMax(mx, (unsigned long long)m);
}
}  // namespace

int condensed_from_arrays(Workspace& ws, const int64_t* parent, const int64_t* child,
                          const float* lambda, const float* csize, int64_t rows, Condensed* out) {
    cudaStream_t s = ws.stream();
    *out = Condensed();
    out->rows = rows;
    if (rows <= 0) return FHG_OK;
    unsigned long long* mx;
    FHG_TRY(ws.alloc(&out->parent, (size_t)rows));
    FHG_TRY(ws.alloc(&out->child, (size_t)rows));
    FHG_TRY(ws.alloc(&mx, 1));
    FHG_CUDA(cudaMemsetAsync(mx, 0, sizeof(unsigned long long), s));
    LAUNCH(narrow_rows_kernel, rows, rows, parent, child, out->parent, out->child, mx);
    int64_t root = 0;
    unsigned long long hmx = 0;
    FHG_CUDA(cudaMemcpyAsync(&root, parent, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaMemcpyAsync(&hmx, mx, sizeof(hmx), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    out->n = root;
    out->n_clusters = (int64_t)hmx - root + 1;
    out->lambda = const_cast<float*>(lambda);
    out->csize = const_cast<float*>(csize);
    return FHG_OK;
}

int select_eom(Workspace& ws, const Condensed& ct, double max_cs, bool allow_single, int32_t* sel,
               int64_t* n_sel, LabelPre* pre) {
    cudaStream_t s = ws.stream();
    *n_sel = 0;
    if (ct.rows == 0) return FHG_OK;
    Stage stage(s, "select");
    Prepared P;
    FHG_TRY(prepare(ws, ct, &P));
    if (pre) FHG_TRY(label_prework(ws, ct, pre));
    P.join();
    const int64_t C = P.C;
    int32_t *depth, *depth2, *jmp, *jmp2, *dcount, *byd, *flags;
    double* ret;
    int8_t *chose, *blocked;
    int64_t* nsel_dev;
    FHG_TRY(ws.alloc(&depth, (size_t)C));
    FHG_TRY(ws.alloc(&depth2, (size_t)C));
    FHG_TRY(ws.alloc(&flags, (size_t)C));
    FHG_TRY(ws.alloc(&jmp, (size_t)C));
    FHG_TRY(ws.alloc(&jmp2, (size_t)C));
    FHG_TRY(ws.alloc(&dcount, (size_t)C + 2));
    FHG_TRY(ws.alloc(&byd, (size_t)C));
    FHG_TRY(ws.alloc(&ret, (size_t)C));
    FHG_TRY(ws.alloc(&chose, (size_t)C));
    FHG_TRY(ws.alloc(&blocked, (size_t)C));
    FHG_TRY(ws.alloc(&nsel_dev, 1));
    ::fhg::note_launch();
    eom_kernel<<<1, kEomThreads, 0, s>>>(C, P.cpar, P.nsize, P.in_tree, P.score, P.cstart, P.ccnt,
                                         P.corder, ct.csize, ct.child, ct.n, max_cs,
                                         allow_single ? 1 : 0, depth, depth2, jmp, jmp2, dcount,
                                         byd, ret, chose, blocked, flags, sel, nsel_dev);
    FHG_CUDA(cudaGetLastError());
    FHG_CUDA(cudaMemcpyAsync(n_sel, nsel_dev, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    return FHG_OK;
}

int select_leaf(Workspace& ws, const Condensed& ct, int32_t* sel, int64_t* n_sel,
                LabelPre* pre) {
    cudaStream_t s = ws.stream();
    *n_sel = 0;
    if (ct.rows == 0) return FHG_OK;
    Prepared P;
    FHG_TRY(prepare(ws, ct, &P));
    if (pre) FHG_TRY(label_prework(ws, ct, pre));
    P.join();
    int32_t* flags;
    int64_t* nsel_dev;
    FHG_TRY(ws.alloc(&flags, (size_t)P.C));
    FHG_TRY(ws.alloc(&nsel_dev, 1));
    ::fhg::note_launch();
    leaf_kernel<<<1, kEomThreads, 0, s>>>(P.C, ct.n, P.cpar, P.in_tree, flags, sel, nsel_dev);
    FHG_CUDA(cudaGetLastError());
    FHG_CUDA(cudaMemcpyAsync(n_sel, nsel_dev, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    return FHG_OK;
}

int label_prework(Workspace& ws, const Condensed& ct, LabelPre* pre) {
    cudaStream_t s = ws.stream();
    const int64_t n = ct.n, rows = ct.rows, C = ct.n_clusters;
    *pre = LabelPre();
    if (rows == 0) return FHG_OK;
    FHG_TRY(ws.alloc(&pre->row_of_point, (size_t)n));
    FHG_TRY(ws.alloc(&pre->row_of_cluster, (size_t)C));
    FHG_TRY(ws.alloc(&pre->cpar, (size_t)C));
    FHG_TRY(ws.alloc(&pre->nsize, (size_t)C));
    FHG_TRY(ws.alloc(&pre->in_tree, (size_t)C));
    FHG_TRY(ws.alloc(&pre->root_max, 1));
    FHG_TRY(ws.alloc(&pre->death, (size_t)C));
    FHG_CUDA(cudaMemsetAsync(pre->root_max, 0, sizeof(unsigned int), s));
    FHG_CUDA(cudaMemsetAsync(pre->death, 0, sizeof(unsigned int) * C, s));
    LAUNCH(fill_i32_kernel, n, pre->row_of_point, n, -1);
    LAUNCH(fill_i32_kernel, C, pre->row_of_cluster, C, -1);
    LAUNCH(row_of_child_kernel, rows, rows, n, ct.child, pre->row_of_cluster, pre->row_of_point);
    LAUNCH(cluster_info_kernel, C, C, n, pre->row_of_cluster, ct.parent, ct.csize, pre->cpar,
           pre->nsize, pre->in_tree);
    LAUNCH(root_stats_kernel, rows, rows, n, ct.parent, ct.lambda, ct.csize, pre->root_max,
           pre->death);
    pre->ready = true;
    return FHG_OK;
}

int label_points(Workspace& ws, const Condensed& ct, const int32_t* sel, int64_t n_sel,
                 double eps, int64_t* labels, float* probs, const LabelPre* pre_in) {
    cudaStream_t s = ws.stream();
    const int64_t n = ct.n, rows = ct.rows, C = ct.n_clusters;
    Stage stage(s, "labels");
    FHG_CUDA(cudaMemsetAsync(probs, 0, sizeof(float) * n, s));
    if (rows == 0 || n_sel == 0) {
        LAUNCH(fill_i64_kernel, n, labels, n, (int64_t)-1);
        return FHG_OK;
    }
    LabelPre own;
    const LabelPre* pre = pre_in;
    if (!pre || !pre->ready) {
        FHG_TRY(label_prework(ws, ct, &own));
        pre = &own;
    }
    const int32_t* row_of_point = pre->row_of_point;
    const int32_t* cpar = pre->cpar;
    unsigned int* root_max = pre->root_max;
    unsigned int* death = pre->death;
    int8_t* is_sel;
    int32_t *label_of, *by_label, *jmp, *sa, *jmp2, *sa2;
    uint32_t* key;
    int32_t* val;
    int* err;
    FHG_TRY(ws.alloc(&is_sel, (size_t)C));
    FHG_TRY(ws.alloc(&label_of, (size_t)C));
    FHG_TRY(ws.alloc(&by_label, (size_t)n_sel));
    FHG_TRY(ws.alloc(&jmp, (size_t)C));
    FHG_TRY(ws.alloc(&sa, (size_t)C));
    FHG_TRY(ws.alloc(&jmp2, (size_t)C));
    FHG_TRY(ws.alloc(&sa2, (size_t)C));
    FHG_TRY(ws.alloc(&key, (size_t)n_sel));
    FHG_TRY(ws.alloc(&val, (size_t)n_sel));
    FHG_TRY(ws.alloc(&err, 1));
    FHG_CUDA(cudaMemsetAsync(is_sel, 0, C, s));
    FHG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    LAUNCH(fill_i32_kernel, C, label_of, C, -1);
    LAUNCH(sel_flags_kernel, n_sel, n_sel, n, C, sel, is_sel, key, val);
    {
        Workspace tmp(s);
        FHG_TRY(radix_sort_u32(tmp, key, val, n_sel, 0, 32));
    }
    LAUNCH(label_map_kernel, n_sel, n_sel, n, C, key, label_of, by_label);
    LAUNCH(anc_init_kernel, C, C, cpar, is_sel, jmp, sa);
    for (int r = 0; r < bits_for(C) + 1; ++r) {
        LAUNCH(anc_step_kernel, C, C, jmp, sa, jmp2, sa2);
        std::swap(jmp, jmp2);
        std::swap(sa, sa2);
    }
    // distinct selected count
    int64_t n_distinct = 0;
    {
        int8_t* h = (int8_t*)malloc((size_t)C);
        FHG_CUDA(cudaMemcpyAsync(h, is_sel, C, cudaMemcpyDeviceToHost, s));
        FHG_CUDA(cudaStreamSynchronize(s));
        for (int64_t c = 0; c < C; ++c) n_distinct += h[c] ? 1 : 0;
        free(h);
    }
    LAUNCH(point_labels_kernel, n, n, n_distinct, eps, row_of_point, ct.parent, ct.lambda, sa,
           is_sel, label_of, root_max, labels, err);
    LAUNCH(probs_kernel, rows, rows, n, ct.child, ct.lambda, labels, by_label, death, probs);
    int h_err = 0;
    FHG_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    if (h_err) {
        set_error("a point resolved to the root cluster, which is not selected (the reference "
                  "raises KeyError here)");
        return FHG_ERR_INVALID;
    }
    return FHG_OK;
}

int membership_strengths(Workspace& ws, const Condensed& ct, const int32_t* sel, int64_t n_sel,
                         const int64_t* labels, float* probs) {
    cudaStream_t s = ws.stream();
    const int64_t n = ct.n, rows = ct.rows, C = ct.n_clusters;
    FHG_CUDA(cudaMemsetAsync(probs, 0, sizeof(float) * n, s));
    if (rows == 0 || n_sel == 0) return FHG_OK;
    int8_t* is_sel;
    int32_t *label_of, *by_label, *val;
    uint32_t* key;
    unsigned int *root_max, *death;
    FHG_TRY(ws.alloc(&is_sel, (size_t)C));
    FHG_TRY(ws.alloc(&label_of, (size_t)C));
    FHG_TRY(ws.alloc(&by_label, (size_t)n_sel));
    FHG_TRY(ws.alloc(&key, (size_t)n_sel));
    FHG_TRY(ws.alloc(&val, (size_t)n_sel));
    FHG_TRY(ws.alloc(&root_max, 1));
    FHG_TRY(ws.alloc(&death, (size_t)C));
    FHG_CUDA(cudaMemsetAsync(is_sel, 0, C, s));
    FHG_CUDA(cudaMemsetAsync(death, 0, sizeof(unsigned int) * C, s));
    LAUNCH(fill_i32_kernel, C, label_of, C, -1);
    LAUNCH(sel_flags_kernel, n_sel, n_sel, n, C, sel, is_sel, key, val);
    {
        Workspace tmp(s);
        FHG_TRY(radix_sort_u32(tmp, key, val, n_sel, 0, 32));
    }
    LAUNCH(label_map_kernel, n_sel, n_sel, n, C, key, label_of, by_label);
    LAUNCH(root_stats_kernel, rows, rows, n, ct.parent, ct.lambda, ct.csize, root_max, death);
    LAUNCH(probs_kernel, rows, rows, n, ct.child, ct.lambda, labels, by_label, death, probs);
    return FHG_OK;
}

}  // namespace fhg
