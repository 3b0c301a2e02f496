// Spanning forest of a cluster's core graph (core_graph.py:198 boruvka_mst,
// the sub-cluster / branch detection back-end) -- or of many clusters' graphs
// side by side, as disjoint blocks of one CSR -- with the reference's choices
// among equal weights, so that the forest -- and the cluster hierarchy built
// from it -- is the reference's own.
//
// The graph is CSR, every row sorted by weight (ties in insertion order).
// A Boruvka round of the reference:
//   * every point's candidate is the first entry of its row that leaves its
//     component (the reference deletes the other entries, keeping order);
//   * a component keeps the candidate of smallest weight, ties to the
//     smallest point, and components come in the order of their smallest
//     point that has a candidate ("pos");
//   * the candidates are added in that order, each unless its ends are
//     already joined.
// The reference reads a point's candidate at its row's first slot, so a
// point with an empty row takes the first remaining entry of the next
// non-empty row (own[p]); such an entry may lie inside the point's own
// component, where it still counts as the component's candidate and is
// then skipped (a one-edge cycle below).
// The candidates form a functional graph on components (each points at the
// component its edge enters); processed in pos order, an edge is rejected
// exactly when it closes that graph's cycle, i.e. the cycle edge of largest
// pos.  So a round is: select (atomicMin on (ordered weight, point) and on
// pos), find every cycle and its largest pos by pointer doubling, drop that
// edge, emit the others in pos order (a scan over pos slots) and hook them
// with the lock-free union-find.
#include <algorithm>
#include <utility>

#include "fhg_common.cuh"
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

constexpr unsigned long long kNone = ~0ull;

// float32 bits -> unsigned key in the float order (negatives included; -0
// compares equal to +0, as in the reference's float comparisons)
__device__ __forceinline__ uint32_t ordered(float w) {
    const uint32_t u = __float_as_uint(w == 0.0f ? 0.0f : w);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void cg_init_kernel(int64_t n, const int32_t* __restrict__ indptr,
                               const int32_t* __restrict__ seg_end, int32_t* __restrict__ comp,
                               int32_t* __restrict__ par, int32_t* __restrict__ ptr,
                               int32_t* __restrict__ own) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    comp[p] = (int32_t)p;
    par[p] = (int32_t)p;
    ptr[p] = indptr[p];
    // the row owning slot indptr[p]: p, or the next non-empty row of p's graph
    const int64_t lim = seg_end ? (int64_t)seg_end[p] : n;
    int64_t r = p;
    while (r < lim && indptr[r + 1] == indptr[r]) ++r;
    own[p] = r < lim ? (int32_t)r : -1;
}

// Every row's first entry outside its component (the reference's rows after
// update_graph_components, :143).
__global__ void cg_advance_kernel(int64_t n, const int32_t* __restrict__ indptr,
                                  const int32_t* __restrict__ indices,
                                  const int32_t* __restrict__ comp, int32_t* __restrict__ ptr) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int32_t c = comp[p], end = indptr[p + 1];
    int32_t e = ptr[p];
    while (e < end && comp[indices[e]] == c) ++e;
    ptr[p] = e;
}

__global__ void cg_reset_kernel(int64_t n, unsigned long long* __restrict__ best,
                                int32_t* __restrict__ pos, uint32_t* __restrict__ take) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    best[c] = kNone;
    pos[c] = INT32_MAX;
    take[c] = 0u;
}

// Each point's candidate (the entry at its row's first slot); the
// component's smallest (weight, point) and its smallest point with one.
__global__ void cg_select_kernel(int64_t n, const int32_t* __restrict__ indptr,
                                 const float* __restrict__ weights,
                                 const int32_t* __restrict__ comp,
                                 const int32_t* __restrict__ ptr,
                                 const int32_t* __restrict__ own,
                                 unsigned long long* __restrict__ best,
                                 int32_t* __restrict__ pos) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int32_t r = own[p];
    if (r < 0) return;
    const int32_t e = ptr[r];
    if (e >= indptr[r + 1]) return;
    const int32_t c = comp[p];
    atomicMin(best + c, ((unsigned long long)ordered(weights[e]) << 32) | (uint32_t)p);
    atomicMin(pos + c, (int32_t)p);
}

// succ / mx of every component slot: the component its candidate enters and
// its pos (self and -1 for slots without a candidate).
__global__ void cg_succ_kernel(int64_t n, const int32_t* __restrict__ indices,
                               const int32_t* __restrict__ comp,
                               const int32_t* __restrict__ ptr,
                               const int32_t* __restrict__ own,
                               const unsigned long long* __restrict__ best,
                               const int32_t* __restrict__ pos, int32_t* __restrict__ succ,
                               int32_t* __restrict__ mx) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const unsigned long long b = best[c];
    if (b == kNone) {
        succ[c] = (int32_t)c;
        mx[c] = -1;
        return;
    }
    const int32_t p = (int32_t)(uint32_t)b;
    succ[c] = comp[indices[ptr[own[p]]]];
    mx[c] = pos[c];
}

__global__ void cg_double_kernel(int64_t n, const int32_t* __restrict__ succ,
                                 const int32_t* __restrict__ mx, int32_t* __restrict__ succ2,
                                 int32_t* __restrict__ mx2) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int32_t t = succ[c];
    succ2[c] = succ[t];
    mx2[c] = max(mx[c], mx[t]);
}

// A slot reached after 2^K >= n steps lies on its part's cycle.
__global__ void cg_mark_kernel(int64_t n, const unsigned long long* __restrict__ best,
                               const int32_t* __restrict__ succK, uint32_t* __restrict__ cyc) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n || best[c] == kNone) return;
    cyc[succK[c]] = 1u;
}

// Candidates kept: all but each cycle's largest-pos edge; take[pos] = 1 and
// slot[pos] = component, so that a scan over pos emits them in pos order.
__global__ void cg_keep_kernel(int64_t n, const unsigned long long* __restrict__ best,
                               const int32_t* __restrict__ pos, const uint32_t* __restrict__ cyc,
                               const int32_t* __restrict__ mxK, uint32_t* __restrict__ take,
                               int32_t* __restrict__ slot) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n || best[c] == kNone) return;
    if (cyc[c] && pos[c] == mxK[c]) return;
    take[pos[c]] = 1u;
    slot[pos[c]] = (int32_t)c;
}

__global__ void cg_emit_kernel(int64_t n, int64_t base, const uint32_t* __restrict__ take,
                               const uint32_t* __restrict__ rank,
                               const int32_t* __restrict__ slot,
                               const unsigned long long* __restrict__ best,
                               const int32_t* __restrict__ ptr,
                               const int32_t* __restrict__ own,
                               const int32_t* __restrict__ indices,
                               const float* __restrict__ weights, const int32_t* __restrict__ comp,
                               double* __restrict__ edges, int32_t* __restrict__ par) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n || !take[q]) return;
    const int32_t c = slot[q];
    const int32_t p = (int32_t)(uint32_t)best[c];
    const int32_t e = ptr[own[p]];
    const int32_t j = indices[e];
    double* row = edges + 3 * (base + rank[q]);
    row[0] = (double)p;
    row[1] = (double)j;
    row[2] = (double)weights[e];
    uf_union(par, c, comp[j]);
}

__global__ void cg_relabel_kernel(int64_t n, int32_t* __restrict__ comp, int32_t* __restrict__ par) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    comp[p] = uf_find(par, comp[p]);
}

// ------------------------------------------------------------ layout
// The core graphs of many clusters as one block CSR (core_graph.py:19
// knn_mst_union + :47 flatten_to_csr + :70 sort_by_lens): row q is point q of
// the block layout (clusters one after another, points in index order).  A
// row holds its kNN children (in neighbour order, each once, those inside the
// cluster) and then its MST children not already present (in MST order),
// sorted by weight with ties in that order; weight = float32(max(lens)),
// distance = float32(max(core)) for kNN children, the MST distance otherwise.

// Row q's MST edges: [lower_bound(q), lower_bound(q + 1)) of the sorted parents.
__device__ __forceinline__ int64_t lower_bound_u32(const uint32_t* a, int64_t m, uint32_t v) {
    int64_t lo = 0, hi = m;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Whether the e-th MST child of row q is kept: not a kNN child of the row
// and not an earlier MST child of it.
__device__ __forceinline__ bool mst_kept(const int32_t* __restrict__ nbq, int k,
                                         const int32_t* __restrict__ mchild,
                                         const int32_t* __restrict__ order, int64_t b, int64_t e) {
    const int32_t ch = mchild[order[e]];
    for (int j = 0; j < k; ++j)
        if (nbq[j] == ch) return false;
    for (int64_t f = b; f < e; ++f)
        if (mchild[order[f]] == ch) return false;
    return true;
}

__device__ __forceinline__ bool knn_kept(const int32_t* __restrict__ nbq, int j) {
    const int32_t ch = nbq[j];
    if (ch < 0) return false;
    for (int i = 0; i < j; ++i)
        if (nbq[i] == ch) return false;
    return true;
}

__global__ void cgl_count_kernel(int64_t P, int k, const int32_t* __restrict__ nb,
                                 const uint32_t* __restrict__ mkey, int64_t M,
                                 const int32_t* __restrict__ mchild,
                                 const int32_t* __restrict__ order, uint32_t* __restrict__ len) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P) return;
    const int32_t* nbq = nb + q * k;
    uint32_t c = 0;
    for (int j = 0; j < k; ++j) c += knn_kept(nbq, j) ? 1u : 0u;
    const int64_t b = lower_bound_u32(mkey, M, (uint32_t)q);
    const int64_t e1 = lower_bound_u32(mkey, M, (uint32_t)(q + 1));
    for (int64_t e = b; e < e1; ++e) c += mst_kept(nbq, k, mchild, order, b, e) ? 1u : 0u;
    len[q] = c;
}

__global__ void cgl_fill_kernel(int64_t P, int k, const int32_t* __restrict__ nb,
                                const uint32_t* __restrict__ mkey, int64_t M,
                                const int32_t* __restrict__ mchild,
                                const double* __restrict__ mdist,
                                const int32_t* __restrict__ order,
                                const double* __restrict__ lens, const float* __restrict__ core,
                                const int32_t* __restrict__ blk_start,
                                const int32_t* __restrict__ blk_end,
                                const uint32_t* __restrict__ off, int32_t* __restrict__ indptr,
                                int32_t* __restrict__ idx_local, int32_t* __restrict__ idx_block,
                                float* __restrict__ w, float* __restrict__ dist,
                                int32_t* __restrict__ seg_end) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P) return;
    const int32_t* nbq = nb + q * k;
    const int32_t s0 = blk_start[q];
    const int64_t r0 = off[q];
    int64_t r = r0;
    indptr[q] = (int32_t)r0;
    seg_end[q] = blk_end[q];
    const double lq = lens[q];
    const float cq = core[q];
    for (int j = 0; j < k; ++j) {
        if (!knn_kept(nbq, j)) continue;
        const int32_t ch = nbq[j];
        idx_local[r] = ch;
        idx_block[r] = s0 + ch;
        w[r] = (float)fmax(lq, lens[s0 + ch]);
        dist[r] = fmaxf(cq, core[s0 + ch]);
        ++r;
    }
    const int64_t b = lower_bound_u32(mkey, M, (uint32_t)q);
    const int64_t e1 = lower_bound_u32(mkey, M, (uint32_t)(q + 1));
    for (int64_t e = b; e < e1; ++e) {
        if (!mst_kept(nbq, k, mchild, order, b, e)) continue;
        const int32_t ch = mchild[order[e]];
        idx_local[r] = ch;
        idx_block[r] = s0 + ch;
        w[r] = (float)fmax(lq, lens[s0 + ch]);
        dist[r] = (float)mdist[order[e]];
        ++r;
    }
    if (q == P - 1) indptr[P] = (int32_t)r;
    // stable insertion sort of the row by weight
    for (int64_t i = r0 + 1; i < r; ++i) {
        const float wi = w[i], di = dist[i];
        const int32_t li = idx_local[i], bi = idx_block[i];
        int64_t j = i;
        while (j > r0 && w[j - 1] > wi) {
            w[j] = w[j - 1];
            dist[j] = dist[j - 1];
            idx_local[j] = idx_local[j - 1];
            idx_block[j] = idx_block[j - 1];
            --j;
        }
        w[j] = wi;
        dist[j] = di;
        idx_local[j] = li;
        idx_block[j] = bi;
    }
}

// ------------------------------------------------------- label propagation
// Noise points of a cluster take the label whose summed inverse lens weight
// over their labelled core-graph neighbours is largest (sub_clusters.py:132).
// The reference sweeps the cluster's noise points in index order, writing
// each new label in place, so a point already sees the labels given earlier
// in the same sweep; sweeps repeat while noise remains.  One thread runs that
// sequence for its cluster, every cluster in parallel.  adj_*: for every
// noise point (entries noise_first[c] .. noise_first[c+1] of cluster c, in
// index order), its neighbours in the order the reference's per-point dict
// holds them and their inverse weights; tab_*: per noise point, room for its
// distinct neighbour labels (one slot per neighbour).  Label sums are
// float64, in neighbour order; the first label reaching the largest sum
// wins.  A sweep that labels nothing ends the cluster's work (points no
// labelled point can reach stay noise).
__global__ void propagate_kernel(int64_t nclusters, const int32_t* __restrict__ noise_first,
                                 const int32_t* __restrict__ noise_pt,
                                 const int32_t* __restrict__ adj_ptr,
                                 const int32_t* __restrict__ adj_other,
                                 const double* __restrict__ adj_w, int32_t* lab,
                                 int32_t* __restrict__ tab_lab, double* __restrict__ tab_sum) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nclusters) return;
    const int32_t a = noise_first[c], b = noise_first[c + 1];
    // every sweep but the last labels at least one point
    for (int32_t sweep = 0; sweep <= b - a; ++sweep) {
        bool changed = false;
        for (int32_t x = a; x < b; ++x) {
            const int32_t p = noise_pt[x];
            if (lab[p] != -1) continue;
            const int32_t e0 = adj_ptr[x], e1 = adj_ptr[x + 1];
            int32_t nd = 0;
            for (int32_t e = e0; e < e1; ++e) {
                const int32_t l = lab[adj_other[e]];
                if (l == -1) continue;
                int32_t t = 0;
                while (t < nd && tab_lab[e0 + t] != l) ++t;
                if (t == nd) {
                    tab_lab[e0 + nd] = l;
                    tab_sum[e0 + nd] = 0.0;
                    ++nd;
                }
                tab_sum[e0 + t] = __dadd_rn(tab_sum[e0 + t], adj_w[e]);
            }
            if (nd == 0) continue;
            double best = -INFINITY;
            int32_t bl = -1;
            for (int32_t t = 0; t < nd; ++t)
                if (tab_sum[e0 + t] > best) {
                    best = tab_sum[e0 + t];
                    bl = tab_lab[e0 + t];
                }
            lab[p] = bl;
            changed = true;
        }
        if (!changed) break;
    }
}

}  // namespace

int propagate_labels(int64_t nclusters, const int32_t* noise_first, const int32_t* noise_pt,
                     const int32_t* adj_ptr, const int32_t* adj_other, const double* adj_w,
                     int32_t* labels, cudaStream_t s) {
    if (nclusters <= 0) return FHG_OK;
    int32_t n_noise = 0, n_adj = 0;
    FHG_CUDA(cudaMemcpyAsync(&n_noise, noise_first + nclusters, sizeof(int32_t),
                             cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    if (n_noise <= 0) return FHG_OK;
    FHG_CUDA(cudaMemcpyAsync(&n_adj, adj_ptr + n_noise, sizeof(int32_t), cudaMemcpyDeviceToHost,
                             s));
    FHG_CUDA(cudaStreamSynchronize(s));
    Workspace ws(s);
    int32_t* tab_lab;
    double* tab_sum;
    FHG_TRY(ws.alloc(&tab_lab, (size_t)(n_adj > 0 ? n_adj : 1)));
    FHG_TRY(ws.alloc(&tab_sum, (size_t)(n_adj > 0 ? n_adj : 1)));
    ::fhg::note_launch();
    propagate_kernel<<<grid_for(nclusters, 64), 64, 0, s>>>(
        nclusters, noise_first, noise_pt, adj_ptr, adj_other, adj_w, labels, tab_lab, tab_sum);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

int core_graph_boruvka(int64_t n, const int32_t* indptr, const int32_t* indices,
                       const float* weights, const int32_t* seg_end, double* edges,
                       int64_t* n_edges, cudaStream_t s) {
    *n_edges = 0;
    if (n <= 1) return FHG_OK;
    if (n > 0x7ffffffeLL) {
        set_error("core graph: more than 2^31 - 2 points");
        return FHG_ERR_UNSUPPORTED;
    }
    Stage stage(s, "core_graph_boruvka");
    Workspace ws(s);
    int32_t *comp, *par, *ptr, *own, *pos, *succ, *mx, *succ2, *mx2, *slot;
    unsigned long long* best;
    uint32_t *take, *rank, *cyc, *total;
    FHG_TRY(ws.alloc(&comp, (size_t)n));
    FHG_TRY(ws.alloc(&par, (size_t)n));
    FHG_TRY(ws.alloc(&ptr, (size_t)n));
    FHG_TRY(ws.alloc(&own, (size_t)n));
    FHG_TRY(ws.alloc(&pos, (size_t)n));
    FHG_TRY(ws.alloc(&succ, (size_t)n));
    FHG_TRY(ws.alloc(&mx, (size_t)n));
    FHG_TRY(ws.alloc(&succ2, (size_t)n));
    FHG_TRY(ws.alloc(&mx2, (size_t)n));
    FHG_TRY(ws.alloc(&slot, (size_t)n));
    FHG_TRY(ws.alloc(&best, (size_t)n));
    FHG_TRY(ws.alloc(&take, (size_t)n));
    FHG_TRY(ws.alloc(&rank, (size_t)n));
    FHG_TRY(ws.alloc(&cyc, (size_t)n));
    FHG_TRY(ws.alloc(&total, 1));
    LAUNCH(cg_init_kernel, n, n, indptr, seg_end, comp, par, ptr, own);
    int K = 1;
    while (((int64_t)1 << K) < n) ++K;
    int64_t m = 0, components = n;
    while (components > 1) {
        LAUNCH(cg_reset_kernel, n, n, best, pos, take);
        FHG_CUDA(cudaMemsetAsync(cyc, 0, sizeof(uint32_t) * n, s));
        // rows are compacted after each round's merges: the first round reads
        // them as given (an entry may point into its own one-point component)
        if (m > 0 || components < n) LAUNCH(cg_advance_kernel, n, n, indptr, indices, comp, ptr);
        LAUNCH(cg_select_kernel, n, n, indptr, weights, comp, ptr, own, best, pos);
        LAUNCH(cg_succ_kernel, n, n, indices, comp, ptr, own, best, pos, succ, mx);
        int32_t *a = succ, *am = mx, *b = succ2, *bm = mx2;
        for (int k = 0; k < K; ++k) {
            LAUNCH(cg_double_kernel, n, n, a, am, b, bm);
            std::swap(a, b);
            std::swap(am, bm);
        }
        LAUNCH(cg_mark_kernel, n, n, best, a, cyc);
        LAUNCH(cg_keep_kernel, n, n, best, pos, cyc, am, take, slot);
        FHG_TRY(scan_exclusive_u32(ws, take, rank, n, total));
        uint32_t added = 0;
        FHG_CUDA(cudaMemcpyAsync(&added, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        FHG_CUDA(cudaStreamSynchronize(s));
        if (added == 0) break;
        if (m + (int64_t)added > n - 1) {
            set_error("core graph: spanning forest overflow");
            return FHG_ERR_NO_CONVERGENCE;
        }
        LAUNCH(cg_emit_kernel, n, n, m, take, rank, slot, best, ptr, own, indices, weights,
               comp, edges, par);
        LAUNCH(cg_relabel_kernel, n, n, comp, par);
        m += added;
        components -= added;
    }
    *n_edges = m;
    return FHG_OK;
}


int core_graphs_layout(int64_t P, int k, const int32_t* nb, const double* lens, const float* core,
                       const int32_t* blk_start, const int32_t* blk_end, int64_t M,
                       const int32_t* mparent, const int32_t* mchild, const double* mdist,
                       int32_t* indptr, int32_t* idx_local, int32_t* idx_block, float* w,
                       float* dist, int32_t* seg_end, int64_t* nnz, cudaStream_t s) {
    *nnz = 0;
    if (P <= 0) return FHG_OK;
    if (P + (int64_t)k * P + M > 0x7fffffffLL) {
        set_error("core graphs: more than 2^31 - 1 entries");
        return FHG_ERR_UNSUPPORTED;
    }
    Stage stage(s, "core_graph_layout");
    Workspace ws(s);
    uint32_t *mkey, *len, *off, *total;
    int32_t* order;
    FHG_TRY(ws.alloc(&mkey, (size_t)std::max<int64_t>(M, 1)));
    FHG_TRY(ws.alloc(&order, (size_t)std::max<int64_t>(M, 1)));
    FHG_TRY(ws.alloc(&len, (size_t)P));
    FHG_TRY(ws.alloc(&off, (size_t)P));
    FHG_TRY(ws.alloc(&total, 1));
    if (M > 0) {
        FHG_CUDA(cudaMemcpyAsync(mkey, mparent, sizeof(uint32_t) * M, cudaMemcpyDeviceToDevice, s));
        FHG_TRY(fill_iota_i32(order, M, s));
        if (M > 1) FHG_TRY(radix_sort_u32(ws, mkey, order, M, 0, 32));  // stable: MST order kept
    }
    LAUNCH(cgl_count_kernel, P, P, k, nb, mkey, M, mchild, order, len);
    FHG_TRY(scan_exclusive_u32(ws, len, off, P, total));
    LAUNCH(cgl_fill_kernel, P, P, k, nb, mkey, M, mchild, mdist, order, lens, core, blk_start,
           blk_end, off, indptr, idx_local, idx_block, w, dist, seg_end);
    uint32_t h = 0;
    FHG_CUDA(cudaMemcpyAsync(&h, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    *nnz = h;
    return FHG_OK;
}

}  // namespace fhg
