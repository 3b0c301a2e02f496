// Condensed tree (cluster_trees.py:205 condense_tree), in parallel.
//
// The reference walks the linkage tree breadth-first from the root and, at
// every node it reaches, applies one of six cases to the two children
// (cluster_trees.py:263-350) by comparing their sizes with
// min_cluster_size: a child either continues the parent's cluster, starts a
// new cluster (both children large), or is eliminated -- all its points are
// emitted as rows at the parent's lambda (eliminate_branch, :148).
//
// The same decisions are local to each node here; what remains are prefix
// properties along root paths, computed for all nodes at once by pointer
// doubling over the linkage tree:
//   depth and DFS preorder      -> breadth-first order = sort by (depth, preorder)
//   topmost non-continuing node -> whether a node is reached, and for a point
//                                  the node that emits it
//   nearest cluster birth       -> the condensed label of a reached node
// Rows are then ordered by (emitting node's row offset, depth, preorder) --
// the reference's emission order -- with a stable radix sort, and new cluster
// labels are numbered by a prefix count of "both children large" nodes in
// breadth-first order.
#include "primitives.cuh"
#include "trees.cuh"

namespace fhg {
namespace {

enum : int8_t { C1 = 1, C2, C3, C4, C5, C6 };

__device__ __forceinline__ float lambda_of(double d) {
    return (float)(d > 0.0 ? 1.0 / d : (double)INFINITY);
}

// Per internal node: case, lambda, and the child flags written into the
// node-indexed arrays of its two children.
__global__ void cases_kernel(int64_t m, int64_t n, const int32_t* __restrict__ left,
                             const int32_t* __restrict__ right, const double* __restrict__ w,
                             const int32_t* __restrict__ size, const float* __restrict__ wsize,
                             double mcs, double max_cs, int8_t* __restrict__ kase,
                             float* __restrict__ lam,
                             int32_t* __restrict__ par, int8_t* __restrict__ cont,
                             int8_t* __restrict__ birth, int8_t* __restrict__ side) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int32_t L = left[i], R = right[i];
    // counts: leaves, or the points' sample weights (cluster_trees.py:253-262)
    const double lc = wsize ? (double)wsize[L] : (double)(float)size[L];
    const double rc = wsize ? (double)wsize[R] : (double)(float)size[R];
    int8_t c;
    if (L < n && rc >= mcs) c = C1;
    else if (lc < mcs && rc >= mcs) c = C2;
    else if (lc >= mcs && rc < mcs) c = C3;
    else if (lc < mcs && rc < mcs) c = C4;
    else if (lc > max_cs && rc > max_cs) c = C5;
    else c = C6;
    kase[i] = c;
    lam[i] = lambda_of(w[i]);
    par[L] = (int32_t)i;
    par[R] = (int32_t)i;
    side[L] = 0;
    side[R] = 1;
    cont[L] = (c == C3 || c == C5 || c == C6) ? 1 : 0;
    cont[R] = (c == C1 || c == C2 || c == C5 || c == C6) ? 1 : 0;
    birth[L] = birth[R] = (c == C6) ? 1 : 0;
}

// Pointer-doubling state of internal node i (node id n + i), one 32-byte
// record so that the gather of an ancestor's state touches a single sector:
//   anc  current ancestor (internal index; the root is its own ancestor)
//   dep  edges from the node up to anc;  pre  preorder offset up to anc
//   top  topmost non-continuing node on the path (-1: none yet)
//   bth  nearest cluster birth on the path (-1: none yet)
struct __align__(32) PjRec {
    int32_t anc, dep, top, bth;
    long long pre, pad;
};
__device__ __forceinline__ PjRec pj_load(const PjRec* __restrict__ R, int64_t i) {
    const int4 a = __ldg(reinterpret_cast<const int4*>(R + i));
    const longlong2 b = __ldg(reinterpret_cast<const longlong2*>(R + i) + 1);
    PjRec r;
    r.anc = a.x; r.dep = a.y; r.top = a.z; r.bth = a.w;
    r.pre = b.x; r.pad = 0;
    return r;
}
__device__ __forceinline__ void pj_store(PjRec* R, int64_t i, const PjRec& r) {
    reinterpret_cast<int4*>(R + i)[0] = make_int4(r.anc, r.dep, r.top, r.bth);
    reinterpret_cast<longlong2*>(R + i)[1] = make_longlong2(r.pre, 0);
}

__global__ void pj_init_kernel(int64_t m, int64_t n, const int32_t* __restrict__ par,
                               const int8_t* __restrict__ cont, const int8_t* __restrict__ birth,
                               const int8_t* __restrict__ side, const int32_t* __restrict__ left,
                               const int32_t* __restrict__ size, PjRec* __restrict__ R) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int64_t v = n + i;
    PjRec r;
    if (i == m - 1) {  // root
        r.anc = (int32_t)i;
        r.dep = 0;
        r.pre = 0;
        r.top = -1;
        r.bth = (int32_t)v;
    } else {
        const int32_t p = par[v];
        r.anc = p;
        r.dep = 1;
        r.pre = side[v] == 0 ? 1 : 2 * (long long)size[left[p]];
        r.top = cont[v] ? -1 : (int32_t)v;
        r.bth = birth[v] ? (int32_t)v : -1;
    }
    pj_store(R, i, r);
}

// One doubling step.  A node's state covers the path from it up to (not
// including) its ancestor; the root's own contribution is an identity for
// dep, pre and top and a default for bth, so a state stops changing one step
// after its ancestor has become the root.  `moving` (nullable) is set when
// some node's ancestor was not yet the root: a step that leaves it clear has
// finished every node.
__global__ void pj_step_kernel(int64_t m, const PjRec* __restrict__ R, PjRec* __restrict__ R2,
                               int* __restrict__ moving) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const PjRec x = pj_load(R, i);
    if (x.anc == (int32_t)i) {  // the root
        pj_store(R2, i, x);
        return;
    }
    if (moving && x.anc != (int32_t)(m - 1)) *moving = 1;
    const PjRec y = pj_load(R, x.anc);
    PjRec z;
    z.anc = y.anc;
    z.dep = x.dep + y.dep;
    z.pre = x.pre + y.pre;
    z.top = y.top != -1 ? y.top : x.top;
    z.bth = x.bth != -1 ? x.bth : y.bth;
    pj_store(R2, i, z);
}

__global__ void pj_split_kernel(int64_t m, const PjRec* __restrict__ R, int32_t* __restrict__ dep,
                                int64_t* __restrict__ pre, int32_t* __restrict__ top,
                                int32_t* __restrict__ bth) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const PjRec x = pj_load(R, i);
    dep[i] = x.dep;
    pre[i] = x.pre;
    top[i] = x.top;
    bth[i] = x.bth;
}

// Points: derive from the parent node; decide the emitting node and segment.
__global__ void points_kernel(int64_t n, int64_t m, const int32_t* __restrict__ par,
                              const int8_t* __restrict__ cont, const int8_t* __restrict__ side,
                              const int32_t* __restrict__ left, const int32_t* __restrict__ size,
                              const int32_t* __restrict__ dep, const int64_t* __restrict__ pre,
                              const int32_t* __restrict__ top, int32_t* __restrict__ emit_u,
                              int8_t* __restrict__ emit_part, int32_t* __restrict__ pdep,
                              int64_t* __restrict__ ppre) {
    int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const int32_t p = par[x];
    pdep[x] = dep[p] + 1;
    ppre[x] = pre[p] + (side[x] == 0 ? 1 : 2 * (int64_t)size[left[p]]);
    int32_t t = top[p];
    if (t == -1) t = cont[x] ? -1 : (int32_t)x;
    if (t == -1) {
        emit_u[x] = -1;
        emit_part[x] = 0;
        return;
    }
    emit_u[x] = par[t];
    emit_part[x] = side[t];
}

// Reached internal nodes (no non-continuing node on the path).
__global__ void reached_flags_kernel(int64_t m, const int32_t* __restrict__ top,
                                     uint32_t* __restrict__ flag) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) flag[i] = top[i] == -1 ? 1u : 0u;
}
__global__ void compact_idx_kernel(int64_t m, const uint32_t* __restrict__ flag,
                                   const uint32_t* __restrict__ pos, int32_t* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m && flag[i]) out[pos[i]] = (int32_t)i;
}
__global__ void gather_keys_kernel(int64_t cnt, const int32_t* __restrict__ items,
                                   const int32_t* __restrict__ dep, const int64_t* __restrict__ pre,
                                   uint32_t* __restrict__ kd, uint32_t* __restrict__ kp, int which) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cnt) return;
    int32_t i = items[j];
    if (which == 0) kp[j] = (uint32_t)pre[i];
    else kd[j] = (uint32_t)dep[i];
}
// Row counts and "new clusters" flags of reached nodes in breadth-first order.
__global__ void reached_counts_kernel(int64_t cnt, const int32_t* __restrict__ items,
                                      const int8_t* __restrict__ kase,
                                      const int32_t* __restrict__ left,
                                      const int32_t* __restrict__ right,
                                      const int32_t* __restrict__ size,
                                      int64_t* __restrict__ nrows, int64_t* __restrict__ nnew,
                                      int32_t* __restrict__ bfs_pos) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cnt) return;
    int32_t i = items[j];
    int8_t c = kase[i];
    int64_t r = 0;
    if (c == C1) r = 1;
    else if (c == C2) r = size[left[i]];
    else if (c == C3) r = size[right[i]];
    else if (c == C4) r = (int64_t)size[left[i]] + size[right[i]];
    else if (c == C6) r = 2;
    nrows[j] = r;
    nnew[j] = c == C6 ? 1 : 0;
    bfs_pos[i] = (int32_t)j;
}
// Condensed label of every reached node (from its nearest birth).
__global__ void reached_labels_kernel(int64_t cnt, int64_t n, const int32_t* __restrict__ items,
                                      const int32_t* __restrict__ bth,
                                      const int32_t* __restrict__ par,
                                      const int8_t* __restrict__ side,
                                      const int32_t* __restrict__ bfs_pos,
                                      const int64_t* __restrict__ k6, int32_t* __restrict__ label) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cnt) return;
    int32_t i = items[j];
    int32_t b = bth[i];
    const int64_t root_node = 2 * n - 2;
    int32_t lab;
    if (b == (int32_t)root_node) lab = (int32_t)n;
    else {
        int32_t u = par[b];
        lab = (int32_t)(n + 1 + 2 * k6[bfs_pos[u]] + side[b]);
    }
    label[i] = lab;
}

// Sort items: points that are emitted, plus two rows per new-cluster node.
// item ids: x in [0, n) for points; n + 2*j + s for the s-th row of reached
// node j (breadth-first position) when that node creates clusters.
__global__ void item_flags_kernel(int64_t n, int64_t cnt, const int32_t* __restrict__ emit_u,
                                  const int64_t* __restrict__ nnew, uint32_t* __restrict__ flag) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) flag[t] = emit_u[t] >= 0 ? 1u : 0u;
    else if (t < n + 2 * cnt) flag[t] = nnew[(t - n) >> 1] ? 1u : 0u;
}
__global__ void item_keys_kernel(int64_t nitems, int64_t n, const int32_t* __restrict__ items,
                                 const int32_t* __restrict__ emit_u,
                                 const int8_t* __restrict__ emit_part,
                                 const int8_t* __restrict__ kase, const int32_t* __restrict__ left,
                                 const int32_t* __restrict__ size,
                                 const int32_t* __restrict__ bfs_pos,
                                 const int64_t* __restrict__ roff, const int32_t* __restrict__ pdep,
                                 const int64_t* __restrict__ ppre, uint32_t* __restrict__ kseg,
                                 uint32_t* __restrict__ kdep, uint32_t* __restrict__ kpre) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nitems) return;
    int32_t it = items[t];
    if (it < n) {
        int32_t u = emit_u[it];
        int64_t base = roff[bfs_pos[u]];
        if (emit_part[it] == 1 && kase[u] == C4) base += size[left[u]];
        kseg[t] = (uint32_t)base;
        kdep[t] = (uint32_t)pdep[it];
        kpre[t] = (uint32_t)ppre[it];
    } else {
        int64_t r = it - n;
        kseg[t] = (uint32_t)(roff[r >> 1] + (r & 1));
        kdep[t] = 0;
        kpre[t] = 0;
    }
}
__global__ void gather_u32_kernel(int64_t cnt, const uint32_t* __restrict__ src,
                                  const int32_t* __restrict__ perm, uint32_t* __restrict__ dst) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cnt) dst[t] = src[perm[t]];
}
__global__ void rows_kernel(int64_t rows, int64_t n, const int32_t* __restrict__ order,
                            const int32_t* __restrict__ items, const int32_t* __restrict__ reached,
                            const int32_t* __restrict__ emit_u, const int32_t* __restrict__ label,
                            const float* __restrict__ lam, const int32_t* __restrict__ left,
                            const int32_t* __restrict__ right, const int32_t* __restrict__ size,
                            const float* __restrict__ wsize, const int64_t* __restrict__ k6,
                            int32_t* __restrict__ oparent,
                            int32_t* __restrict__ ochild, float* __restrict__ olam,
                            float* __restrict__ osize) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    int32_t it = items[order[r]];
    if (it < n) {
        int32_t u = emit_u[it];
        oparent[r] = label[u];
        ochild[r] = it;
        olam[r] = lam[u];
        osize[r] = 1.0f;
    } else {
        int64_t q = it - n;
        int64_t j = q >> 1;
        int s = (int)(q & 1);
        int32_t u = reached[j];
        oparent[r] = label[u];
        ochild[r] = (int32_t)(n + 1 + 2 * k6[j] + s);
        olam[r] = lam[u];
        const int32_t v = s == 0 ? left[u] : right[u];
        osize[r] = wsize ? wsize[v] : (float)size[v];
    }
}

__global__ void condensed_out_kernel(int64_t rows, const int32_t* __restrict__ p,
                                     const int32_t* __restrict__ c, const float* __restrict__ l,
                                     const float* __restrict__ z, int64_t* __restrict__ op,
                                     int64_t* __restrict__ oc, float* __restrict__ ol,
                                     float* __restrict__ oz) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    op[r] = p[r];
    oc[r] = c[r];
    ol[r] = l[r];
    oz[r] = z[r];
}

#define LAUNCH(kernel, count, ...)                                          \
    do {                                                                    \
        if ((count) > 0) {                                                  \
            ::fhg::note_launch(); \
            kernel<<<grid_for((count), 256), 256, 0, s>>>(__VA_ARGS__);     \
            FHG_CUDA(cudaGetLastError());                                   \
        }                                                                   \
    } while (0)

template <class T>
int read1(const T* dev, T* host, cudaStream_t s) {
    FHG_CUDA(cudaMemcpyAsync(host, dev, sizeof(T), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    return FHG_OK;
}

}  // namespace

int condense_tree(Workspace& ws, const Linkage& lk, int64_t mcs, double max_cs, Condensed* out) {
    cudaStream_t s = ws.stream();
    const int64_t n = lk.n, m = lk.m;
    *out = Condensed();
    out->n = n;
    if (m <= 0) return FHG_OK;
    Stage stage(s, "condense");
    const int64_t nodes = n + m;

    int8_t *kase, *cont, *birth, *side, *emit_part;
    float* lam;
    int32_t *par, *dep, *top, *bth, *emit_u, *pdep;
    int64_t *pre, *ppre;
    FHG_TRY(ws.alloc(&kase, (size_t)m));
    FHG_TRY(ws.alloc(&lam, (size_t)m));
    FHG_TRY(ws.alloc(&par, (size_t)nodes));
    FHG_TRY(ws.alloc(&cont, (size_t)nodes));
    FHG_TRY(ws.alloc(&birth, (size_t)nodes));
    FHG_TRY(ws.alloc(&side, (size_t)nodes));
    LAUNCH(cases_kernel, m, m, n, lk.left, lk.right, lk.w, lk.size, lk.wsize, (double)mcs, max_cs,
           kase, lam,
           par, cont, birth, side);

    FHG_TRY(ws.alloc(&dep, (size_t)m));
    FHG_TRY(ws.alloc(&pre, (size_t)m));
    FHG_TRY(ws.alloc(&top, (size_t)m));
    FHG_TRY(ws.alloc(&bth, (size_t)m));
    {
        Workspace tmp(s);
        PjRec *R, *R2;
        int* moving;
        FHG_TRY(tmp.alloc(&R, (size_t)m));
        FHG_TRY(tmp.alloc(&R2, (size_t)m));
        FHG_TRY(tmp.alloc(&moving, 1));
        LAUNCH(pj_init_kernel, m, m, n, par, cont, birth, side, lk.left, lk.size, R);
        // log2(height) + 1 steps finish every node; the height is not known,
        // so from step 12 on every fourth step reports whether it was the last
        const int steps = bits_for(m) + 1;
        for (int r = 0; r < steps; ++r) {
            const bool check = r >= 11 && (r & 3) == 3 && r + 1 < steps;
            if (check) FHG_CUDA(cudaMemsetAsync(moving, 0, sizeof(int), s));
            LAUNCH(pj_step_kernel, m, m, R, R2, check ? moving : nullptr);
            std::swap(R, R2);
            if (check) {
                int h_moving = 1;
                FHG_TRY(read1(moving, &h_moving, s));
                if (!h_moving) break;
            }
        }
        LAUNCH(pj_split_kernel, m, m, R, dep, pre, top, bth);
    }

    FHG_TRY(ws.alloc(&emit_u, (size_t)n));
    FHG_TRY(ws.alloc(&emit_part, (size_t)n));
    FHG_TRY(ws.alloc(&pdep, (size_t)n));
    FHG_TRY(ws.alloc(&ppre, (size_t)n));
    LAUNCH(points_kernel, n, n, m, par, cont, side, lk.left, lk.size, dep, pre, top, emit_u,
           emit_part, pdep, ppre);

    // ---- reached internal nodes in breadth-first order
    uint32_t *flag, *pos, *cnt_dev;
    int32_t *reached, *bfs_pos, *label;
    FHG_TRY(ws.alloc(&flag, (size_t)(n + 2 * m + 1)));
    FHG_TRY(ws.alloc(&pos, (size_t)(n + 2 * m + 1)));
    FHG_TRY(ws.alloc(&cnt_dev, 2));
    LAUNCH(reached_flags_kernel, m, m, top, flag);
    uint32_t h_cnt = 0;
    {
        Workspace tmp(s);
        FHG_TRY(scan_exclusive_u32(tmp, flag, pos, m, cnt_dev));
    }
    FHG_TRY(ws.alloc(&reached, (size_t)m));
    LAUNCH(compact_idx_kernel, m, m, flag, pos, reached);
    FHG_TRY(read1(cnt_dev, &h_cnt, s));
    const int64_t cnt = h_cnt;
    {
        Workspace tmp(s);
        uint32_t *kd, *kp;
        FHG_TRY(tmp.alloc(&kd, (size_t)cnt));
        FHG_TRY(tmp.alloc(&kp, (size_t)cnt));
        LAUNCH(gather_keys_kernel, cnt, cnt, reached, dep, pre, kd, kp, 0);
        FHG_TRY(radix_sort_u32(tmp, kp, reached, cnt, 0, bits_for(2 * n)));
        LAUNCH(gather_keys_kernel, cnt, cnt, reached, dep, pre, kd, kp, 1);
        FHG_TRY(radix_sort_u32(tmp, kd, reached, cnt, 0, bits_for(n)));
    }
    int64_t *nrows, *nnew, *roff, *k6, *tot;
    FHG_TRY(ws.alloc(&nrows, (size_t)cnt));
    FHG_TRY(ws.alloc(&nnew, (size_t)cnt));
    FHG_TRY(ws.alloc(&roff, (size_t)cnt));
    FHG_TRY(ws.alloc(&k6, (size_t)cnt));
    FHG_TRY(ws.alloc(&tot, 2));
    FHG_TRY(ws.alloc(&bfs_pos, (size_t)m));
    FHG_TRY(ws.alloc(&label, (size_t)m));
    LAUNCH(reached_counts_kernel, cnt, cnt, reached, kase, lk.left, lk.right, lk.size, nrows, nnew,
           bfs_pos);
    {
        Workspace tmp(s);
        FHG_TRY(scan_exclusive_i64(tmp, nrows, roff, cnt, tot));
        FHG_TRY(scan_exclusive_i64(tmp, nnew, k6, cnt, tot + 1));
    }
    LAUNCH(reached_labels_kernel, cnt, cnt, n, reached, bth, par, side, bfs_pos, k6, label);
    int64_t h_tot[2] = {0, 0};
    FHG_CUDA(cudaMemcpyAsync(h_tot, tot, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    const int64_t rows = h_tot[0];
    out->rows = rows;
    out->n_clusters = 1 + 2 * h_tot[1];

    // ---- row order: stable sort of items by (segment, depth, preorder)
    const int64_t universe = n + 2 * cnt;
    LAUNCH(item_flags_kernel, universe, n, cnt, emit_u, nnew, flag);
    int32_t* items;
    FHG_TRY(ws.alloc(&items, (size_t)(rows > 0 ? rows : 1)));
    {
        Workspace tmp(s);
        FHG_TRY(scan_exclusive_u32(tmp, flag, pos, universe, cnt_dev));
    }
    {
        // compact: item id = its index in the universe
        LAUNCH(compact_idx_kernel, universe, universe, flag, pos, items);
    }
    FHG_TRY(ws.alloc(&out->parent, (size_t)(rows > 0 ? rows : 1)));
    FHG_TRY(ws.alloc(&out->child, (size_t)(rows > 0 ? rows : 1)));
    FHG_TRY(ws.alloc(&out->lambda, (size_t)(rows > 0 ? rows : 1)));
    FHG_TRY(ws.alloc(&out->csize, (size_t)(rows > 0 ? rows : 1)));
    if (rows == 0) return FHG_OK;
    {
        Workspace tmp(s);
        uint32_t *kseg, *kdep, *kpre, *key;
        int32_t* order;
        FHG_TRY(tmp.alloc(&kseg, (size_t)rows));
        FHG_TRY(tmp.alloc(&kdep, (size_t)rows));
        FHG_TRY(tmp.alloc(&kpre, (size_t)rows));
        FHG_TRY(tmp.alloc(&key, (size_t)rows));
        FHG_TRY(tmp.alloc(&order, (size_t)rows));
        LAUNCH(item_keys_kernel, rows, rows, n, items, emit_u, emit_part, kase, lk.left, lk.size,
               bfs_pos, roff, pdep, ppre, kseg, kdep, kpre);
        FHG_TRY(fill_iota_i32(order, rows, s));
        LAUNCH(gather_u32_kernel, rows, rows, kpre, order, key);
        FHG_TRY(radix_sort_u32(tmp, key, order, rows, 0, bits_for(2 * n)));
        LAUNCH(gather_u32_kernel, rows, rows, kdep, order, key);
        FHG_TRY(radix_sort_u32(tmp, key, order, rows, 0, bits_for(n)));
        LAUNCH(gather_u32_kernel, rows, rows, kseg, order, key);
        FHG_TRY(radix_sort_u32(tmp, key, order, rows, 0, bits_for(rows)));
        LAUNCH(rows_kernel, rows, rows, n, order, items, reached, emit_u, label, lam, lk.left,
               lk.right, lk.size, lk.wsize, k6, out->parent, out->child, out->lambda, out->csize);
    }
    return FHG_OK;
}

int condensed_to_arrays(const Condensed& ct, int64_t* parent, int64_t* child, float* lambda,
                        float* csize, cudaStream_t s) {
    LAUNCH(condensed_out_kernel, ct.rows, ct.rows, ct.parent, ct.child, ct.lambda, ct.csize,
           parent, child, lambda, csize);
    return FHG_OK;
}

}  // namespace fhg
