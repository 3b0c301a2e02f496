// Cluster-selection options on the GPU: the DBSCAN cut of the linkage tree,
// the epsilon search over selected clusters and the persistence
// simplification of the condensed tree.
//
// DBSCAN cut (cluster_trees.py:906 get_cluster_labelling_at_cut).  The
// reference unions, for every linkage row with distance < cut, both children
// with the row's node through a union-by-rank disjoint set, then numbers the
// components whose size reaches min_cluster_size in increasing order of their
// representative.  A row's node is fresh when it is unioned, so the
// representative and rank of every subtree follow from its children alone:
//   L' = max(rank(left), 1)                          (first union bumps it)
//   rank = rank(right) == L' ? L' + 1 : max(L', rank(right))
//   rep  = rank(right) >= L' ? rep(right) : rep(left)
// with points at rank 0 and rep itself.  rank(v) >= r exactly when some node
// s of v's subtree has both children at rank >= r-1 (r >= 3), or, for r = 2,
// an internal right child; so each rank level is one pass of subtree-range
// counts over a preorder numbering.  Representatives follow the dominant
// child by pointer doubling; a point's component is the highest ancestor
// whose distance is below the cut (distances grow towards the root).
//
// Epsilon search (cluster_trees.py:834 cluster_epsilon_search) and
// simplify_hierarchy (:774) work on the cluster tree -- the condensed rows
// with child_size > 1, a few per cluster -- in one thread block each, with
// the reference's exact semantics (including segments_in_branch's unchecked
// searchsorted lookup, :881), followed by point-sized passes that relabel and
// compact the condensed tree.
#include <utility>

#include "primitives.cuh"
#include "trees.cuh"

namespace fhg {
namespace {

#define LAUNCH(kernel, count, ...)                                          \
    do {                                                                    \
        if ((count) > 0) {                                                  \
            ::fhg::note_launch();                                           \
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

// ------------------------------------------------------------ DBSCAN cut
__global__ void cut_parents_kernel(int64_t m, int64_t n, const int32_t* __restrict__ left,
                                   const int32_t* __restrict__ right, int32_t* __restrict__ par,
                                   int8_t* __restrict__ side) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    par[left[i]] = (int32_t)(n + i);
    side[left[i]] = 0;
    par[right[i]] = (int32_t)(n + i);
    side[right[i]] = 1;
    if (i == m - 1) par[n + i] = -1;
}

// Preorder of internal node i (node n+i): anc = internal index of the
// ancestor reached so far, pre = offset accumulated along the way.  In the
// preorder a node's subtree spans [pre, pre + 2*size - 1): itself, the left
// subtree, then the right subtree.
__global__ void cut_pre_init_kernel(int64_t m, int64_t n, const int32_t* __restrict__ par,
                                    const int8_t* __restrict__ side,
                                    const int32_t* __restrict__ left,
                                    const int32_t* __restrict__ size, int32_t* __restrict__ anc,
                                    int64_t* __restrict__ pre) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int32_t p = par[n + i];
    if (p < 0) {
        anc[i] = (int32_t)i;
        pre[i] = 0;
        return;
    }
    const int64_t pi = p - n;
    anc[i] = (int32_t)pi;
    pre[i] = side[n + i] == 0 ? 1 : 2 * (int64_t)size[left[pi]];
}
__global__ void cut_pre_step_kernel(int64_t m, const int32_t* __restrict__ anc,
                                    const int64_t* __restrict__ pre, int32_t* __restrict__ anc2,
                                    int64_t* __restrict__ pre2) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int32_t a = anc[i];
    if (a == (int32_t)i) {
        anc2[i] = a;
        pre2[i] = pre[i];
        return;
    }
    anc2[i] = anc[a];
    pre2[i] = pre[i] + pre[a];
}

__device__ __forceinline__ int32_t rank_of(const int8_t* __restrict__ rk, int64_t n, int32_t v) {
    return v < n ? 0 : rk[v - n];
}

// Seeds of rank level r at their preorder positions.
__global__ void cut_seed_kernel(int64_t m, int64_t n, int r, const int32_t* __restrict__ left,
                                const int32_t* __restrict__ right,
                                const int8_t* __restrict__ rk, const int64_t* __restrict__ pre,
                                uint32_t* __restrict__ flag) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    bool seed;
    if (r == 2) seed = right[i] >= n;
    else seed = rank_of(rk, n, left[i]) >= r - 1 && rank_of(rk, n, right[i]) >= r - 1;
    if (seed) flag[pre[i]] = 1u;
}
__global__ void cut_rank_kernel(int64_t m, int64_t n, int r, int64_t positions,
                                const int64_t* __restrict__ pre,
                                const int32_t* __restrict__ size, const uint32_t* __restrict__ pos,
                                const uint32_t* __restrict__ total, int8_t* __restrict__ rk) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int64_t b = pre[i], e = b + 2 * (int64_t)size[n + i] - 1;
    const uint32_t pe = e < positions ? pos[e] : *total;
    if (pe > pos[b]) rk[i] = (int8_t)r;
}

// Dominant child of every internal node; points point at themselves.
__global__ void cut_dom_kernel(int64_t m, int64_t n, const int32_t* __restrict__ left,
                               const int32_t* __restrict__ right, const int8_t* __restrict__ rk,
                               int32_t* __restrict__ jmp) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int32_t rl = rank_of(rk, n, left[i]), rr = rank_of(rk, n, right[i]);
    const int32_t lp = rl > 1 ? rl : 1;
    jmp[i] = rr >= lp ? right[i] : left[i];
}
// Pointer doubling over node ids: values < n are final (points).
__global__ void cut_jump_kernel(int64_t m, int64_t n, const int32_t* __restrict__ jmp,
                                int32_t* __restrict__ jmp2) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int32_t v = jmp[i];
    jmp2[i] = v < n || v == (int32_t)(n + i) ? v : jmp[v - n];
}

// Highest ancestor below the cut: up = parent while the parent's distance is
// below the cut, else the node itself.
__global__ void cut_up_kernel(int64_t m, int64_t n, double cut, const int32_t* __restrict__ par,
                              const double* __restrict__ w, int32_t* __restrict__ up) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int32_t p = par[n + i];
    up[i] = (p >= 0 && w[p - n] < cut) ? p : (int32_t)(n + i);
}

__global__ void cut_point_rep_kernel(int64_t n, double cut, const int32_t* __restrict__ par,
                                     const double* __restrict__ w, const int32_t* __restrict__ top,
                                     const int32_t* __restrict__ rep, int32_t* __restrict__ prep,
                                     int32_t* __restrict__ count) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int32_t q = par[p];
    int32_t r = (int32_t)p;
    if (q >= 0 && w[q - n] < cut) r = rep[top[q - n] - n];
    prep[p] = r;
    atomicAdd(&count[r], 1);
}
__global__ void cut_flags_kernel(int64_t n, int64_t mcs, const int32_t* __restrict__ count,
                                 uint32_t* __restrict__ flag) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    flag[p] = (count[p] > 0 && count[p] >= mcs) ? 1u : 0u;
}
__global__ void cut_labels_kernel(int64_t n, const int32_t* __restrict__ prep,
                                  const uint32_t* __restrict__ flag,
                                  const uint32_t* __restrict__ pos, int64_t* __restrict__ labels) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int32_t r = prep[p];
    labels[p] = flag[r] ? (int64_t)pos[r] : -1;
}

// ------------------------------------------------------ cluster tree view
// Rows with child_size > 1, compacted in row order.
__global__ void ct_flags_kernel(int64_t rows, const float* __restrict__ csize,
                                uint32_t* __restrict__ flag) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rows) flag[i] = csize[i] > 1.0f ? 1u : 0u;
}
__global__ void ct_compact_kernel(int64_t rows, const uint32_t* __restrict__ flag,
                                  const uint32_t* __restrict__ pos,
                                  const int32_t* __restrict__ parent,
                                  const int32_t* __restrict__ child,
                                  const float* __restrict__ lambda, int32_t* __restrict__ cp,
                                  int32_t* __restrict__ cc, float* __restrict__ cl) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows || !flag[i]) return;
    const uint32_t j = pos[i];
    cp[j] = parent[i];
    cc[j] = child[i];
    cl[j] = lambda[i];
}
__global__ void keys_u32_kernel(int64_t R, const int32_t* __restrict__ v, int32_t base,
                                uint32_t* __restrict__ key, int32_t* __restrict__ row) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R) return;
    key[i] = (uint32_t)(v[i] - base);
    row[i] = (int32_t)i;
}
__global__ void gather_i32_kernel(int64_t R, const int32_t* __restrict__ src,
                                  const int32_t* __restrict__ idx, int32_t* __restrict__ dst) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < R) dst[i] = src[idx[i]];
}
// mm[0] = least parent (the root, cluster_tree.parent.min()), mm[1] = least
// label, mm[2] = largest label
__global__ void minmax_kernel(int64_t R, const int32_t* __restrict__ cp,
                              const int32_t* __restrict__ cc, int32_t* __restrict__ mm) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R) return;
    atomicMin(&mm[0], cp[i]);
    atomicMin(&mm[1], min(cp[i], cc[i]));
    atomicMax(&mm[2], max(cp[i], cc[i]));
}

// numpy's searchsorted(a, v, side='left') on a (nominally sorted) array.
__device__ __forceinline__ int64_t lower_bound(const int32_t* a, int64_t len, int32_t v) {
    int64_t lo = 0, hi = len;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

constexpr int kOptThreads = 1024;

// Single-block epsilon search.  Row-order cluster tree (cp, cc, cl), the
// same rows sorted by child (sc_child, sc_row) and by parent (sp_par,
// sp_child), both stable.  proc: one flag per child position plus one for
// the root (index R).
__global__ void __launch_bounds__(kOptThreads) eps_kernel(
    int64_t R, const int32_t* __restrict__ cp, const int32_t* __restrict__ cc,
    const float* __restrict__ cl, const int32_t* __restrict__ sc_child,
    const int32_t* __restrict__ sc_row, const int32_t* __restrict__ sp_par,
    const int32_t* __restrict__ sp_child, const int32_t* __restrict__ mm,
    const int32_t* __restrict__ sel, int64_t k, double eps, int32_t* proc, int32_t* fa,
    int32_t* fb, int32_t* out, int64_t* n_out) {
    __shared__ int32_t s_action, s_target, s_nf, s_nnext;
    __shared__ int64_t s_out;
    const int t = threadIdx.x;
    const int32_t root = mm[0];
    // first row whose child is v, -1 if none
    auto first_row = [&](int32_t v) -> int64_t {
        const int64_t j = lower_bound(sc_child, R, v);
        return (j < R && sc_child[j] == v) ? sc_row[j] : -1;
    };
    auto proc_slot = [&](int32_t v) -> int64_t {
        if (v == root) return R;
        const int64_t j = lower_bound(sc_child, R, v);
        return (j < R && sc_child[j] == v) ? j : -1;
    };
    if (t == 0) s_out = 0;
    __syncthreads();
    for (int64_t q = 0; q < k; ++q) {
        if (t == 0) {
            const int32_t c = sel[q];
            const int64_t idx = lower_bound(cc, R, c);  // searchsorted(cluster_tree.child, c)
            const float lam = cl[idx < R ? idx : R - 1];
            const double death = lam > 0.0f ? 1.0 / (double)lam : (double)INFINITY;
            s_action = 0;
            if (death < eps) {
                const int64_t slot = proc_slot(c);
                if (slot < 0 || !proc[slot]) {
                    // traverse_upwards (:866)
                    int32_t seg = c, res;
                    for (;;) {
                        const int64_t r = first_row(seg);
                        const int32_t par = r >= 0 ? cp[r] : -1;
                        if (par == root) {
                            res = root;
                            break;
                        }
                        const int64_t pr = first_row(par);
                        const float pl = pr >= 0 ? cl[pr] : 0.0f;
                        const double pe = pl > 0.0f ? 1.0 / (double)pl : (double)INFINITY;
                        if (pe >= eps) {
                            res = par;
                            break;
                        }
                        seg = par;
                    }
                    out[s_out++] = res;
                    s_action = 1;
                    s_target = res;
                }
            } else {
                out[s_out++] = c;
            }
        }
        __syncthreads();
        if (s_action == 1) {
            // segments_in_branch (:881): breadth-first closure, skipping
            // clusters already marked (the marked set is itself closed)
            if (t == 0) {
                const int64_t slot = proc_slot(s_target);
                s_nf = 0;
                if (slot >= 0 && !proc[slot]) {
                    proc[slot] = 1;
                    fa[0] = s_target;
                    s_nf = 1;
                } else if (slot < 0) {
                    fa[0] = s_target;  // not a cluster-tree label: expand it all the same
                    s_nf = 1;
                }
            }
            __syncthreads();
            int32_t* cur = fa;
            int32_t* nxt = fb;
            while (s_nf > 0) {
                if (t == 0) s_nnext = 0;
                __syncthreads();
                for (int j = t; j < s_nf; j += blockDim.x) {
                    const int32_t x = cur[j];
                    const int64_t lb = lower_bound(sp_par, R, x);
                    if (lb >= R) continue;
                    for (int h = 0; h < 2; ++h) {
                        if (lb + h >= R) break;
                        const int32_t ch = sp_child[lb + h];
                        const int64_t slot = proc_slot(ch);
                        if (slot < 0) continue;
                        if (atomicExch(&proc[slot], 1) == 0) nxt[atomicAdd(&s_nnext, 1)] = ch;
                    }
                }
                __syncthreads();
                if (t == 0) s_nf = s_nnext;
                int32_t* tp = cur;
                cur = nxt;
                nxt = tp;
                __syncthreads();
            }
        }
        __syncthreads();
    }
    if (t == 0) *n_out = s_out;
}

// ------------------------------------------------------- simplification
__global__ void leaf_clear_kernel(int64_t R, int64_t n, const int32_t* __restrict__ cp,
                                  int8_t* __restrict__ leaf) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < R) leaf[cp[i] - n] = 0;
}
__global__ void last_row_kernel(int64_t rows, int64_t n, const int32_t* __restrict__ parent,
                                int32_t* __restrict__ last) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rows) atomicMax(&last[parent[i] - n], (int32_t)i);
}
// max_births[parent - n] = lambda_val, the last row of each parent winning
// (the reference's fancy-index assignment); 0 where no row names the label.
__global__ void births_init_kernel(int64_t L, int64_t n, const int32_t* __restrict__ last,
                                   const float* __restrict__ lambda, float* __restrict__ maxb,
                                   int32_t* __restrict__ pmap, int8_t* __restrict__ has_lm,
                                   int32_t* __restrict__ cpar) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= L) return;
    maxb[j] = last[j] >= 0 ? lambda[last[j]] : 0.0f;
    pmap[j] = (int32_t)(n + j);
    has_lm[j] = 0;
    cpar[j] = -1;
}
__global__ void cluster_parent_kernel(int64_t R, int64_t n, const int32_t* __restrict__ cp,
                                      const int32_t* __restrict__ cc, int32_t* __restrict__ cpar) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < R) cpar[cc[i] - n] = cp[i] - (int32_t)n;
}

// Single block: the reference's loop over sibling pairs (rows idx-1, idx for
// idx = R-1, R-3, ...), children before parents.  Pairs whose parents lie at
// the same depth touch disjoint entries, so they run together, deepest first.
__global__ void __launch_bounds__(kOptThreads) simplify_pairs_kernel(
    int64_t R, int64_t L, int64_t n, double thr, const int32_t* __restrict__ cp,
    const int32_t* __restrict__ cc, const float* __restrict__ cl,
    const int32_t* __restrict__ cpar, int32_t* depth, int32_t* depth2, int32_t* jmp,
    int32_t* jmp2, int32_t* dcount, int32_t* byd, float* maxb, int8_t* leaf, float* lmap,
    int8_t* has_lm, int32_t* pmap) {
    const int t = threadIdx.x;
    __shared__ int32_t s_maxd;
    for (int64_t c = t; c < L; c += blockDim.x) {
        const bool inner = cpar[c] >= 0;
        depth[c] = inner ? 1 : 0;
        jmp[c] = inner ? cpar[c] : (int32_t)c;
    }
    __syncthreads();
    int rounds = 1;
    while (((int64_t)1 << rounds) < L + 1) ++rounds;
    for (int r = 0; r <= rounds; ++r) {
        for (int64_t c = t; c < L; c += blockDim.x) {
            const int32_t a = jmp[c];
            depth2[c] = a == (int32_t)c ? depth[c] : depth[c] + depth[a];
            jmp2[c] = jmp[a];
        }
        __syncthreads();
        int32_t* tp = depth; depth = depth2; depth2 = tp;
        tp = jmp; jmp = jmp2; jmp2 = tp;
    }
    const int64_t P = R / 2;  // pair j: rows R-2-2j, R-1-2j
    if (t == 0) s_maxd = 0;
    __syncthreads();
    for (int64_t j = t; j < P; j += blockDim.x)
        atomicMax(&s_maxd, depth[cp[R - 1 - 2 * j] - n]);
    __syncthreads();
    const int32_t maxd = s_maxd;
    for (int64_t d = t; d <= maxd + 1; d += blockDim.x) dcount[d] = 0;
    __syncthreads();
    for (int64_t j = t; j < P; j += blockDim.x) atomicAdd(&dcount[depth[cp[R - 1 - 2 * j] - n]], 1);
    __syncthreads();
    if (t == 0) {  // exclusive prefix over depths (few entries)
        int32_t run = 0;
        for (int32_t d = 0; d <= maxd + 1; ++d) {
            const int32_t v = dcount[d];
            dcount[d] = run;
            run += v;
        }
    }
    __syncthreads();
    for (int64_t j = t; j < P; j += blockDim.x)
        byd[atomicAdd(&dcount[depth[cp[R - 1 - 2 * j] - n]], 1)] = (int32_t)j;
    __syncthreads();
    // dcount[d] is now the end of depth d
    for (int32_t d = maxd; d >= 0; --d) {
        const int32_t b = d == 0 ? 0 : dcount[d - 1], e = dcount[d];
        for (int32_t q = b + t; q < e; q += blockDim.x) {
            const int64_t idx = R - 1 - 2 * (int64_t)byd[q];
            const int32_t par = cp[idx], ch0 = cc[idx - 1], ch1 = cc[idx];
            const float death = cl[idx];
            const int32_t n0 = ch0 - (int32_t)n, n1 = ch1 - (int32_t)n, pn = par - (int32_t)n;
            const float b0 = maxb[n0], b1 = maxb[n1];
            const float bmax = b0 > b1 ? b0 : b1, bmin = b0 < b1 ? b0 : b1;
            const float cur = maxb[pn];
            maxb[pn] = cur > bmax ? cur : bmax;
            if ((double)__fsub_rn(bmin, death) >= thr) continue;
            const bool sib = b0 <= b1;  // the more persistent child
            if (leaf[sib ? n1 : n0]) {
                leaf[pn] = 1;
            } else {
                const int32_t other = sib ? n0 : n1;
                has_lm[other] = 1;
                lmap[other] = death;
            }
            pmap[n0] = par;
            pmap[n1] = par;
        }
        __syncthreads();
    }
}

__global__ void pmap_jump_kernel(int64_t L, int64_t n, const int32_t* __restrict__ pm,
                                 int32_t* __restrict__ pm2) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < L) pm2[j] = pm[pm[j] - n];
}
__global__ void skipped_kernel(int64_t L, int64_t n, const int32_t* __restrict__ pm,
                               uint32_t* __restrict__ sk) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < L) sk[j] = pm[j] != (int32_t)(n + j) ? 1u : 0u;
}
// Relabel the kept rows in place (the reference mutates its argument) and
// flag them for compaction.
__global__ void simplify_apply_kernel(int64_t rows, int64_t n, const int32_t* __restrict__ pm,
                                      const uint32_t* __restrict__ sk,
                                      const uint32_t* __restrict__ skpos,
                                      const int8_t* __restrict__ has_lm,
                                      const float* __restrict__ lmap, int32_t* parent,
                                      int32_t* child, float* lambda, uint32_t* __restrict__ keep) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    const int32_t ch = child[i];
    const int64_t key = ch - n > 0 ? ch - n : 0;
    if (sk[key]) {
        keep[i] = 0u;
        return;
    }
    keep[i] = 1u;
    const int32_t p = parent[i], pn = p - (int32_t)n;
    if (has_lm[pn]) lambda[i] = lmap[pn];
    const int32_t np_ = pm[pn];
    parent[i] = np_ - (int32_t)skpos[np_ - n];
    if (ch >= n) {
        const int32_t nc = pm[ch - n];
        child[i] = nc - (int32_t)skpos[nc - n];
    }
}
__global__ void rows_compact_kernel(int64_t rows, const uint32_t* __restrict__ keep,
                                    const uint32_t* __restrict__ pos,
                                    const int32_t* __restrict__ parent,
                                    const int32_t* __restrict__ child,
                                    const float* __restrict__ lambda,
                                    const float* __restrict__ csize, int32_t* __restrict__ op,
                                    int32_t* __restrict__ oc, float* __restrict__ ol,
                                    float* __restrict__ os) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows || !keep[i]) return;
    const uint32_t j = pos[i];
    op[j] = parent[i];
    oc[j] = child[i];
    ol[j] = lambda[i];
    os[j] = csize[i];
}

// ---------------------------------------------------------- sample weights
__global__ void point_pre_kernel(int64_t n, int64_t m, const int32_t* __restrict__ par,
                                 const int8_t* __restrict__ side,
                                 const int32_t* __restrict__ left,
                                 const int32_t* __restrict__ size,
                                 const int64_t* __restrict__ pre, const float* __restrict__ w,
                                 double* __restrict__ vals) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int32_t q = par[p];
    if (q < 0) return;
    const int64_t qi = q - n;
    vals[pre[qi] + (side[p] == 0 ? 1 : 2 * (int64_t)size[left[qi]])] = (double)w[p];
}
__global__ void subtree_sums_kernel(int64_t m, int64_t n, int64_t positions,
                                    const int64_t* __restrict__ pre,
                                    const int32_t* __restrict__ size,
                                    const double* __restrict__ excl,
                                    const double* __restrict__ total, float* __restrict__ wsize) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int64_t b = pre[i], e = b + 2 * (int64_t)size[n + i] - 1;
    const double hi = e < positions ? excl[e] : *total;
    wsize[n + i] = (float)(hi - excl[b]);
}
// Representative point of every internal node: its leftmost leaf.
__global__ void rep_init_kernel(int64_t m, const int32_t* __restrict__ left,
                                int32_t* __restrict__ jmp) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) jmp[i] = left[i];
}
__global__ void rep_edges_kernel(int64_t m, int64_t n, const int32_t* __restrict__ left,
                                 const int32_t* __restrict__ right,
                                 const int32_t* __restrict__ rep, int32_t* __restrict__ src,
                                 int32_t* __restrict__ dst) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int32_t l = left[i], r = right[i];
    src[i] = l < n ? l : rep[l - n];
    dst[i] = r < n ? r : rep[r - n];
}

}  // namespace

// Parent and side (0 left, 1 right) of every node, and the preorder position
// of every internal node (subtree of node n+i: [pre[i], pre[i] + 2*size - 1)).
static int linkage_preorder(Workspace& ws, const Linkage& lk, int32_t* par, int8_t* side,
                            int64_t* pre) {
    cudaStream_t s = ws.stream();
    const int64_t n = lk.n, m = lk.m, nodes = n + m;
    if (m == 0) {
        FHG_CUDA(cudaMemsetAsync(par, 0xff, sizeof(int32_t) * nodes, s));
        return FHG_OK;
    }
    LAUNCH(cut_parents_kernel, m, m, n, lk.left, lk.right, par, side);
    const int R = bits_for(m) + 1;
    Workspace tmp(s);
    int32_t *anc, *anc2;
    int64_t* pre2;
    FHG_TRY(tmp.alloc(&anc, (size_t)m));
    FHG_TRY(tmp.alloc(&anc2, (size_t)m));
    FHG_TRY(tmp.alloc(&pre2, (size_t)m));
    LAUNCH(cut_pre_init_kernel, m, m, n, par, side, lk.left, lk.size, anc, pre);
    int64_t* cur = pre;
    for (int r = 0; r < R; ++r) {
        int64_t* nxt = cur == pre ? pre2 : pre;
        LAUNCH(cut_pre_step_kernel, m, m, anc, cur, anc2, nxt);
        std::swap(anc, anc2);
        cur = nxt;
    }
    if (cur != pre)
        FHG_CUDA(cudaMemcpyAsync(pre, cur, sizeof(int64_t) * m, cudaMemcpyDeviceToDevice, s));
    return FHG_OK;
}

int weighted_sizes(Workspace& ws, Linkage& lk, const float* weights) {
    cudaStream_t s = ws.stream();
    const int64_t n = lk.n, m = lk.m, nodes = n + m;
    FHG_TRY(ws.alloc(&lk.wsize, (size_t)nodes));
    FHG_CUDA(cudaMemcpyAsync(lk.wsize, weights, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    if (m == 0) return FHG_OK;
    Workspace tmp(s);
    int32_t* par;
    int8_t* side;
    int64_t* pre;
    double *vals, *excl, *total;
    const int64_t positions = 2 * n - 1;
    FHG_TRY(tmp.alloc(&par, (size_t)nodes));
    FHG_TRY(tmp.alloc(&side, (size_t)nodes));
    FHG_TRY(tmp.alloc(&pre, (size_t)m));
    FHG_TRY(linkage_preorder(tmp, lk, par, side, pre));
    FHG_TRY(tmp.alloc(&vals, (size_t)positions));
    FHG_TRY(tmp.alloc(&excl, (size_t)positions));
    FHG_TRY(tmp.alloc(&total, 1));
    FHG_CUDA(cudaMemsetAsync(vals, 0, sizeof(double) * positions, s));
    LAUNCH(point_pre_kernel, n, n, m, par, side, lk.left, lk.size, pre, weights, vals);
    FHG_TRY(scan_exclusive_f64(tmp, vals, excl, positions, total));
    LAUNCH(subtree_sums_kernel, m, m, n, positions, pre, lk.size, excl, total, lk.wsize);
    return FHG_OK;
}

int linkage_leaf_counts(Workspace& ws, Linkage& lk) {
    cudaStream_t s = ws.stream();
    const int64_t n = lk.n, m = lk.m;
    if (m == 0) return FHG_OK;
    int32_t *jmp, *jmp2, *src, *dst;
    FHG_TRY(ws.alloc(&src, (size_t)m));
    FHG_TRY(ws.alloc(&dst, (size_t)m));
    {
        Workspace tmp(s);
        FHG_TRY(tmp.alloc(&jmp, (size_t)m));
        FHG_TRY(tmp.alloc(&jmp2, (size_t)m));
        LAUNCH(rep_init_kernel, m, m, lk.left, jmp);
        const int R = bits_for(m) + 1;
        for (int r = 0; r < R; ++r) {
            LAUNCH(cut_jump_kernel, m, m, n, jmp, jmp2);
            std::swap(jmp, jmp2);
        }
        LAUNCH(rep_edges_kernel, m, m, n, lk.left, lk.right, jmp, src, dst);
    }
    Linkage rebuilt;
    FHG_TRY(sort_and_link(ws, n, src, dst, lk.w, nullptr, &rebuilt, /*presorted=*/true));
    lk.size = rebuilt.size;
    return FHG_OK;
}

// The cluster tree (child_size > 1 rows, in row order) with the lookups the
// option passes need.
struct ClusterTree {
    int64_t R = 0;
    int32_t *cp = nullptr, *cc = nullptr;
    float* cl = nullptr;
    int32_t* mm = nullptr;  // device: root, least label, largest label
};

static int cluster_tree_of(Workspace& ws, const Condensed& ct, ClusterTree* out) {
    cudaStream_t s = ws.stream();
    *out = ClusterTree();
    if (ct.rows == 0) return FHG_OK;
    uint32_t *flag, *pos, *total;
    Workspace tmp(s);
    FHG_TRY(tmp.alloc(&flag, (size_t)ct.rows));
    FHG_TRY(tmp.alloc(&pos, (size_t)ct.rows));
    FHG_TRY(tmp.alloc(&total, 1));
    LAUNCH(ct_flags_kernel, ct.rows, ct.rows, ct.csize, flag);
    FHG_TRY(scan_exclusive_u32(tmp, flag, pos, ct.rows, total));
    uint32_t h = 0;
    FHG_TRY(read1(total, &h, s));
    out->R = h;
    const int64_t R = h;
    FHG_TRY(ws.alloc(&out->cp, (size_t)(R > 0 ? R : 1)));
    FHG_TRY(ws.alloc(&out->cc, (size_t)(R > 0 ? R : 1)));
    FHG_TRY(ws.alloc(&out->cl, (size_t)(R > 0 ? R : 1)));
    FHG_TRY(ws.alloc(&out->mm, 3));
    LAUNCH(ct_compact_kernel, ct.rows, ct.rows, flag, pos, ct.parent, ct.child, ct.lambda,
           out->cp, out->cc, out->cl);
    const int32_t init[3] = {INT32_MAX, INT32_MAX, INT32_MIN};
    FHG_CUDA(cudaMemcpyAsync(out->mm, init, sizeof(init), cudaMemcpyHostToDevice, s));
    LAUNCH(minmax_kernel, R, R, out->cp, out->cc, out->mm);
    FHG_CUDA(cudaStreamSynchronize(s));  // init is a host stack array
    return FHG_OK;
}

// Stable order of the cluster-tree rows by one column: the sorted column and
// the rows' other column in that order.
static int sort_rows_by(Workspace& ws, const ClusterTree& t, const int32_t* by,
                        const int32_t* other, int32_t base, int32_t span, int32_t* sorted_by,
                        int32_t* sorted_other, int32_t* rows_out) {
    cudaStream_t s = ws.stream();
    const int64_t R = t.R;
    Workspace tmp(s);
    uint32_t* key;
    FHG_TRY(tmp.alloc(&key, (size_t)R));
    LAUNCH(keys_u32_kernel, R, R, by, base, key, rows_out);
    FHG_TRY(radix_sort_u32(tmp, key, rows_out, R, 0, bits_for(span)));
    LAUNCH(gather_i32_kernel, R, R, by, rows_out, sorted_by);
    if (sorted_other) LAUNCH(gather_i32_kernel, R, R, other, rows_out, sorted_other);
    return FHG_OK;
}

int epsilon_search(Workspace& ws, const Condensed& ct, const int32_t* sel, int64_t k, double eps,
                   int32_t* out, int64_t* n_out) {
    cudaStream_t s = ws.stream();
    Stage stage(s, "epsilon");
    *n_out = 0;
    if (k <= 0) return FHG_OK;
    ClusterTree t;
    FHG_TRY(cluster_tree_of(ws, ct, &t));
    if (t.R == 0) {  // nothing to search (the reference is never called so)
        FHG_CUDA(cudaMemcpyAsync(out, sel, sizeof(int32_t) * k, cudaMemcpyDeviceToDevice, s));
        *n_out = k;
        return FHG_OK;
    }
    const int64_t R = t.R;
    int32_t hmm[3];
    FHG_CUDA(cudaMemcpyAsync(hmm, t.mm, sizeof(hmm), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    const int32_t base = hmm[1], span = hmm[2] - hmm[1];
    int32_t *sc_child, *sc_row, *sp_par, *sp_child, *sp_row, *proc, *fa, *fb;
    int64_t* nout_dev;
    FHG_TRY(ws.alloc(&sc_child, (size_t)R));
    FHG_TRY(ws.alloc(&sc_row, (size_t)R));
    FHG_TRY(ws.alloc(&sp_par, (size_t)R));
    FHG_TRY(ws.alloc(&sp_child, (size_t)R));
    FHG_TRY(ws.alloc(&sp_row, (size_t)R));
    FHG_TRY(ws.alloc(&proc, (size_t)(R + 1)));
    FHG_TRY(ws.alloc(&fa, (size_t)(R + 2)));
    FHG_TRY(ws.alloc(&fb, (size_t)(R + 2)));
    FHG_TRY(ws.alloc(&nout_dev, 1));
    FHG_TRY(sort_rows_by(ws, t, t.cc, nullptr, base, span, sc_child, nullptr, sc_row));
    FHG_TRY(sort_rows_by(ws, t, t.cp, t.cc, base, span, sp_par, sp_child, sp_row));
    FHG_CUDA(cudaMemsetAsync(proc, 0, sizeof(int32_t) * (R + 1), s));
    ::fhg::note_launch();
    eps_kernel<<<1, kOptThreads, 0, s>>>(R, t.cp, t.cc, t.cl, sc_child, sc_row, sp_par, sp_child,
                                         t.mm, sel, k, eps, proc, fa, fb, out, nout_dev);
    FHG_CUDA(cudaGetLastError());
    FHG_TRY(read1(nout_dev, n_out, s));
    return FHG_OK;
}

int simplify_hierarchy(Workspace& ws, const Condensed& ct, double thr, Condensed* out) {
    cudaStream_t s = ws.stream();
    Stage stage(s, "simplify");
    *out = ct;
    if (ct.rows == 0) return FHG_OK;
    ClusterTree t;
    FHG_TRY(cluster_tree_of(ws, ct, &t));
    if (t.R == 0) return FHG_OK;  // no cluster rows: nothing to simplify
    const int64_t R = t.R, n = ct.n;
    int32_t last_child = 0;
    FHG_CUDA(cudaMemcpyAsync(&last_child, t.cc + (R - 1), sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    const int64_t L = (int64_t)last_child + 1 - n;  // n_nodes - n_points
    if (L <= 0) return FHG_OK;
    int8_t *leaf, *has_lm;
    float *maxb, *lmap;
    int32_t *last, *pmap, *pm2, *cpar, *depth, *depth2, *jmp, *jmp2, *dcount, *byd;
    uint32_t *sk, *skpos, *keep, *kpos, *total;
    FHG_TRY(ws.alloc(&leaf, (size_t)L));
    FHG_TRY(ws.alloc(&has_lm, (size_t)L));
    FHG_TRY(ws.alloc(&maxb, (size_t)L));
    FHG_TRY(ws.alloc(&lmap, (size_t)L));
    FHG_TRY(ws.alloc(&last, (size_t)L));
    FHG_TRY(ws.alloc(&pmap, (size_t)L));
    FHG_TRY(ws.alloc(&pm2, (size_t)L));
    FHG_TRY(ws.alloc(&cpar, (size_t)L));
    FHG_TRY(ws.alloc(&depth, (size_t)L));
    FHG_TRY(ws.alloc(&depth2, (size_t)L));
    FHG_TRY(ws.alloc(&jmp, (size_t)L));
    FHG_TRY(ws.alloc(&jmp2, (size_t)L));
    FHG_TRY(ws.alloc(&dcount, (size_t)(L + 2)));
    FHG_TRY(ws.alloc(&byd, (size_t)(R / 2 + 1)));
    FHG_TRY(ws.alloc(&sk, (size_t)L));
    FHG_TRY(ws.alloc(&skpos, (size_t)L));
    FHG_TRY(ws.alloc(&keep, (size_t)ct.rows));
    FHG_TRY(ws.alloc(&kpos, (size_t)ct.rows));
    FHG_TRY(ws.alloc(&total, 2));
    FHG_CUDA(cudaMemsetAsync(leaf, 1, (size_t)L, s));
    FHG_CUDA(cudaMemsetAsync(last, 0xff, sizeof(int32_t) * L, s));
    LAUNCH(leaf_clear_kernel, R, R, n, t.cp, leaf);
    LAUNCH(last_row_kernel, ct.rows, ct.rows, n, ct.parent, last);
    LAUNCH(births_init_kernel, L, L, n, last, ct.lambda, maxb, pmap, has_lm, cpar);
    LAUNCH(cluster_parent_kernel, R, R, n, t.cp, t.cc, cpar);
    ::fhg::note_launch();
    simplify_pairs_kernel<<<1, kOptThreads, 0, s>>>(R, L, n, thr, t.cp, t.cc, t.cl, cpar, depth,
                                                    depth2, jmp, jmp2, dcount, byd, maxb, leaf,
                                                    lmap, has_lm, pmap);
    FHG_CUDA(cudaGetLastError());
    const int rounds = bits_for(L) + 1;
    for (int r = 0; r < rounds; ++r) {
        LAUNCH(pmap_jump_kernel, L, L, n, pmap, pm2);
        std::swap(pmap, pm2);
    }
    LAUNCH(skipped_kernel, L, L, n, pmap, sk);
    FHG_TRY(scan_exclusive_u32(ws, sk, skpos, L, total));
    LAUNCH(simplify_apply_kernel, ct.rows, ct.rows, n, pmap, sk, skpos, has_lm, lmap, ct.parent,
           ct.child, ct.lambda, keep);
    FHG_TRY(scan_exclusive_u32(ws, keep, kpos, ct.rows, total + 1));
    uint32_t h[2] = {0, 0};
    FHG_CUDA(cudaMemcpyAsync(h, total, sizeof(h), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    Condensed o;
    o.n = n;
    o.rows = h[1];
    o.n_clusters = L - (int64_t)h[0];
    FHG_TRY(ws.alloc(&o.parent, (size_t)(o.rows > 0 ? o.rows : 1)));
    FHG_TRY(ws.alloc(&o.child, (size_t)(o.rows > 0 ? o.rows : 1)));
    FHG_TRY(ws.alloc(&o.lambda, (size_t)(o.rows > 0 ? o.rows : 1)));
    FHG_TRY(ws.alloc(&o.csize, (size_t)(o.rows > 0 ? o.rows : 1)));
    LAUNCH(rows_compact_kernel, ct.rows, ct.rows, keep, kpos, ct.parent, ct.child, ct.lambda,
           ct.csize, o.parent, o.child, o.lambda, o.csize);
    *out = o;
    return FHG_OK;
}

int labelling_at_cut(Workspace& ws, const Linkage& lk, double cut, int64_t mcs,
                     int64_t* labels) {
    cudaStream_t s = ws.stream();
    const int64_t n = lk.n, m = lk.m, nodes = n + m;
    Stage stage(s, "dbscan_cut");
    int32_t *par, *jmp, *jmp2, *up, *up2, *prep, *count;
    int8_t *side, *rk;
    int64_t* pre;
    uint32_t *flag, *pos, *total;
    FHG_TRY(ws.alloc(&par, (size_t)nodes));
    FHG_TRY(ws.alloc(&side, (size_t)nodes));
    FHG_TRY(ws.alloc(&prep, (size_t)n));
    FHG_TRY(ws.alloc(&count, (size_t)n));
    FHG_TRY(ws.alloc(&total, 1));
    FHG_CUDA(cudaMemsetAsync(count, 0, sizeof(int32_t) * n, s));
    if (m == 0) FHG_CUDA(cudaMemsetAsync(par, 0xff, sizeof(int32_t) * nodes, s));
    FHG_TRY(ws.alloc(&jmp, (size_t)(m > 0 ? m : 1)));
    FHG_TRY(ws.alloc(&up, (size_t)(m > 0 ? m : 1)));
    if (m > 0) {
        const int R = bits_for(m) + 1;
        FHG_TRY(ws.alloc(&pre, (size_t)m));
        FHG_TRY(ws.alloc(&rk, (size_t)m));
        FHG_TRY(linkage_preorder(ws, lk, par, side, pre));
        // ranks, one level at a time
        FHG_CUDA(cudaMemsetAsync(rk, 1, (size_t)m, s));
        const int64_t positions = 2 * n - 1;
        {
            Workspace tmp(s);
            FHG_TRY(tmp.alloc(&flag, (size_t)positions));
            FHG_TRY(tmp.alloc(&pos, (size_t)positions));
            for (int r = 2; r < 127; ++r) {
                FHG_CUDA(cudaMemsetAsync(flag, 0, sizeof(uint32_t) * positions, s));
                LAUNCH(cut_seed_kernel, m, m, n, r, lk.left, lk.right, rk, pre, flag);
                FHG_TRY(scan_exclusive_u32(tmp, flag, pos, positions, total));
                uint32_t h_total = 0;
                FHG_TRY(read1(total, &h_total, s));
                if (h_total == 0) break;
                LAUNCH(cut_rank_kernel, m, m, n, r, positions, pre, lk.size, pos, total, rk);
            }
        }
        // representatives and components
        {
            Workspace tmp(s);
            FHG_TRY(tmp.alloc(&jmp2, (size_t)m));
            FHG_TRY(tmp.alloc(&up2, (size_t)m));
            LAUNCH(cut_dom_kernel, m, m, n, lk.left, lk.right, rk, jmp);
            LAUNCH(cut_up_kernel, m, m, n, cut, par, lk.w, up);
            for (int r = 0; r < R; ++r) {
                LAUNCH(cut_jump_kernel, m, m, n, jmp, jmp2);
                LAUNCH(cut_jump_kernel, m, m, n, up, up2);
                std::swap(jmp, jmp2);
                std::swap(up, up2);
            }
            if (R & 1) {
                FHG_CUDA(cudaMemcpyAsync(jmp2, jmp, sizeof(int32_t) * m, cudaMemcpyDeviceToDevice, s));
                FHG_CUDA(cudaMemcpyAsync(up2, up, sizeof(int32_t) * m, cudaMemcpyDeviceToDevice, s));
                std::swap(jmp, jmp2);
                std::swap(up, up2);
            }
        }
    }
    LAUNCH(cut_point_rep_kernel, n, n, cut, par, lk.w, up, jmp, prep, count);
    Workspace tmp(s);
    FHG_TRY(tmp.alloc(&flag, (size_t)n));
    FHG_TRY(tmp.alloc(&pos, (size_t)n));
    LAUNCH(cut_flags_kernel, n, n, mcs, count, flag);
    FHG_TRY(scan_exclusive_u32(tmp, flag, pos, n, total));
    LAUNCH(cut_labels_kernel, n, n, prep, flag, pos, labels);
    return FHG_OK;
}

}  // namespace fhg
