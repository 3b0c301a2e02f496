// Boruvka minimum spanning tree over mutual reachability, on the GPU.
//
// Replaces boruvka.py:474-647 (initialize_boruvka_from_knn,
// update_component_vectors, boruvka_tree_query, merge_components,
// parallel_boruvka).  Weights are squared float32 mutual-reachability
// distances max(rdist(p, q), core2[p], core2[q]) until the final sqrt.
//
// Round 0 (boruvka.py:474): every point p links to its first kNN neighbour q
// (position >= 1) with core2[p] >= core2[q], weight max(core2[p], rdist).
// These links form a forest except for cycles through equal core distances;
// the reference unions them in point order, so on every cycle the link of
// the largest point index is the one it skips -- dropped here the same way.
//
// Round r >= 1: for every point, the best edge to another component by
// (weight, caller index of the far end), found by a warp-cooperative walk of
// the bucket tree that skips nodes lying wholly inside the point's own
// component (node_comp, boruvka.py:98-124) and nodes beyond the component's
// running bound (boruvka.py:182-186).  Each component keeps its minimum in a
// 64-bit word (weight bits << 32 | min endpoint index) updated by atomicMin,
// with a second 32-bit atomicMin on the max endpoint index: together the
// total order (weight, min index, max index).  Under a total order two
// components can only choose each other with the same edge; the edge is
// then written once, oriented from the component whose lowest point index
// is smaller -- the component the reference's merge loop visits first.
// Components merge with a lock-free union-find; edges of a round are written
// in order of each component's lowest point index (the reference's dict
// insertion order).
#include "mst.cuh"
#include "radius.cuh"
#include "primitives.cuh"
#include "reftree.cuh"
#include "uf.cuh"

#include <memory>

namespace fhg {
namespace {

constexpr int kSW = 4;        // warps per block, search kernel
// A round's search runs on a list of the searching points when they are fewer
// than kSparseNum / kSparseDen of all points.
constexpr int64_t kSparseNum = 1, kSparseDen = 4;
constexpr int kStack = 64;
constexpr int kMaxRounds = 64;
constexpr int kLocalLevels = 4;  // first search pass: subtrees of up to 16 buckets
constexpr int32_t kEmpty = -2;  // node_comp of a node with no points
constexpr int32_t kMixed = -1;  // node_comp of a node spanning components

__device__ __forceinline__ unsigned long long pack_key(float w, int32_t lo) {
    return ((unsigned long long)__float_as_uint(w) << 32) | (uint32_t)lo;
}
__device__ __forceinline__ float key_weight(unsigned long long k) {
    return __uint_as_float((uint32_t)(k >> 32));
}

// ------------------------------------------------------------- kNN to core
// core2 = squared distance to the k-th neighbour (itself included); +inf when
// there are fewer than k points, 0 for min_samples <= 1 (boruvka.py:581-601).
// open[p] arrives as the kNN kernel's boundary-tie flag and leaves as "a seed
// of weight core2[p] is not provably final": some point outside p's list may
// lie within core2[p] in squared distance (the core value passes the list's
// k-th squared distance, or reaches it while another point ties with it).
__device__ __forceinline__ int8_t seed_open(float c, float kth, int8_t tie) {
    return (!(c < kth) && (c > kth || tie)) ? 1 : 0;
}
__global__ void core_from_knn_kernel(int64_t n, int kk, int k, int ms,
                                     const float* __restrict__ knn_d_s, float* __restrict__ core2,
                                     int8_t* __restrict__ open) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float kth = knn_d_s[p * kk + kk - 1];
    const float c = ms <= 1 ? 0.0f : (k > kk ? INFINITY : kth);
    core2[p] = c;
    open[p] = seed_open(c, kth, open[p]);
}

// Weighted core distance (boruvka.py:527 sample_weight_core_distance): the
// plain distance (sqrt of the squared one, boruvka.py:563 queries without
// output_rdist) to the first neighbour at which the running weight, the
// point's own included, reaches min_samples.  Slots past the list are the
// reference's padding (+inf, index -1 -> the weight of the last point).
__global__ void weighted_core_kernel(int64_t n, int kk, int kq, int ms,
                                     const float* __restrict__ knn_d_s,
                                     const int32_t* __restrict__ knn_s,
                                     const float* __restrict__ w_s, float w_last,
                                     float* __restrict__ core2, int8_t* __restrict__ open) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    double total = 0.0;
    int j = 0;
    while (total < (double)ms && j < kq) {
        const int32_t q = j < kk ? knn_s[p * kk + j] : -1;
        total += (double)(q >= 0 ? w_s[q] : w_last);
        ++j;
    }
    const int jj = j > 0 ? j - 1 : kq - 1;
    const float c = jj < kk ? __fsqrt_rn(knn_d_s[p * kk + jj]) : INFINITY;
    core2[p] = c;
    open[p] = seed_open(c, knn_d_s[p * kk + kk - 1], open[p]);
}
__global__ void gather_weights_kernel(int64_t n, const int32_t* __restrict__ orig,
                                      const float* __restrict__ w, float* __restrict__ w_s) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) w_s[p] = w[orig[p]];
}

// Core distances in caller order; neighbour columns past the kNN list (the
// reference's padding when k exceeds the point count) are -1.  The kNN kernel
// writes the other neighbour columns itself.
__global__ void outputs_kernel(int64_t n, int kk, int k, const int32_t* __restrict__ orig,
                               const float* __restrict__ core2, float* __restrict__ core_o,
                               int32_t* __restrict__ nbr_o) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int64_t o = orig[p];
    if (core_o) core_o[o] = __fsqrt_rn(core2[p]);
    if (nbr_o)
        for (int j = kk > 1 ? kk : 1; j < k; ++j) nbr_o[o * (k - 1) + j - 1] = -1;
}

// ----------------------------------------------------------------- round 0
// plain_d: the weighted path's round 0 works on plain (not squared) distances.
__global__ void round0_kernel(int64_t n, int k, const int32_t* __restrict__ knn_s,
                              const float* __restrict__ knn_d, const float* __restrict__ core2,
                              int plain_d, int32_t* __restrict__ target, float* __restrict__ w0,
                              int* __restrict__ eq_flag) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float cp = core2[p];
    int32_t t = -1;
    float w = 0.0f;
    for (int j = 1; j < k; ++j) {
        int32_t q = knn_s[p * k + j];
        if (q < 0) break;
        float cq = core2[q];
        if (cp >= cq) {
            if (q != p) {
                t = q;
                const float d = knn_d[p * k + j];
                w = fmaxf(cp, plain_d ? __fsqrt_rn(d) : d);
                if (cq == cp) atomicOr(eq_flag, 1);
            }
            break;
        }
    }
    target[p] = t;
    w0[p] = w;
}

__global__ void iota_kernel(int32_t* a, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = (int32_t)i;
}

__global__ void union_targets_kernel(int32_t* par, const int32_t* __restrict__ target, int64_t n) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int32_t t = target[p];
    if (t >= 0) uf_union(par, (int32_t)p, t);
}

__global__ void flatten_kernel(int32_t* par, int32_t* __restrict__ comp, int64_t n) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    comp[p] = uf_find(par, (int32_t)p);
}

// Functional-graph cycle detection by pointer doubling (only run when some
// round-0 link joins two equal core distances).
__global__ void cyc_init_kernel(int64_t n, const int32_t* __restrict__ target,
                                const int32_t* __restrict__ orig, int32_t* nxt, int32_t* mx) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    nxt[p] = target[p] >= 0 ? target[p] : (int32_t)p;
    mx[p] = orig[p];
}
// `changed` (nullable) is set when some node's window maximum grew.  A step
// that grows none has converged: every node's maximum is then at least the
// next window's, and by induction the maximum over all it reaches.
__global__ void cyc_step_kernel(int64_t n, const int32_t* __restrict__ nxt,
                                const int32_t* __restrict__ mx, int32_t* __restrict__ nxt2,
                                int32_t* __restrict__ mx2, int* __restrict__ changed) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int32_t q = nxt[p];
    nxt2[p] = nxt[q];
    const int32_t a = mx[p], b = mx[q];
    mx2[p] = max(a, b);
    if (changed && b > a) *changed = 1;
}
__global__ void cyc_drop_kernel(int64_t n, const int32_t* __restrict__ nxt,
                                const int32_t* __restrict__ mx, const int32_t* __restrict__ orig,
                                int32_t* __restrict__ target) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    if (target[p] >= 0 && mx[nxt[p]] == orig[p]) target[p] = -1;
}

// `by` (nullable) numbers the points for the edge order: caller indices, or
// NULL for the index positions themselves.
__global__ void r0_flags_kernel(int64_t n, const int32_t* __restrict__ target,
                                const int32_t* __restrict__ by, uint32_t* __restrict__ flag) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    flag[by ? by[p] : p] = target[p] >= 0 ? 1u : 0u;
}
__global__ void r0_emit_kernel(int64_t n, const int32_t* __restrict__ target,
                               const float* __restrict__ w0, const int32_t* __restrict__ orig,
                               const int32_t* __restrict__ by, const uint32_t* __restrict__ pos,
                               int32_t* __restrict__ src, int32_t* __restrict__ dst,
                               float* __restrict__ w2) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int32_t t = target[p];
    if (t < 0) return;
    int32_t op = orig[p];
    uint32_t i = pos[by ? by[p] : p];
    src[i] = op;
    dst[i] = orig[t];
    w2[i] = w0[p];
}

__global__ void cmin_init_kernel(int64_t n, int32_t* cmin) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) cmin[p] = INT32_MAX;
}
__global__ void cmin_points_kernel(int64_t n, const int32_t* __restrict__ comp,
                                   const int32_t* __restrict__ orig, int32_t* cmin) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) atomicMin(&cmin[comp[p]], orig[p]);
}
__global__ void rep_flags_kernel(int64_t n, const int32_t* __restrict__ comp,
                                 uint32_t* __restrict__ flag) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) flag[p] = comp[p] == (int32_t)p ? 1u : 0u;
}
__global__ void compact_kernel(int64_t n, const uint32_t* __restrict__ flag,
                               const uint32_t* __restrict__ pos, const int32_t* __restrict__ src,
                               int32_t* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flag[i]) out[pos[i]] = src ? src[i] : (int32_t)i;
}

// ---------------------------------------------------------- per round: nodes
// Per node: x = its single component (node_comp, boruvka.py:98-124), kMixed
// or kEmpty; y = bits of the least core distance of its points.  Every edge
// into the node weighs at least that core distance, so a node whose least
// core distance exceeds a query's threshold is skipped like a distant one.
__global__ void node_comp_leaf_kernel(const int32_t* __restrict__ comp,
                                      const float* __restrict__ core2, int64_t n,
                                      int64_t nleaves, int64_t slots, int2* __restrict__ nc) {
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (leaf >= slots) return;
    int64_t i = leaf * kLeaf + lane;
    bool valid = leaf < nleaves && i < n;
    int32_t c = valid ? comp[i] : 0;
    // non-negative floats order like their bit patterns
    int32_t kb = valid ? __float_as_int(core2[i]) : INT32_MAX;
    int32_t c0 = __shfl_sync(kFull, c, 0);
    bool same = __all_sync(kFull, !valid || c == c0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) kb = min(kb, __shfl_xor_sync(kFull, kb, o));
    if (lane == 0)
        nc[slots - 1 + leaf] = make_int2(leaf >= nleaves ? kEmpty : (same ? c0 : kMixed), kb);
}
__global__ void node_comp_level_kernel(int2* __restrict__ nc, int64_t first, int64_t count) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    int64_t node = first + t;
    const int2 l = nc[2 * node + 1], r = nc[2 * node + 2];
    nc[node] = make_int2(l.x == kEmpty ? r.x : (r.x == kEmpty ? l.x : (l.x == r.x ? l.x : kMixed)),
                         min(l.y, r.y));
}

__global__ void reset_keys_kernel(const int32_t* __restrict__ reps, int64_t nrep,
                                  unsigned long long* keyA, uint32_t* keyB, int32_t* winner,
                                  int32_t* par) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrep) return;
    int32_t c = reps[i];
    keyA[c] = ~0ull;
    keyB[c] = 0xffffffffu;
    winner[c] = -1;
    par[c] = c;
}

// ------------------------------------------------------- per round: seeds
// Every point's best edge among its own kNN list (boruvka.py:474 uses the same
// lists), published to its component's key before any point searches, so the
// search starts from every component's seed bound.
// exhausted[p]: every kNN neighbour of p was already in p's component in an
// earlier round -- it stays so, as components only merge.
__global__ void seed_kernel(int64_t n, int k, const int32_t* __restrict__ knn_s,
                            const float* __restrict__ knn_d, const float* __restrict__ core2,
                            const int32_t* __restrict__ comp, const int32_t* __restrict__ orig,
                            unsigned long long* keyA, float* __restrict__ cand_w,
                            int32_t* __restrict__ cand_q, int8_t* __restrict__ exhausted,
                            int ref_ties) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int32_t c = comp[p];
    // The previous round's candidate of this point is still an edge out of
    // its component when its target has not been merged in: it seeds the
    // point's best (when it beats the kNN seed) and its component's key
    // before any point searches.  The search still finds every edge within
    // that bound, so the point's final candidate is its exact best.  (Its
    // weight equals the core distance only for a target inside the kNN
    // radius, which the kNN seed has already met, so the seed-finality rule
    // below is unaffected.)
    const int32_t oq = cand_q[p];
    const float ow = cand_w[p];
    const int32_t oo = (oq >= 0 && comp[oq] != c) ? orig[oq] : -1;
    float bw = INFINITY;
    int32_t bq = -1, bo = INT32_MAX;
    if (!exhausted[p]) {
        const float cp = core2[p];
        for (int j = 1; j < k; ++j) {
            int32_t qs = knn_s[p * k + j];
            if (qs < 0) break;
            if (comp[qs] == c) continue;
            float w = fmaxf(fmaxf(knn_d[p * k + j], cp), core2[qs]);
            int32_t o = orig[qs];
            if (w < bw || (w == bw && o < bo)) {
                bw = w;
                bq = qs;
                bo = o;
            }
        }
        if (bq < 0) exhausted[p] = 1;  // no other component in the kNN list
    }
    if (oo >= 0 && (ow < bw || (ow == bw && oo < bo))) {
        bw = ow;
        bq = oq;
        bo = oo;
    }
    cand_w[p] = bw;
    cand_q[p] = bq;
    if (bq >= 0) {
        unsigned long long key = pack_key(bw, ref_ties ? orig[p] : min(orig[p], bo));
        if (key < *(volatile unsigned long long*)&keyA[c]) atomicMin(&keyA[c], key);
    }
}

// ------------------------------------------------------- per round: search
// One warp per bucket of 32 query points, as in the kNN kernel.  A node is
// entered when some lane's point lies outside the node's single component
// (node_comp) and within that lane's threshold -- the smaller of its own best
// weight and its component's running best (boruvka.py:182-191).  Candidates
// of a leaf are staged in shared memory; a candidate in the query's own
// component, or with a core distance above the threshold, costs one compare.
//
// A point whose seed already weighs its own core distance (the least weight
// any of its edges can have) is settled without a search when every point
// at that distance is in its kNN list: the core distance is below the k-th
// distance, or no point outside the list lies exactly at the k-th distance
// (knn_open clear).  Any other edge then weighs more than the seed.
template <int DIM, int SP>
__global__ void __launch_bounds__(kSW * 32) search_kernel(
    IndexView ix, const int8_t* __restrict__ knn_open,
    const float* __restrict__ core2, const int32_t* __restrict__ comp,
    const int2* __restrict__ nc, unsigned long long* keyA, float* __restrict__ cand_w,
    int32_t* __restrict__ cand_q, int lvl_lo, int lvl_hi, const int32_t* __restrict__ plist,
    int64_t plen, int ref_ties) {
    __shared__ int32_t s_stack[kSW][kStack];
    __shared__ float4 s_xyz[kSW][32 * (SP / 4)];
    __shared__ int2 s_cc[kSW][32];      // (component, core bits)
    __shared__ int32_t s_orig[kSW][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // Dense: warp = bucket, lane = point.  Sparse (plist): warp = 32
    // consecutive entries of a list of the points still searching (in index
    // order), each searching from the root.
    const bool sparse = plist != nullptr;
    const int64_t leaf = (int64_t)blockIdx.x * kSW + warp;
    if (sparse ? leaf * 32 >= plen : leaf >= ix.nleaves) return;
    const int64_t li = leaf * 32 + lane;
    const int64_t p = sparse ? (li < plen ? plist[li] : 0) : leaf * kLeaf + lane;
    const bool valid = sparse ? li < plen : p < ix.n;
    int32_t c = -3;
    float cp = 0.0f, bw = INFINITY;
    int32_t bq = -1, bo = INT32_MAX;
    bool active = false;
    if (valid) {
        c = comp[p];
        cp = core2[p];
        bw = cand_w[p];
        bq = cand_q[p];
        if (bq >= 0) bo = ix.orig[bq];
        const bool settled = bq >= 0 && bw == cp && !knn_open[p];
        const float thr0 = fminf(bw, key_weight(*(volatile unsigned long long*)&keyA[c]));
        active = !settled && !(cp > thr0);
    }
    if (!__any_sync(kFull, active)) return;
    const int32_t seed_q = bq;
    float thr = bw;
    if (valid) thr = fminf(thr, key_weight(*(volatile unsigned long long*)&keyA[c]));
    float q[DIM];
    {
        float t[SP];
        if (valid) {
            load_pt<SP>(ix.pts, p, t);
        } else {
#pragma unroll
            for (int j = 0; j < SP; ++j) t[j] = 0.0f;
        }
#pragma unroll
        for (int j = 0; j < DIM; ++j) q[j] = t[j];
    }

    float4* xyz = s_xyz[warp];
    int2* cc = s_cc[warp];
    int32_t* co = s_orig[warp];

    auto scan_leaf = [&](int64_t lf, bool need) {
        const int64_t base = lf * kLeaf;
        const int cnt = (int)(ix.n - base < kLeaf ? ix.n - base : kLeaf);
        if (lane < cnt) {
            const float4* src = reinterpret_cast<const float4*>(ix.pts) + (base + lane) * (SP / 4);
#pragma unroll
            for (int h = 0; h < SP / 4; ++h) xyz[lane * (SP / 4) + h] = __ldg(src + h);
            cc[lane] = make_int2(comp[base + lane], __float_as_int(core2[base + lane]));
            co[lane] = ix.orig[base + lane];
        }
        __syncwarp();
        // Only candidates that can matter to some needing lane are visited:
        // a core distance within the largest needing threshold, and -- when
        // every needing lane is in one component -- outside it.  The best
        // edge is a minimum over (weight, index), so the order of the visits
        // does not change it.
        const unsigned needers = __ballot_sync(kFull, need);
        const float mthr =
            __uint_as_float(__reduce_max_sync(kFull, need ? __float_as_uint(thr) : 0u));
        const int32_t c0 = __shfl_sync(kFull, c, __ffs(needers) - 1);
        const bool one_comp = __all_sync(kFull, !need || c == c0);
        bool relevant = false;
        if (lane < cnt) {
            const int2 mine = cc[lane];
            relevant = !(__int_as_float(mine.y) > mthr) && !(one_comp && mine.x == c0);
        }
        for (unsigned todo = __ballot_sync(kFull, relevant); todo; todo &= todo - 1u) {
            const int t = __ffs(todo) - 1;
            const int2 tcc = cc[t];
            const float tk = __int_as_float(tcc.y);
            if (need && tcc.x != c && tk <= thr) {
                float x[SP];
#pragma unroll
                for (int h = 0; h < SP / 4; ++h) {
                    float4 v = xyz[t * (SP / 4) + h];
                    x[4 * h] = v.x; x[4 * h + 1] = v.y; x[4 * h + 2] = v.z; x[4 * h + 3] = v.w;
                }
                const float w = fmaxf(fmaxf(rdist_rn<DIM>(q, x), cp), tk);
                if (w <= bw) {
                    const int32_t to = co[t];
                    if (w < bw || to < bo) {
                        bw = w;
                        bq = (int32_t)(base + t);
                        bo = to;
                        thr = fminf(thr, bw);
                    }
                }
            }
        }
        __syncwarp();
        if (active) {
            thr = fminf(thr, key_weight(*(volatile unsigned long long*)&keyA[c]));
            active = !(cp > thr);
        }
    };

    const int64_t first_leaf_node = ix.slots - 1;
    const int64_t home_node = first_leaf_node + (sparse ? 0 : leaf);
    // A home bucket spanning several components holds the nearest candidates.
    const bool home_first = !sparse && lvl_lo == 0 && nc[home_node].x == kMixed;
    if (home_first && __any_sync(kFull, active)) scan_leaf(leaf, active);

    // Walk up from the home bucket to the root, searching the sibling subtree
    // at every ancestor (nearest subtrees first).  As in the kNN walk,
    // children are tested when their parent is expanded and only needed ones
    // are pushed; a bucket's test is repeated from registers right before it
    // is scanned.  A lane's key for a node is max(box bound, least core) when
    // the node holds points of another component, else +inf; the node is
    // needed when the key is within the lane's threshold.
    int32_t* st = s_stack[warp];
    auto other = [&](int2 ncn) { return ncn.x != c && ncn.x != kEmpty; };
    // (Sparse: one pass over the whole tree from the root, children of least
    // bound over the searching lanes first.)
    int64_t x = home_node;
    if (!sparse)
        for (int lv = 0; lv < lvl_lo && x > 0; ++lv) x = (x - 1) >> 1;
    for (int lv = lvl_lo; sparse ? lv == lvl_lo : (lv < lvl_hi && x > 0); ++lv) {
        const int32_t sib = sparse ? 0 : (int32_t)((x & 1) ? x + 1 : x - 1);
        // children nearer the home bucket in Morton order first
        const bool right_side = (x & 1) != 0;
        if (!sparse) x = (x - 1) >> 1;
        {
            const int2 ncn = nc[sib];
            bool need = active && other(ncn) && !(__int_as_float(ncn.y) > thr);
            if (need) {
                float b[2 * SP];
                load_box<SP>(ix.box, sib, b);
                need = box_lb_n<DIM, SP>(b, q) <= thr;
            }
            if (!__any_sync(kFull, need)) continue;
            if (sib >= first_leaf_node) {
                scan_leaf(sib - first_leaf_node, need);
                continue;
            }
        }
        int sp = 1;
        if (lane == 0) st[0] = sib;
        __syncwarp();
        while (sp > 0) {
            --sp;
            const int32_t node = st[sp];
            __syncwarp();
            const int32_t l = 2 * node + 1, r = l + 1;
            const int2 ncl = nc[l], ncr = nc[r];
            bool nl = active && other(ncl) && !(__int_as_float(ncl.y) > thr);
            bool nr = active && other(ncr) && !(__int_as_float(ncr.y) > thr);
            const bool pl = __any_sync(kFull, nl), pr = __any_sync(kFull, nr);
            if (!pl && !pr) continue;
            float bl[2 * SP], br[2 * SP];
            float kl = INFINITY, kr = INFINITY;
            if (pl) {
                load_box<SP>(ix.box, l, bl);
                if (other(ncl)) kl = fmaxf(box_lb_n<DIM, SP>(bl, q), __int_as_float(ncl.y));
                nl = nl && kl <= thr;
            }
            if (pr) {
                load_box<SP>(ix.box, r, br);
                if (other(ncr)) kr = fmaxf(box_lb_n<DIM, SP>(br, q), __int_as_float(ncr.y));
                nr = nr && kr <= thr;
            }
            const bool al = __any_sync(kFull, nl), ar = __any_sync(kFull, nr);
            if (!al && !ar) continue;
            bool left_first = !(al && ar) ? al : right_side;
            if (sparse && al && ar)  // non-negative floats order like their bits
                left_first = __reduce_min_sync(kFull, nl ? __float_as_uint(kl) : 0x7f800000u) <=
                             __reduce_min_sync(kFull, nr ? __float_as_uint(kr) : 0x7f800000u);
            if (l >= first_leaf_node) {
                // thresholds may shrink while the first bucket is scanned
                const int32_t n1 = left_first ? l : r, n2 = left_first ? r : l;
                if (left_first ? al : ar) scan_leaf(n1 - first_leaf_node, left_first ? nl : nr);
                if (left_first ? ar : al) {
                    const bool need2 = active && (left_first ? kr : kl) <= thr;
                    if (__any_sync(kFull, need2)) scan_leaf(n2 - first_leaf_node, need2);
                }
            } else {
                const int32_t nearc = left_first ? l : r, farc = left_first ? r : l;
                const bool an = left_first ? al : ar, af = left_first ? ar : al;
                if (lane == 0) {
                    int t = sp;
                    if (af) st[t++] = farc;
                    if (an) st[t] = nearc;
                }
                sp += (an ? 1 : 0) + (af ? 1 : 0);
                __syncwarp();
            }
        }
    }
    if (!valid || bq == seed_q) return;
    cand_w[p] = bw;
    cand_q[p] = bq;
    unsigned long long key = pack_key(bw, ref_ties ? ix.orig[p] : min(ix.orig[p], bo));
    if (key < *(volatile unsigned long long*)&keyA[c]) atomicMin(&keyA[c], key);
}

// The points that start the global pass searching (as search_kernel decides).
__global__ void searching_flags_kernel(int64_t n, const int8_t* __restrict__ knn_open,
                                       const float* __restrict__ core2,
                                       const int32_t* __restrict__ comp,
                                       const unsigned long long* __restrict__ keyA,
                                       const float* __restrict__ cand_w,
                                       const int32_t* __restrict__ cand_q,
                                       uint32_t* __restrict__ flag) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float cp = core2[p], bw = cand_w[p];
    const bool settled = cand_q[p] >= 0 && bw == cp && !knn_open[p];
    const float thr0 = fminf(bw, key_weight(keyA[comp[p]]));
    flag[p] = (!settled && !(cp > thr0)) ? 1u : 0u;
}
__global__ void iota_list_kernel(int64_t n, const uint32_t* __restrict__ flag,
                                 const uint32_t* __restrict__ pos, int32_t* __restrict__ list) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n && flag[p]) list[pos[p]] = (int32_t)p;
}

__global__ void stage_b_kernel(int64_t n, const int32_t* __restrict__ comp,
                               const int32_t* __restrict__ orig, const float* __restrict__ cand_w,
                               const int32_t* __restrict__ cand_q,
                               const unsigned long long* __restrict__ keyA, uint32_t* keyB) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int32_t q = cand_q[p];
    if (q < 0) return;
    int32_t c = comp[p], op = orig[p], oq = orig[q];
    if (keyA[c] == pack_key(cand_w[p], min(op, oq))) atomicMin(&keyB[c], (uint32_t)max(op, oq));
}
__global__ void stage_c_kernel(int64_t n, const int32_t* __restrict__ comp,
                               const int32_t* __restrict__ orig, const float* __restrict__ cand_w,
                               const int32_t* __restrict__ cand_q,
                               const unsigned long long* __restrict__ keyA,
                               const uint32_t* __restrict__ keyB, int32_t* winner) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int32_t q = cand_q[p];
    if (q < 0) return;
    int32_t c = comp[p], op = orig[p], oq = orig[q];
    if (keyA[c] == pack_key(cand_w[p], min(op, oq)) && keyB[c] == (uint32_t)max(op, oq))
        winner[c] = (int32_t)p;
}

__global__ void select_kernel(const int32_t* __restrict__ reps, int64_t nrep,
                              const int32_t* __restrict__ winner,
                              const int32_t* __restrict__ cand_q,
                              const int32_t* __restrict__ comp, int32_t* __restrict__ tgt,
                              int* __restrict__ missing) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrep) return;
    int32_t c = reps[i], p = winner[c];
    if (p < 0) {
        tgt[c] = -1;
        atomicOr(missing, 1);
        return;
    }
    tgt[c] = comp[cand_q[p]];
}

__global__ void emit_flags_kernel(const int32_t* __restrict__ reps, int64_t nrep,
                                  const int32_t* __restrict__ tgt,
                                  const int32_t* __restrict__ cmin, uint32_t* __restrict__ flag) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrep) return;
    int32_t c = reps[i], t = tgt[c];
    if (t < 0) return;
    bool mutual = tgt[t] == c;
    if (!mutual || cmin[c] < cmin[t]) flag[cmin[c]] = 1u;
}

__global__ void emit_write_kernel(const int32_t* __restrict__ reps, int64_t nrep,
                                  const int32_t* __restrict__ tgt,
                                  const int32_t* __restrict__ cmin,
                                  const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos,
                                  const int32_t* __restrict__ winner,
                                  const int32_t* __restrict__ cand_q,
                                  const float* __restrict__ cand_w,
                                  const int32_t* __restrict__ orig, int64_t base,
                                  int32_t* __restrict__ src, int32_t* __restrict__ dst,
                                  float* __restrict__ w2) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrep) return;
    int32_t c = reps[i];
    if (tgt[c] < 0 || !flag[cmin[c]]) return;
    int32_t p = winner[c];
    int64_t e = base + pos[cmin[c]];
    src[e] = orig[p];
    dst[e] = orig[cand_q[p]];
    w2[e] = cand_w[p];
}

__global__ void emit_clear_kernel(const int32_t* __restrict__ reps, int64_t nrep,
                                  const int32_t* __restrict__ cmin, uint32_t* __restrict__ flag) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nrep) flag[cmin[reps[i]]] = 0u;
}

__global__ void union_reps_kernel(const int32_t* __restrict__ reps, int64_t nrep,
                                  const int32_t* __restrict__ tgt, int32_t* par) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrep) return;
    int32_t c = reps[i], t = tgt[c];
    if (t >= 0) uf_union(par, c, t);
}
__global__ void relabel_points_kernel(int64_t n, int32_t* par, int32_t* __restrict__ comp) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) comp[p] = uf_find(par, comp[p]);
}
__global__ void merge_cmin_kernel(const int32_t* __restrict__ reps, int64_t nrep, int32_t* par,
                                  int32_t* cmin, uint32_t* __restrict__ keep) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrep) return;
    int32_t c = reps[i];
    int32_t r = uf_find(par, c);
    keep[i] = r == c ? 1u : 0u;
    if (r != c) atomicMin(&cmin[r], cmin[c]);
}

// ------------------------------------------- reference tie mode, per round
// The reference's choice of a component's edge (boruvka.py:34-60 over the
// candidates of boruvka.py:290-331, its loops run in order): the point of
// lowest caller index among those attaining the component's least weight w,
// and that point's first candidate at weight w in its KD-tree walk.  (The
// shared bound never cuts that point's search short: when it runs, the bound
// only holds weights above w.)  With the component keys packed as (weight,
// caller index of the choosing point), the key's low word is that point.
__global__ void ref_winner_kernel(const int32_t* __restrict__ reps, int64_t nrep,
                                  const unsigned long long* __restrict__ keyA,
                                  const int32_t* __restrict__ rank, int32_t* __restrict__ winner) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrep) return;
    const int32_t c = reps[i];
    const unsigned long long key = keyA[c];
    winner[c] = key == ~0ull ? -1 : rank[(uint32_t)(key & 0xffffffffu)];
}

// One warp per component: every point of another component at exactly the
// winner's weight w (max(rdist, core, core) == w, the search's expression)
// is found by a walk of the bucket tree limited to nodes that can hold one;
// the reference's walk meets them in its own tree's depth-first order, and
// the first of them in that order (ref_before) is the edge's far end.
template <int DIM, int SP>
__global__ void __launch_bounds__(kSW * 32) tie_walk_kernel(
    IndexView ix, RefTreeView rt, const int32_t* __restrict__ reps, int64_t nrep,
    const int32_t* __restrict__ comp, const float* __restrict__ core2,
    const int2* __restrict__ nc, const int32_t* __restrict__ winner,
    const float* __restrict__ cand_w, int32_t* __restrict__ cand_q, int32_t* __restrict__ tgt,
    int* __restrict__ missing) {
    __shared__ int32_t s_stack[kSW][kStack];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t i = (int64_t)blockIdx.x * kSW + warp;
    if (i >= nrep) return;
    const int32_t c = reps[i];
    const int32_t p = winner[c];
    if (p < 0) {
        if (lane == 0) {
            tgt[c] = -1;
            atomicOr(missing, 1);
        }
        return;
    }
    const float w = cand_w[p], cp = core2[p];
    float q[DIM];
    {
        float t[SP];
        load_pt<SP>(ix.pts, p, t);
#pragma unroll
        for (int j = 0; j < DIM; ++j) q[j] = t[j];
    }
    int32_t best = -1;
    int64_t best_pos = -1;
    int32_t* st = s_stack[warp];
    const int64_t first_leaf = ix.slots - 1;
    auto wanted = [&](int64_t node) {
        const int2 ncn = nc[node];
        if (ncn.x == c || ncn.x == kEmpty || __int_as_float(ncn.y) > w) return false;
        float b[2 * SP];
        load_box<SP>(ix.box, node, b);
        return box_lb_n<DIM, SP>(b, q) <= w;
    };
    int sp = 0;
    if (wanted(0)) {
        if (lane == 0) st[0] = 0;
        sp = 1;
    }
    __syncwarp();
    while (sp > 0) {
        --sp;
        const int32_t node = st[sp];
        __syncwarp();
        if (node >= first_leaf) {
            const int64_t leaf = node - first_leaf;
            const int64_t qp = leaf * kLeaf + lane;
            int32_t my = -1;
            int64_t mypos = -1;
            if (leaf < ix.nleaves && qp < ix.n && comp[qp] != c) {
                const float ck = core2[qp];
                if (!(ck > w)) {
                    float x[SP];
                    load_pt<SP>(ix.pts, qp, x);
                    const float wt = fmaxf(fmaxf(rdist_rn<DIM>(q, x), cp), ck);
                    if (wt == w) {
                        my = (int32_t)qp;
                        mypos = rt.pos[ix.orig[qp]];
                    }
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const int32_t other = __shfl_xor_sync(kFull, my, o);
                const int64_t opos = __shfl_xor_sync(kFull, mypos, o);
                if (other >= 0 && (my < 0 || ref_before(rt, q, opos, mypos))) {
                    my = other;
                    mypos = opos;
                }
            }
            if (my >= 0 && (best < 0 || ref_before(rt, q, mypos, best_pos))) {
                best = my;
                best_pos = mypos;
            }
            continue;
        }
        const int32_t l = 2 * node + 1, r = l + 1;
        const bool wl = wanted(l), wr = wanted(r);
        if (lane == 0) {
            int t = sp;
            if (wl) st[t++] = l;
            if (wr) st[t] = r;
        }
        sp += (wl ? 1 : 0) + (wr ? 1 : 0);
        __syncwarp();
    }
    if (lane == 0) {
        if (best < 0) {
            tgt[c] = -1;
            atomicOr(missing, 2);
        } else {
            cand_q[p] = best;
            tgt[c] = comp[best];
        }
    }
}

// The reference adds the components' edges in its dict order (each
// component's lowest caller index, cmin) and skips an edge whose ends are
// already joined.  The edges form a functional graph on components; an edge
// is skipped exactly when it closes its part's cycle, i.e. it is the cycle's
// edge of largest cmin.  Pointer doubling finds every cycle's largest cmin.
__global__ void crep_init_kernel(const int32_t* __restrict__ reps, int64_t nrep,
                                 const int32_t* __restrict__ tgt, const int32_t* __restrict__ cmin,
                                 int32_t* __restrict__ nxt, int32_t* __restrict__ mx) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrep) return;
    const int32_t c = reps[i];
    nxt[c] = tgt[c] >= 0 ? tgt[c] : c;
    mx[c] = cmin[c];
}
__global__ void crep_step_kernel(const int32_t* __restrict__ reps, int64_t nrep,
                                 const int32_t* __restrict__ nxt, const int32_t* __restrict__ mx,
                                 int32_t* __restrict__ nxt2, int32_t* __restrict__ mx2,
                                 int* __restrict__ changed) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrep) return;
    const int32_t c = reps[i], x = nxt[c];
    nxt2[c] = nxt[x];
    const int32_t a = mx[c], b = mx[x];
    mx2[c] = max(a, b);
    if (changed && b > a) *changed = 1;
}
__global__ void crep_drop_kernel(const int32_t* __restrict__ reps, int64_t nrep,
                                 const int32_t* __restrict__ nxt, const int32_t* __restrict__ mx,
                                 const int32_t* __restrict__ cmin, int32_t* __restrict__ tgt) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrep) return;
    const int32_t c = reps[i];
    if (tgt[c] >= 0 && mx[nxt[c]] == cmin[c]) tgt[c] = -1;
}
__global__ void ref_emit_flags_kernel(const int32_t* __restrict__ reps, int64_t nrep,
                                      const int32_t* __restrict__ tgt,
                                      const int32_t* __restrict__ cmin, uint32_t* __restrict__ flag) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrep) return;
    const int32_t c = reps[i];
    if (tgt[c] >= 0) flag[cmin[c]] = 1u;
}

__global__ void finalize_edges_kernel(int64_t m, const int32_t* __restrict__ src,
                                      const int32_t* __restrict__ dst,
                                      const float* __restrict__ w2, double* __restrict__ edges) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    edges[3 * e + 0] = (double)src[e];
    edges[3 * e + 1] = (double)dst[e];
    edges[3 * e + 2] = __dsqrt_rn((double)w2[e]);
}

template <int DIM>
int launch_search(const fhg_index& ix, const int8_t* knn_open,
                  const float* core2, const int32_t* comp, const int2* nc,
                  unsigned long long* keyA, float* cand_w, int32_t* cand_q, bool* try_sparse,
                  int ref_ties, cudaStream_t s) {
    constexpr int SP = DIM <= 4 ? 4 : (DIM <= 8 ? 8 : DIM);  // as in the kNN kernel
    const int64_t n = ix.n;
    // When few points search (early rounds: most points' best edge is settled
    // by the seeds), one pass runs on a list of them, 32 to a warp, each from
    // the root -- instead of a warp per bucket walking for one or two of its
    // lanes.  Searching only grows with the components, so after the first
    // dense round the list is not made again.
    if (*try_sparse) {
        Workspace tmp(s);
        uint32_t *flag, *pos, *cnt;
        int32_t* list;
        FHG_TRY(tmp.alloc(&flag, (size_t)n));
        FHG_TRY(tmp.alloc(&pos, (size_t)n));
        FHG_TRY(tmp.alloc(&list, (size_t)n));
        FHG_TRY(tmp.alloc(&cnt, 1));
        ::fhg::note_launch();
        searching_flags_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, knn_open, core2, comp, keyA,
                                                                  cand_w, cand_q, flag);
        FHG_CUDA(cudaGetLastError());
        FHG_TRY(scan_exclusive_u32(tmp, flag, pos, n, cnt));
        uint32_t h_cnt = 0;
        FHG_CUDA(cudaMemcpyAsync(&h_cnt, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        FHG_CUDA(cudaStreamSynchronize(s));
        const int64_t ns = h_cnt;
        if (ns == 0) return FHG_OK;
        *try_sparse = ns * kSparseDen < n * kSparseNum;
        if (*try_sparse) {
            ::fhg::note_launch();
            iota_list_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, flag, pos, list);
            FHG_CUDA(cudaGetLastError());
            Stage stage(s, "search_kernel");
            ::fhg::note_launch();
            search_kernel<DIM, SP><<<grid_for((ns + 31) / 32, kSW), kSW * 32, 0, s>>>(
                view_of(ix), knn_open, core2, comp, nc, keyA, cand_w, cand_q, 0, 64, list, ns,
                ref_ties);
            FHG_CUDA(cudaGetLastError());
            return FHG_OK;
        }
    }
    // Dense: a local pass (home bucket and the kLocalLevels nearest sibling
    // subtrees), then the rest of the walk -- every component's bound from
    // its nearby candidates is published before any point searches far away.
    const int spans[2][2] = {{0, kLocalLevels}, {kLocalLevels, 64}};
    for (const auto& sp : spans) {
        Stage stage(s, "search_kernel");
        ::fhg::note_launch();
        search_kernel<DIM, SP><<<grid_for(ix.nleaves, kSW), kSW * 32, 0, s>>>(
            view_of(ix), knn_open, core2, comp, nc, keyA, cand_w, cand_q, sp[0], sp[1],
            nullptr, 0, ref_ties);
        FHG_CUDA(cudaGetLastError());
    }
    return FHG_OK;
}

template <int DIM>
int launch_tie_walk(const fhg_index& ix, const RefTree& rt, const int32_t* reps, int64_t nrep,
                    const int32_t* comp, const float* core2, const int2* nc,
                    const int32_t* winner, const float* cand_w, int32_t* cand_q, int32_t* tgt,
                    int* missing, cudaStream_t s) {
    constexpr int SP = DIM <= 4 ? 4 : (DIM <= 8 ? 8 : DIM);
    if (nrep <= 0) return FHG_OK;
    Stage stage(s, "tie_walk_kernel");
    ::fhg::note_launch();
    tie_walk_kernel<DIM, SP><<<grid_for(nrep, kSW), kSW * 32, 0, s>>>(
        view_of(ix), view_of(rt), reps, nrep, comp, core2, nc, winner, cand_w, cand_q, tgt,
        missing);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

int tie_walk(const fhg_index& ix, const RefTree& rt, const int32_t* reps, int64_t nrep,
             const int32_t* comp, const float* core2, const int2* nc, const int32_t* winner,
             const float* cand_w, int32_t* cand_q, int32_t* tgt, int* missing, cudaStream_t s) {
#define FHG_TW(D) launch_tie_walk<D>(ix, rt, reps, nrep, comp, core2, nc, winner, cand_w, cand_q, \
                                     tgt, missing, s)
    switch (ix.d) {
        case 1: return FHG_TW(1);
        case 2: return FHG_TW(2);
        case 3: return FHG_TW(3);
        case 4: return FHG_TW(4);
        case 5: return FHG_TW(5);
        case 6: return FHG_TW(6);
        case 7: return FHG_TW(7);
        case 8: return FHG_TW(8);
        default:
            if (ix.d <= 16) return FHG_TW(16);
            return FHG_TW(32);
    }
#undef FHG_TW
}

int search_round(const fhg_index& ix, int k, const int32_t* knn_s, const float* knn_d,
                 const int8_t* knn_open, int8_t* exhausted, const float* core2,
                 const int32_t* comp,
                 const int2* nc, unsigned long long* keyA, float* cand_w, int32_t* cand_q,
                 bool* try_sparse, int ref_ties, cudaStream_t s) {
    const int64_t n = ix.n;
    if (n > 0) {
        ::fhg::note_launch();
        seed_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, k, knn_s, knn_d, core2, comp, ix.orig,
                                                       keyA, cand_w, cand_q, exhausted, ref_ties);
        FHG_CUDA(cudaGetLastError());
    }
    switch (ix.d) {
        case 1: return launch_search<1>(ix, knn_open, core2, comp, nc, keyA, cand_w, cand_q, try_sparse, ref_ties, s);
        case 2: return launch_search<2>(ix, knn_open, core2, comp, nc, keyA, cand_w, cand_q, try_sparse, ref_ties, s);
        case 3: return launch_search<3>(ix, knn_open, core2, comp, nc, keyA, cand_w, cand_q, try_sparse, ref_ties, s);
        case 4: return launch_search<4>(ix, knn_open, core2, comp, nc, keyA, cand_w, cand_q, try_sparse, ref_ties, s);
        case 5: return launch_search<5>(ix, knn_open, core2, comp, nc, keyA, cand_w, cand_q, try_sparse, ref_ties, s);
        case 6: return launch_search<6>(ix, knn_open, core2, comp, nc, keyA, cand_w, cand_q, try_sparse, ref_ties, s);
        case 7: return launch_search<7>(ix, knn_open, core2, comp, nc, keyA, cand_w, cand_q, try_sparse, ref_ties, s);
        case 8: return launch_search<8>(ix, knn_open, core2, comp, nc, keyA, cand_w, cand_q, try_sparse, ref_ties, s);
        default:
            if (ix.d <= 16)
                return launch_search<16>(ix, knn_open, core2, comp, nc, keyA, cand_w, cand_q, try_sparse, ref_ties, s);
            return launch_search<32>(ix, knn_open, core2, comp, nc, keyA, cand_w, cand_q, try_sparse, ref_ties, s);
    }
}

#define LAUNCH(kernel, count, ...)                                                   \
    do {                                                                             \
        if ((count) > 0) {                                                           \
            ::fhg::note_launch(); \
            kernel<<<grid_for((count), 256), 256, 0, s>>>(__VA_ARGS__);              \
            FHG_CUDA(cudaGetLastError());                                            \
        }                                                                            \
    } while (0)

}  // namespace

// The tie rule of the calling host thread (fhg_set_tie_rule).
namespace {
thread_local int t_tie_rule = FHG_TIES_CANONICAL;
}
int tie_rule() { return t_tie_rule; }
int set_tie_rule(int rule) {
    const int old = t_tie_rule;
    t_tie_rule = rule;
    return old;
}

int finalize_edges(const MstResult& r, double* edges, cudaStream_t s) {
    LAUNCH(finalize_edges_kernel, r.m, r.m, r.src, r.dst, r.w2, edges);
    return FHG_OK;
}

int boruvka_mst(Workspace& ws, const fhg_index& ix, int min_samples, MstResult* out,
                float* core_o, int32_t* nbr_o, const float* weights, int weighted_k,
                bool any_order) {
    cudaStream_t s = ws.stream();
    const int64_t n = ix.n;
    const bool weighted = weights != nullptr && n > 1;
    const int ref_ties = tie_rule() == FHG_TIES_REFERENCE ? 1 : 0;
    // the reference's k (boruvka.py:561-585)
    const int kq = weighted ? weighted_k : (min_samples > 1 ? min_samples + 1 : 2);
    const int k = (int)(kq < n ? kq : n);  // neighbours that exist
    *out = MstResult();
    if (kq < 1) {
        set_error("weighted kNN: k = %d (2 * min_samples / mean weight) is below 1", kq);
        return FHG_ERR_INVALID;
    }
    // lists of up to 64 live in registers (and the reference tie mode's
    // re-query takes no more); longer ones in shared memory
    const int k_max = ref_ties ? 64 : kKnnMaxK;
    if (k > k_max) {
        if (weighted)
            set_error("weighted kNN: k = %d (2 * min_samples / mean weight) exceeds %d%s", kq,
                      k_max, ref_ties ? " in the reference tie mode" : "");
        else
            set_error("min_samples must be at most %d (got %d)%s", k_max - 1, min_samples,
                      ref_ties ? " in the reference tie mode" : "");
        return FHG_ERR_UNSUPPORTED;
    }
    const int64_t m_cap = n > 1 ? n - 1 : 1;
    FHG_TRY(ws.alloc(&out->src, (size_t)m_cap));
    FHG_TRY(ws.alloc(&out->dst, (size_t)m_cap));
    FHG_TRY(ws.alloc(&out->w2, (size_t)m_cap));

    float *knn_d, *core2, *knn_d_o = nullptr, *w0, *cand_w;
    int32_t *knn_s, *target, *par, *comp, *cmin, *reps, *reps2, *winner, *tgt,
        *cand_q;
    int2* nc;
    uint32_t *flag, *pos, *keyB, *cnt;
    unsigned long long* keyA;
    int* iflag;
    FHG_TRY(ws.alloc(&knn_d, (size_t)(n * k)));
    FHG_TRY(ws.alloc(&knn_s, (size_t)(n * k)));
    int8_t* knn_open;  // the kNN kernel's tie flags, then "seed not provably final"
    FHG_TRY(ws.alloc(&knn_open, (size_t)n));
    // the neighbours[:, 1:] matrix (kq - 1 columns) straight from the kNN kernel
    const RadiusUse* ru = k <= 64 ? radius_in_use() : nullptr;  // (radius passes: k <= 64)
    if (ru)
        FHG_TRY(knn_with_radius(ix, k, *ru, knn_d, knn_s, knn_d_o, nbr_o, s, knn_open, kq - 1, 1));
    else
        FHG_TRY(index_knn(ix, k, knn_d, knn_s, knn_d_o, nbr_o, s, knn_open, kq - 1, 1));
    // the reference tie mode breaks ties in the order of the reference's own
    // KD-tree, built here exactly; its kNN lists (and so round 0 and the
    // neighbour matrix) list equal distances in the order of the reference's
    // query and heap, and replace the engine's rows (the same distances)
    RefTree rt;
    if (ref_ties && n > 1) {
        FHG_TRY(ref_tree_build(ws, ix, &rt));
        FHG_TRY(ref_knn(rt, ix, kq, weighted, knn_open, knn_d, knn_s, nbr_o, kq - 1, s));
    }
    FHG_TRY(ws.alloc(&core2, (size_t)n));
    if (weighted) {
        float* w_s;
        float w_last = 0.0f;
        FHG_TRY(ws.alloc(&w_s, (size_t)n));
        LAUNCH(gather_weights_kernel, n, n, ix.orig, weights, w_s);
        FHG_CUDA(cudaMemcpyAsync(&w_last, weights + (n - 1), sizeof(float), cudaMemcpyDeviceToHost,
                                 s));
        FHG_CUDA(cudaStreamSynchronize(s));
        LAUNCH(weighted_core_kernel, n, n, k, kq, min_samples, knn_d, knn_s, w_s, w_last, core2,
               knn_open);
    } else {
        LAUNCH(core_from_knn_kernel, n, n, k, kq, min_samples, knn_d, core2, knn_open);
    }
    if (core_o || nbr_o)
        LAUNCH(outputs_kernel, n, n, k, kq, ix.orig, core2, core_o, nbr_o);
    if (n < 2) return FHG_OK;

    FHG_TRY(ws.alloc(&target, (size_t)n));
    FHG_TRY(ws.alloc(&w0, (size_t)n));
    FHG_TRY(ws.alloc(&par, (size_t)n));
    FHG_TRY(ws.alloc(&comp, (size_t)n));
    FHG_TRY(ws.alloc(&cmin, (size_t)n));
    FHG_TRY(ws.alloc(&flag, (size_t)n));
    FHG_TRY(ws.alloc(&pos, (size_t)n));
    FHG_TRY(ws.alloc(&cnt, 2));
    FHG_TRY(ws.alloc(&iflag, 2));
    FHG_CUDA(cudaMemsetAsync(iflag, 0, 2 * sizeof(int), s));

    // ---- round 0: kNN-seeded links (boruvka.py:474)
    std::unique_ptr<Stage> r0_stage(new Stage(s, "boruvka_round0"));
    LAUNCH(round0_kernel, n, n, k, knn_s, knn_d, core2, weighted ? 1 : 0, target, w0, iflag);
    int h_flag[2] = {0, 0};
    FHG_CUDA(cudaMemcpyAsync(h_flag, iflag, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    if (h_flag[0]) {
        int32_t *nxt, *mx, *nxt2, *mx2;
        FHG_TRY(ws.alloc(&nxt, (size_t)n));
        FHG_TRY(ws.alloc(&mx, (size_t)n));
        FHG_TRY(ws.alloc(&nxt2, (size_t)n));
        FHG_TRY(ws.alloc(&mx2, (size_t)n));
        LAUNCH(cyc_init_kernel, n, n, target, ix.orig, nxt, mx);
        // link chains are short: every fourth step reports whether it changed
        // anything, and the doubling stops at the first that did not
        int R = bits_for(n) + 1;
        for (int r = 0; r < R; ++r) {
            const bool check = (r & 3) == 3 && r + 1 < R;
            if (check) FHG_CUDA(cudaMemsetAsync(iflag, 0, sizeof(int), s));
            LAUNCH(cyc_step_kernel, n, n, nxt, mx, nxt2, mx2, check ? iflag : nullptr);
            int32_t* t1 = nxt; nxt = nxt2; nxt2 = t1;
            t1 = mx; mx = mx2; mx2 = t1;
            if (check) {
                int h_changed = 1;
                FHG_CUDA(cudaMemcpyAsync(&h_changed, iflag, sizeof(int), cudaMemcpyDeviceToHost, s));
                FHG_CUDA(cudaStreamSynchronize(s));
                if (!h_changed) break;
            }
        }
        LAUNCH(cyc_drop_kernel, n, n, nxt, mx, ix.orig, target);
    }
    // round-0 edges by caller index of the choosing point (the reference's
    // order), or by index position when the order does not matter
    const int32_t* by = any_order ? nullptr : ix.orig;
    LAUNCH(r0_flags_kernel, n, n, target, by, flag);
    FHG_TRY(scan_exclusive_u32(ws, flag, pos, n, cnt));
    LAUNCH(r0_emit_kernel, n, n, target, w0, ix.orig, by, pos, out->src, out->dst, out->w2);
    uint32_t h_cnt = 0;
    FHG_CUDA(cudaMemcpyAsync(&h_cnt, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    LAUNCH(iota_kernel, n, par, n);
    LAUNCH(union_targets_kernel, n, par, target, n);
    LAUNCH(flatten_kernel, n, par, comp, n);
    LAUNCH(cmin_init_kernel, n, n, cmin);
    LAUNCH(cmin_points_kernel, n, n, comp, ix.orig, cmin);
    FHG_CUDA(cudaStreamSynchronize(s));
    int64_t m = h_cnt;

    // representatives (component ids) in Morton order
    FHG_TRY(ws.alloc(&reps, (size_t)n));
    FHG_TRY(ws.alloc(&reps2, (size_t)n));
    LAUNCH(rep_flags_kernel, n, n, comp, flag);
    FHG_TRY(scan_exclusive_u32(ws, flag, pos, n, cnt));
    LAUNCH(compact_kernel, n, n, flag, pos, (const int32_t*)nullptr, reps);
    uint32_t h_ncomp = 0;
    FHG_CUDA(cudaMemcpyAsync(&h_ncomp, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    r0_stage.reset();
    FHG_CUDA(cudaStreamSynchronize(s));
    int64_t ncomp = h_ncomp;

    FHG_TRY(ws.alloc(&keyA, (size_t)n));
    FHG_TRY(ws.alloc(&keyB, (size_t)n));
    FHG_TRY(ws.alloc(&winner, (size_t)n));
    FHG_TRY(ws.alloc(&tgt, (size_t)n));
    FHG_TRY(ws.alloc(&nc, (size_t)ix.nnodes));
    FHG_TRY(ws.alloc(&cand_w, (size_t)n));
    FHG_TRY(ws.alloc(&cand_q, (size_t)n));
    FHG_CUDA(cudaMemsetAsync(cand_q, 0xff, sizeof(int32_t) * n, s));  // no candidate yet (-1)
    int8_t* exhausted;
    FHG_TRY(ws.alloc(&exhausted, (size_t)n));
    FHG_CUDA(cudaMemsetAsync(exhausted, 0, (size_t)n, s));
    uint32_t* kpos;
    FHG_TRY(ws.alloc(&kpos, (size_t)n));
    FHG_CUDA(cudaMemsetAsync(flag, 0, sizeof(uint32_t) * n, s));

    // the reference tie mode's pointer-doubling buffers
    int32_t *cy_nxt = nullptr, *cy_mx = nullptr, *cy_nxt2 = nullptr, *cy_mx2 = nullptr;
    if (ref_ties && ncomp > 1) {
        FHG_TRY(ws.alloc(&cy_nxt, (size_t)n));
        FHG_TRY(ws.alloc(&cy_mx, (size_t)n));
        FHG_TRY(ws.alloc(&cy_nxt2, (size_t)n));
        FHG_TRY(ws.alloc(&cy_mx2, (size_t)n));
    }

    int rounds = 0;
    bool try_sparse = true;  // until a round's global pass is dense
    while (ncomp > 1) {
        if (rounds >= kMaxRounds) {
            set_error("boruvka: no convergence after %d rounds (%lld components left)", rounds,
                      (long long)ncomp);
            return FHG_ERR_NO_CONVERGENCE;
        }
        profile_count("boruvka_components", (double)ncomp);  // C_r of the round
        {  // node_comp (boruvka.py:98-124), bottom-up
            Stage stage(s, "boruvka_nodes");
            LAUNCH(node_comp_leaf_kernel, ix.slots * 32, comp, core2, n, ix.nleaves, ix.slots, nc);
            for (int64_t width = ix.slots / 2; width >= 1; width /= 2)
                LAUNCH(node_comp_level_kernel, width, nc, width - 1, width);
            LAUNCH(reset_keys_kernel, ncomp, reps, ncomp, keyA, keyB, winner, par);
        }
        {
            Stage stage(s, "boruvka_search");
            FHG_TRY(search_round(ix, k, knn_s, knn_d, knn_open, exhausted, core2, comp, nc, keyA,
                                 cand_w, cand_q, &try_sparse, ref_ties, s));
        }
        Stage merge_stage(s, "boruvka_merge");
        FHG_CUDA(cudaMemsetAsync(iflag + 1, 0, sizeof(int), s));
        if (ref_ties) {
            LAUNCH(ref_winner_kernel, ncomp, reps, ncomp, keyA, ix.rank, winner);
            FHG_TRY(tie_walk(ix, rt, reps, ncomp, comp, core2, nc, winner, cand_w, cand_q, tgt,
                             iflag + 1, s));
            LAUNCH(crep_init_kernel, ncomp, reps, ncomp, tgt, cmin, cy_nxt, cy_mx);
            const int R = bits_for(ncomp) + 1;
            for (int r = 0; r < R; ++r) {
                const bool check = (r & 3) == 3 && r + 1 < R;
                if (check) FHG_CUDA(cudaMemsetAsync(iflag, 0, sizeof(int), s));
                LAUNCH(crep_step_kernel, ncomp, reps, ncomp, cy_nxt, cy_mx, cy_nxt2, cy_mx2,
                       check ? iflag : nullptr);
                int32_t* t1 = cy_nxt; cy_nxt = cy_nxt2; cy_nxt2 = t1;
                t1 = cy_mx; cy_mx = cy_mx2; cy_mx2 = t1;
                if (check) {
                    int h_changed = 1;
                    FHG_CUDA(cudaMemcpyAsync(&h_changed, iflag, sizeof(int),
                                             cudaMemcpyDeviceToHost, s));
                    FHG_CUDA(cudaStreamSynchronize(s));
                    if (!h_changed) break;
                }
            }
            LAUNCH(crep_drop_kernel, ncomp, reps, ncomp, cy_nxt, cy_mx, cmin, tgt);
            LAUNCH(ref_emit_flags_kernel, ncomp, reps, ncomp, tgt, cmin, flag);
        } else {
            LAUNCH(stage_b_kernel, n, n, comp, ix.orig, cand_w, cand_q, keyA, keyB);
            LAUNCH(stage_c_kernel, n, n, comp, ix.orig, cand_w, cand_q, keyA, keyB, winner);
            LAUNCH(select_kernel, ncomp, reps, ncomp, winner, cand_q, comp, tgt, iflag + 1);
            LAUNCH(emit_flags_kernel, ncomp, reps, ncomp, tgt, cmin, flag);
        }
        Workspace tmp(s);  // per-round scan scratch, released at the end of the round
        FHG_TRY(scan_exclusive_u32(tmp, flag, pos, n, cnt));
        LAUNCH(emit_write_kernel, ncomp, reps, ncomp, tgt, cmin, flag, pos, winner, cand_q, cand_w,
               ix.orig, m, out->src, out->dst, out->w2);
        LAUNCH(emit_clear_kernel, ncomp, reps, ncomp, cmin, flag);
        LAUNCH(union_reps_kernel, ncomp, reps, ncomp, tgt, par);
        LAUNCH(relabel_points_kernel, n, n, par, comp);
        uint32_t* keep = pos;  // pos is free again after emit_write
        LAUNCH(merge_cmin_kernel, ncomp, reps, ncomp, par, cmin, keep);
        FHG_TRY(scan_exclusive_u32(tmp, keep, kpos, ncomp, cnt + 1));
        LAUNCH(compact_kernel, ncomp, ncomp, keep, kpos, reps, reps2);
        uint32_t h2[2] = {0, 0};
        int h_missing = 0;
        FHG_CUDA(cudaMemcpyAsync(h2, cnt, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        FHG_CUDA(cudaMemcpyAsync(&h_missing, iflag + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
        FHG_CUDA(cudaStreamSynchronize(s));
        int32_t* tr = reps; reps = reps2; reps2 = tr;
        int64_t new_ncomp = h2[1];
        int64_t added = h2[0];
        if (h_missing || added != ncomp - new_ncomp) {
            set_error("boruvka round %d: inconsistent merge (added %lld, components %lld -> %lld, "
                      "missing=%d)", rounds, (long long)added, (long long)ncomp,
                      (long long)new_ncomp, h_missing);
            return FHG_ERR_NO_CONVERGENCE;
        }
        m += added;
        ncomp = new_ncomp;
        ++rounds;
    }
    out->m = m;
    out->rounds = rounds;
    return FHG_OK;
}

}  // namespace fhg
