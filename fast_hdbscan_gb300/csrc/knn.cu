// Exact k-nearest-neighbour search (core distances), warp-cooperative.
//
// One warp owns one bucket of 32 Morton-consecutive query points (lane =
// query).  It first scans its own bucket -- which contains the queries
// themselves -- to get a tight k-th distance, then walks up the bucket tree to
// the root: at every ancestor it searches the sibling subtree depth-first
// (shared-memory stack; a node is entered when ANY lane's lower bound is
// within that lane's current k-th distance).  At a
// leaf the warp stages the bucket's points in shared memory with one
// coalesced load per lane, and every lane reads candidate t with a broadcast
// shared-memory load and marks it if it is within the lane's k-th distance;
// then each lane inserts its own marked candidates.  Each lane keeps its
// sorted top-K list (squared distance, caller index) in registers: exact
// distance ties are broken without a memory access, and the Morton positions
// of the result are looked up once at the end.
//
// Ordering: (squared distance, caller index), ascending -- the reference's
// parallel_tree_query order with equal distances ordered by index.
// Replaces numba_kdtree.py:680-792 (tree_query_recursion, simple_heap_push,
// deheap_sort, parallel_tree_query).
#include "index.cuh"

namespace fhg {
namespace {

constexpr int kKnnWarps = 4;
// Buckets needed by at most this many lanes are scanned query by query.
constexpr int kTransposeMax = 20;
// Resident blocks asked of the register allocator: small lists fit in 80
// registers, which keeps 24 warps per SM; larger lists take what they need.
template <int DIM, int K>
constexpr int knn_min_blocks() { return (K <= 16 && DIM <= 8) ? 6 : 1; }
constexpr int kStack = 64;

__device__ __forceinline__ unsigned long long pack_entry(float d, int32_t o) {
    return ((unsigned long long)__float_as_uint(d) << 32) | (uint32_t)o;
}
__device__ __forceinline__ float entry_dist(unsigned long long e) {
    return __uint_as_float((uint32_t)(e >> 32));
}
__device__ __forceinline__ int32_t entry_orig(unsigned long long e) { return (int32_t)(uint32_t)e; }

template <int DIM, int SP, int K>
__global__ void __launch_bounds__(kKnnWarps * 32, knn_min_blocks<DIM, K>()) knn_kernel(IndexView ix, int k,
                                                              float* __restrict__ d_s,
                                                              int32_t* __restrict__ i_s,
                                                              float* __restrict__ d_o,
                                                              int32_t* __restrict__ i_o,
                                                              int8_t* __restrict__ tie_s,
                                                              int io_stride, int io_skip,
                                                              const float* __restrict__ cap2,
                                                              const uint8_t* __restrict__ redo,
                                                              uint8_t* __restrict__ fail,
                                                              unsigned long long* fail_count,
                                                              unsigned long long* scan_count) {
    __shared__ int32_t s_stack[kKnnWarps][kStack];
    __shared__ float4 s_cand[kKnnWarps][32 * (SP / 4)];
    __shared__ int32_t s_corig[kKnnWarps][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t leaf = (int64_t)blockIdx.x * kKnnWarps + warp;
    if (leaf >= ix.nleaves) return;
    const int64_t qi = leaf * kLeaf + lane;
    // redo (nullable): only these queries search (the fallback of a capped
    // pass); cap2 (nullable): every query's list starts full of sentinels at
    // its squared search radius, so only points within it are considered.
    const bool valid = qi < ix.n && (!redo || redo[qi]);
    if (redo && !__any_sync(kFull, valid)) return;
    float q[DIM];
    {
        float t[SP];
        if (valid) load_pt<SP>(ix.pts, qi, t);
        else
#pragma unroll
            for (int j = 0; j < SP; ++j) t[j] = 0.0f;
#pragma unroll
        for (int j = 0; j < DIM; ++j) q[j] = t[j];
    }
    // Each list entry is one 64-bit key: squared distance bits above the
    // caller index.  Non-negative floats order like their bit patterns, so
    // one unsigned compare orders entries by (distance, caller index).
    // Slots [0, K-k) hold a 0 sentinel so that the live list has length k;
    // empty live slots hold (+inf, INT32_MAX).
    unsigned long long key[K];
    const unsigned long long kEmptyKey =
        pack_entry(cap2 && valid ? cap2[qi] : INFINITY, INT32_MAX);
#pragma unroll
    for (int j = 0; j < K; ++j) key[j] = (j < K - k) ? 0ull : kEmptyKey;
    float4* cand = s_cand[warp];
    int32_t* corig = s_corig[warp];
    const int32_t* __restrict__ orig = ix.orig;

    // Smallest distance of a point examined but left out of the list: equal to
    // the final k-th distance exactly when another point ties with the k-th.
    float rejmin = INFINITY;
    // Inserts (dd, o) into this lane's sorted list if it precedes the k-th.
    // Every slot's new value depends only on the old list (no chain of
    // compare-and-swap steps): slot j takes slot j-1's entry if that entry
    // follows (dd, o), else (dd, o) if slot j's own entry follows it.
    auto insert = [&](float dd, int32_t o) {
        const unsigned long long nk = pack_entry(dd, o);
        if (!(nk < key[K - 1])) {
            rejmin = fminf(rejmin, dd);
            return;
        }
        // (a sentinel of a capped list leaving is no point)
        if (entry_orig(key[K - 1]) != INT32_MAX) rejmin = fminf(rejmin, entry_dist(key[K - 1]));
        bool gt_hi = true;
#pragma unroll
        for (int j = K - 1; j > 0; --j) {
            const bool gt_lo = key[j - 1] > nk;
            key[j] = gt_lo ? key[j - 1] : (gt_hi ? nk : key[j]);
            gt_hi = gt_lo;
        }
        if (gt_hi) key[0] = nk;
    };

    // One bucket: first every lane marks the candidates within its current
    // k-th distance (one bit each), then each lane inserts only its own
    // marked candidates -- the warp pays for the busiest lane, not for every
    // candidate some lane wants.
    int scans = 0;  // buckets this warp scanned
    auto scan_leaf = [&](int64_t lf, bool need) {
        ++scans;
        const int64_t base = lf * kLeaf;
        const int cnt = (int)(ix.n - base < kLeaf ? ix.n - base : kLeaf);
        float own[SP];  // this lane's candidate (lane t holds candidate t)
#pragma unroll
        for (int j = 0; j < SP; ++j) own[j] = 0.0f;
        if (lane < cnt) {
            const float4* src = reinterpret_cast<const float4*>(ix.pts) + (base + lane) * (SP / 4);
#pragma unroll
            for (int h = 0; h < SP / 4; ++h) {
                const float4 v = __ldg(src + h);
                cand[lane * (SP / 4) + h] = v;
                own[4 * h] = v.x; own[4 * h + 1] = v.y; own[4 * h + 2] = v.z; own[4 * h + 3] = v.w;
            }
            corig[lane] = __ldg(orig + base + lane);
        }
        __syncwarp();
        const float thr = need ? entry_dist(key[K - 1]) : -INFINITY;
        uint32_t acc = 0u;
        const unsigned needy = __ballot_sync(kFull, need);
        if (__popc(needy) <= kTransposeMax) {
            // Few lanes need the bucket: each lane takes its own candidate and
            // the warp visits only the needing queries; the ballot over the
            // candidates is that query's mask.  Same distances bit for bit.
            unsigned mq = needy;
            while (mq) {
                const int i = __ffs(mq) - 1;
                mq &= mq - 1u;
                float qi[DIM];
#pragma unroll
                for (int j = 0; j < DIM; ++j) qi[j] = __shfl_sync(kFull, q[j], i);
                const float ti = __shfl_sync(kFull, thr, i);
                const unsigned bits = __ballot_sync(kFull, lane < cnt && rdist_rn<DIM>(qi, own) <= ti);
                if (lane == i) acc = bits;
            }
        } else {
#pragma unroll 4
            for (int t = 0; t < cnt; ++t) {
                float c[SP];
#pragma unroll
                for (int h = 0; h < SP / 4; ++h) {
                    float4 v = cand[t * (SP / 4) + h];
                    c[4 * h] = v.x; c[4 * h + 1] = v.y; c[4 * h + 2] = v.z; c[4 * h + 3] = v.w;
                }
                acc |= (rdist_rn<DIM>(q, c) <= thr ? 1u : 0u) << t;
            }
        }
        while (acc) {
            const int t = __ffs(acc) - 1;
            acc &= acc - 1u;
            float c[SP];
#pragma unroll
            for (int h = 0; h < SP / 4; ++h) {
                float4 v = cand[t * (SP / 4) + h];
                c[4 * h] = v.x; c[4 * h + 1] = v.y; c[4 * h + 2] = v.z; c[4 * h + 3] = v.w;
            }
            insert(rdist_rn<DIM>(q, c), corig[t]);
        }
        __syncwarp();
    };

    // Seed with the warp's own bucket (it holds the queries themselves), so
    // that the walk below starts with a tight k-th distance; the walk then
    // skips this bucket.
    scan_leaf(leaf, valid);

    // Walk up from the home bucket to the root: at each ancestor search the
    // sibling subtree depth first, pruned by lower bounds.  Subtrees' boxes
    // overlap, so no ancestor box bounds the search; but near subtrees come
    // first, and a far sibling whose box is out of every lane's reach costs a
    // single box test.  Inside a sibling subtree the child nearer the home
    // bucket in Morton order goes first: the left child of a subtree to the
    // right of the home path, the right child of one to its left.
    int32_t* st = s_stack[warp];
    const int64_t first_leaf_node = ix.slots - 1;
    int64_t x = first_leaf_node + leaf;
    while (x > 0) {
        const int32_t sib = (int32_t)((x & 1) ? x + 1 : x - 1);
        const bool right_side = (x & 1) != 0;
        int sp = 1;
        if (lane == 0) st[0] = sib;
        __syncwarp();
        while (sp > 0) {
            --sp;
            const int32_t node = st[sp];
            __syncwarp();
            float b[2 * SP];
            load_box<SP>(ix.box, node, b);
            const float lb = box_lb_n<DIM, SP>(b, q);
            const bool need = valid && lb <= entry_dist(key[K - 1]);
            if (!__any_sync(kFull, need)) continue;
            if (node >= first_leaf_node) {
                scan_leaf(node - first_leaf_node, need);
            } else {
                const int32_t l = 2 * node + 1, r = l + 1;
                const int32_t near = right_side ? l : r, far = right_side ? r : l;
                if (lane == 0) {
                    st[sp] = far;
                    st[sp + 1] = near;
                }
                sp += 2;
                __syncwarp();
            }
        }
        x = (x - 1) >> 1;
    }
    if (scan_count && lane == 0) atomicAdd(scan_count, (unsigned long long)scans);
    if (!valid) return;
    // Certification: a capped list whose k-th slot still holds a sentinel had
    // fewer than k points within the radius -- its query is searched again
    // without a cap.  A full list is the exact answer: every point closer than
    // its k-th entry lies within the radius and was considered.
    if (cap2 && entry_orig(key[K - 1]) == INT32_MAX) {
        fail[qi] = 1;
        if (fail_count) atomicAdd(fail_count, 1ull);
        return;
    }
    if (tie_s) tie_s[qi] = rejmin == entry_dist(key[K - 1]) ? 1 : 0;
    const int64_t o_row = orig[qi];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        if (j < K - k) continue;
        const int jj = j - (K - k);
        const float dj = entry_dist(key[j]);
        const int32_t oj = entry_orig(key[j]);
        const int32_t o = oj == INT32_MAX ? -1 : oj;  // k > n leaves slots empty
        if (d_s) {
            d_s[qi * k + jj] = dj;
            i_s[qi * k + jj] = o >= 0 ? __ldg(ix.rank + o) : -1;
        }
        if (d_o) d_o[o_row * k + jj] = dj;
        if (i_o && jj >= io_skip) i_o[o_row * io_stride + jj - io_skip] = o;
    }
}

// ---------------------------------------------------------------------------
// Lists longer than 64: one warp per query, its sorted list in shared memory.
//
// The list (k keys in (squared distance, caller index) order, unfilled slots
// (+inf, INT32_MAX)) and a merge buffer take 2 * kpad 64-bit words of
// dynamic shared memory (kpad = k rounded up to 32, at most kKnnMaxK), the
// sorted candidates of one bucket 32 more.  The walk is knn_kernel's for a
// single query: the home bucket, then every ancestor's sibling subtree,
// entered while its box bound is within the k-th distance.  A bucket's 32
// candidates are the warp's lanes; those below the k-th key are sorted across
// the warp (bitonic) and merged into the list by rank (each entry's place =
// its own index + the entries of the other sequence below it; no key occurs
// twice, so the places are distinct).  The list is the k smallest keys of all
// points and the tie flag has knn_kernel's meaning, so both kernels give the
// same outputs bit for bit.

// Ascending bitonic sort of 32 keys, one per lane.
__device__ __forceinline__ unsigned long long warp_sort_u64(unsigned long long v, int lane) {
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const unsigned long long o = __shfl_xor_sync(kFull, v, stride);
            const bool ascending = (lane & size) == 0;
            const bool lower = (lane & stride) == 0;
            v = (lower == ascending) ? (o < v ? o : v) : (o > v ? o : v);
        }
    }
    return v;
}

// Number of entries of the ascending a[0, len) below key.
__device__ __forceinline__ int count_below(const unsigned long long* a, int len,
                                           unsigned long long key) {
    int lo = 0, hi = len;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

template <int DIM, int SP>
__global__ void __launch_bounds__(32) knn_large_kernel(IndexView ix, int k, float* __restrict__ d_s,
                                                       int32_t* __restrict__ i_s,
                                                       float* __restrict__ d_o,
                                                       int32_t* __restrict__ i_o,
                                                       int8_t* __restrict__ tie_s, int io_stride,
                                                       int io_skip,
                                                       unsigned long long* scan_count) {
    extern __shared__ unsigned long long s_lists[];  // [kpad] list, [kpad] buffer, [32] bucket
    __shared__ int32_t st[kStack];
    const int lane = threadIdx.x;
    const int64_t qi = blockIdx.x;
    if (qi >= ix.n) return;
    const int kpad = (k + 31) & ~31;
    unsigned long long* A = s_lists;
    unsigned long long* B = s_lists + kpad;
    unsigned long long* S = s_lists + 2 * kpad;
    const unsigned long long kEmptyKey = pack_entry(INFINITY, INT32_MAX);
    for (int j = lane; j < kpad; j += 32) A[j] = kEmptyKey;
    float q[DIM];
    {
        float t[SP];
        load_pt<SP>(ix.pts, qi, t);
#pragma unroll
        for (int j = 0; j < DIM; ++j) q[j] = t[j];
    }
    __syncwarp();
    float rejmin = INFINITY;  // least distance of an examined point left out
    int scans = 0;
    auto scan_leaf = [&](int64_t lf) {
        ++scans;
        const int64_t base = lf * kLeaf;
        const int cnt = (int)(ix.n - base < kLeaf ? ix.n - base : kLeaf);
        unsigned long long key = ~0ull;
        float dd = INFINITY;
        if (lane < cnt) {
            float c[SP];
            load_pt<SP>(ix.pts, base + lane, c);
            dd = rdist_rn<DIM>(q, c);
            key = pack_entry(dd, __ldg(ix.orig + base + lane));
        }
        const bool keep = lane < cnt && key < A[k - 1];
        if (lane < cnt && !keep) rejmin = fminf(rejmin, dd);
        const unsigned kmask = __ballot_sync(kFull, keep);
        if (kmask == 0u) return;
        const int ns = __popc(kmask);
        const unsigned long long sv = warp_sort_u64(keep ? key : ~0ull, lane);
        S[lane] = sv;
        __syncwarp();
        for (int j = lane; j < k; j += 32) {
            const unsigned long long e = A[j];
            const int at = j + count_below(S, ns, e);
            if (at < k) B[at] = e;
            else if (entry_orig(e) != INT32_MAX) rejmin = fminf(rejmin, entry_dist(e));
        }
        if (lane < ns) {
            const int at = lane + count_below(A, k, sv);
            if (at < k) B[at] = sv;
            else rejmin = fminf(rejmin, entry_dist(sv));
        }
        __syncwarp();
        unsigned long long* t = A;
        A = B;
        B = t;
    };

    const int64_t leaf = qi / kLeaf;
    scan_leaf(leaf);
    const int64_t first_leaf_node = ix.slots - 1;
    int64_t x = first_leaf_node + leaf;
    while (x > 0) {
        const int32_t sib = (int32_t)((x & 1) ? x + 1 : x - 1);
        const bool right_side = (x & 1) != 0;
        int sp = 1;
        if (lane == 0) st[0] = sib;
        __syncwarp();
        while (sp > 0) {
            --sp;
            const int32_t node = st[sp];
            __syncwarp();
            float b[2 * SP];
            load_box<SP>(ix.box, node, b);
            const float lb = box_lb_n<DIM, SP>(b, q);
            if (!(lb <= entry_dist(A[k - 1]))) continue;
            if (node >= first_leaf_node) {
                scan_leaf(node - first_leaf_node);
            } else {
                const int32_t l = 2 * node + 1, r = l + 1;
                const int32_t near = right_side ? l : r, far = right_side ? r : l;
                if (lane == 0) {
                    st[sp] = far;
                    st[sp + 1] = near;
                }
                sp += 2;
                __syncwarp();
            }
        }
        x = (x - 1) >> 1;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rejmin = fminf(rejmin, __shfl_xor_sync(kFull, rejmin, o));
    if (scan_count && lane == 0) atomicAdd(scan_count, (unsigned long long)scans);
    if (tie_s && lane == 0) tie_s[qi] = rejmin == entry_dist(A[k - 1]) ? 1 : 0;
    const int64_t o_row = ix.orig[qi];
    for (int j = lane; j < k; j += 32) {
        const unsigned long long e = A[j];
        const float dj = entry_dist(e);
        const int32_t oj = entry_orig(e);
        const int32_t o = oj == INT32_MAX ? -1 : oj;  // k > n leaves slots empty
        if (d_s) {
            d_s[qi * k + j] = dj;
            i_s[qi * k + j] = o >= 0 ? __ldg(ix.rank + o) : -1;
        }
        if (d_o) d_o[o_row * k + j] = dj;
        if (i_o && j >= io_skip) i_o[o_row * io_stride + j - io_skip] = o;
    }
}

template <int DIM>
int launch_knn_large(const fhg_index& ix, int k, float* d_s, int32_t* i_s, float* d_o,
                     int32_t* i_o, int8_t* tie_s, int io_stride, int io_skip, const KnnCap& cap,
                     cudaStream_t s) {
    constexpr int SP = DIM <= 4 ? 4 : (DIM <= 8 ? 8 : DIM);
    if (cap.cap2 || cap.redo) {
        set_error("knn: a search radius takes k <= 64 (got %d)", k);
        return FHG_ERR_UNSUPPORTED;
    }
    if (ix.n <= 0) return FHG_OK;
    const int kpad = (k + 31) & ~31;
    const size_t smem = sizeof(unsigned long long) * (size_t)(2 * kpad + 32);
    Stage stage(s, "knn_kernel");
    ::fhg::note_launch();
    knn_large_kernel<DIM, SP><<<(unsigned)ix.n, 32, smem, s>>>(view_of(ix), k, d_s, i_s, d_o, i_o,
                                                               tie_s, io_stride, io_skip,
                                                               cap.scan_count);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

template <int DIM, int K>
int launch_knn(const fhg_index& ix, int k, float* d_s, int32_t* i_s, float* d_o, int32_t* i_o,
               int8_t* tie_s, int io_stride, int io_skip, const KnnCap& cap, cudaStream_t s) {
    // padded width; for d > 8 the kernels run over all SP = DIM padded
    // coordinates (the padding is zero and adds exact zeros to distances)
    constexpr int SP = DIM <= 4 ? 4 : (DIM <= 8 ? 8 : DIM);
    unsigned g = grid_for(ix.nleaves, kKnnWarps);
    Stage stage(s, "knn_kernel");
    ::fhg::note_launch();
    knn_kernel<DIM, SP, K><<<g, kKnnWarps * 32, 0, s>>>(view_of(ix), k, d_s, i_s, d_o, i_o,
                                                         tie_s, io_stride, io_skip, cap.cap2,
                                                         cap.redo, cap.fail, cap.fail_count,
                                                         cap.scan_count);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

template <int DIM>
int dispatch_k(const fhg_index& ix, int k, float* d_s, int32_t* i_s, float* d_o, int32_t* i_o,
               int8_t* tie_s, int ios, int iok, const KnnCap& c, cudaStream_t s) {
    if (k <= 8) return launch_knn<DIM, 8>(ix, k, d_s, i_s, d_o, i_o, tie_s, ios, iok, c, s);
    if (k <= 16) return launch_knn<DIM, 16>(ix, k, d_s, i_s, d_o, i_o, tie_s, ios, iok, c, s);
    if (k <= 24) return launch_knn<DIM, 24>(ix, k, d_s, i_s, d_o, i_o, tie_s, ios, iok, c, s);
    if (k <= 32) return launch_knn<DIM, 32>(ix, k, d_s, i_s, d_o, i_o, tie_s, ios, iok, c, s);
    return launch_knn<DIM, 64>(ix, k, d_s, i_s, d_o, i_o, tie_s, ios, iok, c, s);
}

}  // namespace

int index_knn(const fhg_index& ix, int k, float* d_s, int32_t* i_s, float* d_o, int32_t* i_o,
              cudaStream_t s, int8_t* tie_s, int io_stride, int io_skip, const KnnCap& cap) {
    if (io_stride <= 0) io_stride = k;
    if (k < 1 || k > kKnnMaxK) {
        set_error("knn: k must be in [1, %d] (got %d)", kKnnMaxK, k);
        return k < 1 ? FHG_ERR_INVALID : FHG_ERR_UNSUPPORTED;
    }
    if ((d_s == nullptr) != (i_s == nullptr) || (d_o != nullptr && i_o == nullptr) ||
        (d_o != nullptr && (io_stride != k || io_skip != 0))) {
        set_error("knn: Morton-order outputs come in pairs; caller-order distances need ids");
        return FHG_ERR_INVALID;
    }
    Stage stage(s, "knn");
    if (k > 64) {  // the list no longer fits in registers
#define FHG_LARGE(D) launch_knn_large<D>(ix, k, d_s, i_s, d_o, i_o, tie_s, io_stride, io_skip, cap, s)
        switch (ix.d) {
            case 1: return FHG_LARGE(1);
            case 2: return FHG_LARGE(2);
            case 3: return FHG_LARGE(3);
            case 4: return FHG_LARGE(4);
            case 5: return FHG_LARGE(5);
            case 6: return FHG_LARGE(6);
            case 7: return FHG_LARGE(7);
            case 8: return FHG_LARGE(8);
            default: return ix.d <= 16 ? FHG_LARGE(16) : FHG_LARGE(32);
        }
#undef FHG_LARGE
    }
    switch (ix.d) {
        case 1: return dispatch_k<1>(ix, k, d_s, i_s, d_o, i_o, tie_s, io_stride, io_skip, cap, s);
        case 2: return dispatch_k<2>(ix, k, d_s, i_s, d_o, i_o, tie_s, io_stride, io_skip, cap, s);
        case 3: return dispatch_k<3>(ix, k, d_s, i_s, d_o, i_o, tie_s, io_stride, io_skip, cap, s);
        case 4: return dispatch_k<4>(ix, k, d_s, i_s, d_o, i_o, tie_s, io_stride, io_skip, cap, s);
        case 5: return dispatch_k<5>(ix, k, d_s, i_s, d_o, i_o, tie_s, io_stride, io_skip, cap, s);
        case 6: return dispatch_k<6>(ix, k, d_s, i_s, d_o, i_o, tie_s, io_stride, io_skip, cap, s);
        case 7: return dispatch_k<7>(ix, k, d_s, i_s, d_o, i_o, tie_s, io_stride, io_skip, cap, s);
        case 8: return dispatch_k<8>(ix, k, d_s, i_s, d_o, i_o, tie_s, io_stride, io_skip, cap, s);
        default:
            if (ix.d <= 16)
                return dispatch_k<16>(ix, k, d_s, i_s, d_o, i_o, tie_s, io_stride, io_skip, cap, s);
            return dispatch_k<32>(ix, k, d_s, i_s, d_o, i_o, tie_s, io_stride, io_skip, cap, s);
    }
}

}  // namespace fhg
