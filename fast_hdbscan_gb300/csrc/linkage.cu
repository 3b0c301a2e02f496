// MST sort (hdbscan.py:511) and single-linkage tree (cluster_trees.py:65).
//
// The reference builds the linkage tree with a sequential union-find over
// the sorted edges: edge i merges the current roots of its two endpoints
// into node n + i.  Here the same tree is built by rank-halving divide and
// conquer, level-synchronously:
//   For an interval of sorted ranks [a, a+s), every endpoint carries the id
//   of its component's root node at time a.  The lower half [a, a+s/2) is
//   contracted by a lock-free union-find over those ids; each contracted
//   component's new root is node n + (largest rank in it), and every endpoint
//   of the upper half [a+s/2, a+s) that was touched is relabelled to that
//   node.  Then both halves recurse with s/2.  After the last level every
//   edge holds the roots at its own time: exactly the reference's
//   (left, right) children.
// An id can be an endpoint label in at most one interval per level (a root
// touched by an interval is no longer a root in any later interval), so one
// global parent array serves every interval of a level at once.  Work is
// O(n log n), depth O(log^2 n), whatever the height of the dendrogram.
#include "primitives.cuh"
#include "trees.cuh"

namespace fhg {
namespace {

__device__ __forceinline__ uint64_t f64_key(double x) {
    if (x == 0.0) x = 0.0;  // -0.0 sorts with +0.0, as np.lexsort compares values
    uint64_t b = (uint64_t)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void iota_kernel(int32_t* a, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = (int32_t)i;
}
__global__ void gather_key32_kernel(const int32_t* __restrict__ v, const int32_t* __restrict__ perm,
                                    uint32_t* __restrict__ keys, int64_t m) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) keys[i] = (uint32_t)v[perm[i]];
}
__global__ void gather_wkey_kernel(const double* __restrict__ w, const float* __restrict__ w2,
                                   const int32_t* __restrict__ perm, uint64_t* __restrict__ k64,
                                   uint32_t* __restrict__ k32, int64_t m) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    if (w) k64[i] = f64_key(w[perm[i]]);
    else k32[i] = __float_as_uint(w2[perm[i]]);  // non-negative: bits are monotone
}
__global__ void apply_perm_kernel(const int32_t* __restrict__ perm, const int32_t* __restrict__ src,
                                  const int32_t* __restrict__ dst, const double* __restrict__ w,
                                  const float* __restrict__ w2, int32_t* __restrict__ ssrc,
                                  int32_t* __restrict__ sdst, double* __restrict__ sw,
                                  int32_t* __restrict__ A, int32_t* __restrict__ B, int64_t m) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int32_t e = perm[i];
    ssrc[i] = A[i] = src[e];
    sdst[i] = B[i] = dst[e];
    sw[i] = w ? w[e] : __dsqrt_rn((double)w2[e]);
}
// Per-node state of the contraction, one 32-byte record per node id so that
// every access to a (randomly placed) node touches a single sector:
//   P      union-find parent (valid when stamp == the current level)
//   stamp  level at which the node was last an endpoint of a lower half
//   M      largest rank of its contracted component (at the root)
//   SUM    size of its contracted component (at the root)
//   claim  level at which its size was last added to a SUM
//   SZ     number of points under the node
struct __align__(32) NodeRec {
    int32_t P, stamp, M, SUM, claim, SZ, pad0, pad1;
};

// Union-find in which a parent is never younger than its child.  Age order:
// cluster nodes (ids n + rank) by rank, then points by label (points are
// renumbered by the rank of their first edge, so a smaller label is an older
// point).  A union links the younger root under the older one, so the points
// a cluster absorbs within an interval link under the cluster's node -- each
// its own record, no contended update -- and paths stay short.  The
// renumbering only keeps the records an interval touches cache-resident: any
// total age order gives a correct union-find, and the allocation-free entry
// point runs on the raw point labels.
__device__ __forceinline__ uint32_t age_key(int32_t x, int32_t n) {
    return x >= n ? (uint32_t)(x - n) : (uint32_t)x + 0x80000000u;
}
__device__ __forceinline__ int32_t rec_find(NodeRec* R, int32_t x, int32_t n) {
    int32_t cur = R[x].P;
    if (cur != x) {
        int32_t prev = x, next;
        while (age_key(cur, n) > age_key(next = R[cur].P, n)) {
            R[prev].P = next;
            prev = cur;
            cur = next;
        }
    }
    return cur;
}

// Root of x without path compression, for the passes after the unions: a
// large cluster's label is looked up by long runs of ranks, and compressing
// writes from all of them would queue on one record.
__device__ __forceinline__ int32_t rec_root(const NodeRec* R, int32_t x) {
    int32_t cur = x, next;
    while ((next = R[cur].P) != cur) cur = next;
    return cur;
}
// rec_root of every lane's label, looked up once per distinct label in the
// warp (the lanes in `act` call it together).
__device__ __forceinline__ int32_t warp_root(const NodeRec* R, int32_t x, unsigned act) {
    const unsigned peers = __match_any_sync(act, x);
    const int lead = __ffs(peers) - 1;
    int32_t r = 0;
    if ((int)(threadIdx.x & 31) == lead) r = rec_root(R, x);
    return __shfl_sync(act, r, lead);
}

__device__ __forceinline__ void rec_union(NodeRec* R, int32_t a, int32_t b, int32_t n) {
    int32_t ra = rec_find(R, a, n), rb = rec_find(R, b, n);
    while (ra != rb) {
        if (age_key(ra, n) < age_key(rb, n)) {
            int32_t t = ra; ra = rb; rb = t;
        }
        int32_t old = atomicCAS(&R[ra].P, ra, rb);
        if (old == ra) return;
        ra = rec_find(R, old, n);
        rb = rec_find(R, rb, n);
    }
}

__global__ void node_init_kernel(int64_t nodes, int64_t n, NodeRec* R) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nodes) return;
    NodeRec r;
    r.P = (int32_t)i;
    r.stamp = -1;
    r.M = -1;
    r.SUM = 0;
    r.claim = -1;
    r.SZ = i < n ? 1 : 0;
    r.pad0 = r.pad1 = 0;
    R[i] = r;
}

__global__ void node_sizes_kernel(int64_t nodes, const NodeRec* __restrict__ R,
                                  int32_t* __restrict__ size) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nodes) size[i] = R[i].SZ;
}

// Thread t of a level works on the t-th rank of the lower (or upper) halves
// of the rank intervals [a, a + s), a = 0, s, 2s, ...
__device__ __forceinline__ int64_t low_rank(int64_t t, int64_t s, int64_t half) {
    return (t / half) * s + (t % half);
}

__global__ void lvl_init_kernel(int64_t m, int64_t s, int64_t half, const int32_t* __restrict__ A,
                                const int32_t* __restrict__ B, NodeRec* R, int lev) {
    const int64_t i = low_rank((int64_t)blockIdx.x * blockDim.x + threadIdx.x, s, half);
    if (i >= m) return;
    const int32_t a = A[i], b = B[i];
    *reinterpret_cast<int4*>(&R[a]) = make_int4(a, lev, -1, 0);
    *reinterpret_cast<int4*>(&R[b]) = make_int4(b, lev, -1, 0);
}
__global__ void lvl_union_kernel(int64_t m, int64_t s, int64_t half, int64_t n,
                                 const int32_t* __restrict__ A, const int32_t* __restrict__ B,
                                 NodeRec* R) {
    const int64_t i = low_rank((int64_t)blockIdx.x * blockDim.x + threadIdx.x, s, half);
    if (i >= m) return;
    rec_union(R, A[i], B[i], (int32_t)n);
}
constexpr int kReduceThreads = 256;
__global__ void __launch_bounds__(kReduceThreads) lvl_reduce_kernel(
    int64_t m, int64_t s, int64_t half, int64_t n, const int32_t* __restrict__ A,
    const int32_t* __restrict__ B, NodeRec* R, int lev) {
    __shared__ int32_t s_root[kReduceThreads / 32], s_mx[kReduceThreads / 32];
    __shared__ int32_t s_sum[kReduceThreads / 32];
    __shared__ int s_uniform;
    const int64_t i = low_rank((int64_t)blockIdx.x * blockDim.x + threadIdx.x, s, half);
    const bool valid = i < m;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned act = __ballot_sync(kFull, valid);
    int32_t r = -1, add = 0;
    if (valid) {
        // A label claims its size for its component once.  A large cluster's
        // label is an endpoint of long runs of ranks: one lane per label per
        // warp, and only while unclaimed, goes to the atomic.
        const int32_t a = A[i], b = B[i];
        const unsigned pa = __match_any_sync(act, a), pb = __match_any_sync(act, b);
        r = warp_root(R, a, act);
        if (lane == __ffs(pa) - 1 && R[a].claim != lev && atomicExch(&R[a].claim, lev) != lev)
            add += R[a].SZ;
        if (lane == __ffs(pb) - 1 && R[b].claim != lev && atomicExch(&R[b].claim, lev) != lev)
            add += R[b].SZ;
    }
    // Consecutive ranks mostly share a root (a large component absorbs long
    // runs of edges): combine the lanes of each root first, then the warps of
    // the block when they all share one root, so that a large component takes
    // one atomic per block rather than one per rank.
    unsigned peers = 0;
    int32_t mx = -1, sum = 0;
    if (valid) {
        peers = __match_any_sync(act, r);
        mx = __reduce_max_sync(peers, (int32_t)i);
        sum = (int32_t)__reduce_add_sync(peers, (unsigned)add);
    }
    const bool wuni = __all_sync(kFull, !valid || peers == act);
    {
        const int lead = act ? __ffs(act) - 1 : 0;
        const int32_t rl = __shfl_sync(kFull, r, lead);
        const int32_t ml = __shfl_sync(kFull, mx, lead);
        const int32_t sl = __shfl_sync(kFull, sum, lead);
        if (lane == 0) {
            // -1: no edge in the warp; -3: several roots; else the warp's root
            s_root[warp] = act == 0 ? -1 : (wuni ? rl : -3);
            s_mx[warp] = ml;
            s_sum[warp] = sl;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int32_t root = -1, bm = -1, bs = 0;
        int uni = 1;
        for (int w = 0; w < kReduceThreads / 32; ++w) {
            const int32_t x = s_root[w];
            if (x == -1) continue;
            if (x == -3 || (root >= 0 && x != root)) {
                uni = 0;
                break;
            }
            root = x;
            bm = max(bm, s_mx[w]);
            bs += s_sum[w];
        }
        if (uni && root >= 0) {
            atomicMax(&R[root].M, bm);
            if (bs) atomicAdd(&R[root].SUM, bs);
        }
        s_uniform = uni;
    }
    __syncthreads();
    if (s_uniform || !valid) return;
    if (lane == __ffs(peers) - 1) {
        atomicMax(&R[r].M, mx);
        if (sum) atomicAdd(&R[r].SUM, sum);
    }
}
__global__ void lvl_size_kernel(int64_t m, int64_t s, int64_t half, int64_t n,
                                const int32_t* __restrict__ A, NodeRec* R) {
    const int64_t i = low_rank((int64_t)blockIdx.x * blockDim.x + threadIdx.x, s, half);
    const unsigned act = __ballot_sync(kFull, i < m);
    if (i >= m) return;
    const int32_t r = warp_root(R, A[i], act);
    if (R[r].M == (int32_t)i) R[n + i].SZ = R[r].SUM;
}
__global__ void lvl_relabel_kernel(int64_t m, int64_t s, int64_t half, int64_t n, int32_t* A,
                                   int32_t* B, NodeRec* R, int lev) {
    const int64_t i = low_rank((int64_t)blockIdx.x * blockDim.x + threadIdx.x, s, half) + half;
    if (i >= m) return;
    const int32_t a = A[i], b = B[i];
    if (R[a].stamp == lev) A[i] = (int32_t)(n + R[rec_root(R, a)].M);
    if (R[b].stamp == lev) B[i] = (int32_t)(n + R[rec_root(R, b)].M);
}
// Final levels: one block per interval of L <= kLeafRanks consecutive ranks.
// Every endpoint label is already the root node at the interval's start, so
// the block replays the reference's sequential union-find
// (cluster_trees.py:72-93) over at most 2 * L distinct labels held in shared
// memory.
constexpr int kLeafRanks = 512;
constexpr int kLeafThreads = 128;

// Open-addressing table of the interval's labels (SLOTS a power of two, at
// least the 2L labels an interval can hold).
template <int SLOTS>
__device__ __forceinline__ int32_t leaf_slot(int32_t* keys, int32_t label) {
    constexpr int kBits = SLOTS == 1024 ? 10 : 11;
    uint32_t h = ((uint32_t)label * 2654435761u) >> (32 - kBits);
    for (;;) {
        int32_t prev = atomicCAS(&keys[h], -1, label);
        if (prev == -1 || prev == label) return (int32_t)h;
        h = (h + 1) & (SLOTS - 1);
    }
}

// Small tables (L <= 384: 1024 slots, 16 KB) let 14 intervals share an SM,
// each replayed by one thread.
template <int SLOTS>
__global__ void __launch_bounds__(kLeafThreads) leaf_interval_kernel(int64_t m, int64_t n, int L,
                                                                     int32_t* A, int32_t* B,
                                                                     NodeRec* R) {
    static_assert(SLOTS == 1024 || SLOTS == 2048, "table size");
    __shared__ int32_t keys[SLOTS], node[SLOTS], size[SLOTS];
    __shared__ int16_t par[SLOTS];
    __shared__ int16_t sa[kLeafRanks], sb[kLeafRanks];
    const int64_t a = (int64_t)blockIdx.x * L;
    const int cnt = (int)(m - a < L ? m - a : L);
    for (int t = threadIdx.x; t < SLOTS; t += blockDim.x) keys[t] = -1;
    __syncthreads();
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
        int32_t la = A[a + t], lb = B[a + t];
        int32_t ha = leaf_slot<SLOTS>(keys, la), hb = leaf_slot<SLOTS>(keys, lb);
        sa[t] = (int16_t)ha;
        sb[t] = (int16_t)hb;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < SLOTS; t += blockDim.x) {
        int32_t k = keys[t];
        par[t] = (int16_t)t;
        node[t] = k;
        size[t] = k >= 0 ? R[k].SZ : 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int t = 0; t < cnt; ++t) {
            int32_t x = sa[t], y = sb[t];
            while (par[x] != x) { par[x] = par[par[x]]; x = par[x]; }
            while (par[y] != y) { par[y] = par[par[y]]; y = par[y]; }
            const int64_t i = a + t;
            A[i] = node[x];
            B[i] = node[y];
            const int32_t sz = size[x] + size[y];
            R[n + i].SZ = sz;
            par[y] = (int16_t)x;
            node[x] = (int32_t)(n + i);
            size[x] = sz;
        }
    }
}

// inv (nullable) maps renumbered point labels back to the caller's indices.
__global__ void linkage_rows_kernel(int64_t m, int64_t n, const int32_t* __restrict__ A,
                                    const int32_t* __restrict__ B,
                                    const int32_t* __restrict__ inv, int32_t* __restrict__ left,
                                    int32_t* __restrict__ right) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int32_t a = A[i], b = B[i];
    if (inv) {
        if (a < n) a = inv[a];
        if (b < n) b = inv[b];
    }
    left[i] = max(a, b);
    right[i] = min(a, b);
}

// Point renumbering.  A point's new label orders it by the rank of its first
// (lightest) edge, the lower endpoint of that edge first; in every interval
// of the contraction the point labels then lie in a window about as wide as
// the interval, so the node records the level touches stay cache resident.
__global__ void fill_i32_kernel(int32_t* a, int64_t n, int32_t v) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}
__global__ void first_rank_kernel(int64_t m, const int32_t* __restrict__ A,
                                  const int32_t* __restrict__ B, int32_t* first) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    atomicMin(&first[A[i]], (int32_t)i);
    atomicMin(&first[B[i]], (int32_t)i);
}
__device__ __forceinline__ int64_t first_slot(const int32_t* __restrict__ B, int32_t f,
                                              int32_t p) {
    return 2 * (int64_t)f + (B[f] == p ? 1 : 0);
}
__global__ void slot_flags_kernel(int64_t n, const int32_t* __restrict__ first,
                                  const int32_t* __restrict__ B, uint32_t* __restrict__ flag) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int32_t f = first[p];
    if (f != INT32_MAX) flag[first_slot(B, f, (int32_t)p)] = 1u;
}
__global__ void new_labels_kernel(int64_t n, const int32_t* __restrict__ first,
                                  const int32_t* __restrict__ B, const uint32_t* __restrict__ pos,
                                  int32_t* __restrict__ newid, int32_t* __restrict__ inv) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int32_t f = first[p];
    if (f == INT32_MAX) {  // no edge: never a label
        newid[p] = -1;
        return;
    }
    const int32_t id = (int32_t)pos[first_slot(B, f, (int32_t)p)];
    newid[p] = id;
    inv[id] = (int32_t)p;
}
__global__ void relabel_edges_kernel(int64_t m, const int32_t* __restrict__ newid, int32_t* A,
                                     int32_t* B) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    A[i] = newid[A[i]];
    B[i] = newid[B[i]];
}

__global__ void linkage_f64_kernel(int64_t m, const int32_t* __restrict__ left,
                                   const int32_t* __restrict__ right, const double* __restrict__ w,
                                   const int32_t* __restrict__ sz, const float* __restrict__ wsz,
                                   int64_t n, double* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    out[4 * i + 0] = (double)left[i];
    out[4 * i + 1] = (double)right[i];
    out[4 * i + 2] = w[i];
    out[4 * i + 3] = wsz ? (double)wsz[n + i] : (double)sz[n + i];
}
__global__ void sorted_mst_f64_kernel(int64_t m, const int32_t* __restrict__ ssrc,
                                      const int32_t* __restrict__ sdst,
                                      const double* __restrict__ w, double* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    out[3 * i + 0] = (double)ssrc[i];
    out[3 * i + 1] = (double)sdst[i];
    out[3 * i + 2] = w[i];
}

#define LAUNCH(kernel, count, ...)                                          \
    do {                                                                    \
        if ((count) > 0) {                                                  \
            ::fhg::note_launch(); \
            kernel<<<grid_for((count), 256), 256, 0, s>>>(__VA_ARGS__);     \
            FHG_CUDA(cudaGetLastError());                                   \
        }                                                                   \
    } while (0)

// The whole contraction over m > 0 sorted edges with endpoint labels A, B.
// The leaf interval length L = ceil(m / 2^K) <= kLeafRanks makes the top
// interval L * 2^K just cover m, so every level splits its intervals at their
// middle: the lower halves hold about m / 2 ranks at every level.
int contract_ranks(int64_t m, int64_t n, int32_t* A, int32_t* B, NodeRec* R, cudaStream_t s) {
    int K = 0;
    while (((m + (int64_t{1} << K) - 1) >> K) > kLeafRanks) ++K;
    const int64_t L = (m + (int64_t{1} << K) - 1) >> K;
    int lev = 0;
    for (int64_t sz = L << K; sz >= 2 * L; sz /= 2, ++lev) {
        const int64_t half = sz / 2;
        const int64_t intervals = (m + sz - 1) / sz;
        const int64_t lo_threads = intervals * half;
        const int64_t hi_threads = m > half ? ((m - half + sz - 1) / sz) * half : 0;
        LAUNCH(lvl_init_kernel, lo_threads, m, sz, half, A, B, R, lev);
        LAUNCH(lvl_union_kernel, lo_threads, m, sz, half, n, A, B, R);
        LAUNCH(lvl_reduce_kernel, lo_threads, m, sz, half, n, A, B, R, lev);
        LAUNCH(lvl_size_kernel, lo_threads, m, sz, half, n, A, R);
        LAUNCH(lvl_relabel_kernel, hi_threads, m, sz, half, n, A, B, R, lev);
    }
    const int64_t blocks = (m + L - 1) / L;
    ::fhg::note_launch();
    if (L <= 384)
        leaf_interval_kernel<1024><<<(unsigned)blocks, kLeafThreads, 0, s>>>(m, n, (int)L, A, B, R);
    else
        leaf_interval_kernel<2048><<<(unsigned)blocks, kLeafThreads, 0, s>>>(m, n, (int)L, A, B, R);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

}  // namespace

int sort_and_link(Workspace& ws, int64_t n, const int32_t* src, const int32_t* dst,
                  const double* w, const float* w2, Linkage* out, bool presorted) {
    cudaStream_t s = ws.stream();
    const int64_t m = n - 1;
    *out = Linkage();
    out->n = n;
    out->m = m > 0 ? m : 0;
    const int64_t nodes = n + (m > 0 ? m : 0);
    FHG_TRY(ws.alloc(&out->size, (size_t)nodes));
    NodeRec* R;
    FHG_TRY(ws.alloc(&R, (size_t)nodes));
    LAUNCH(node_init_kernel, nodes, nodes, n, R);
    if (m <= 0) {
        LAUNCH(node_sizes_kernel, nodes, nodes, R, out->size);
        return FHG_OK;
    }

    // ---- sort by (weight, src, dst): stable LSD over dst, src, weight
    int32_t* perm;
    uint32_t* k32;
    uint64_t* k64 = nullptr;
    FHG_TRY(ws.alloc(&perm, (size_t)m));
    FHG_TRY(ws.alloc(&k32, (size_t)m));
    if (w) FHG_TRY(ws.alloc(&k64, (size_t)m));
    LAUNCH(iota_kernel, m, perm, m);
    const int ibits = bits_for(n);
    if (!presorted) {
        Stage stage(s, "mst_sort");
        Workspace tmp(s);
        LAUNCH(gather_key32_kernel, m, dst, perm, k32, m);
        FHG_TRY(radix_sort_u32(tmp, k32, perm, m, 0, ibits));
        LAUNCH(gather_key32_kernel, m, src, perm, k32, m);
        FHG_TRY(radix_sort_u32(tmp, k32, perm, m, 0, ibits));
        LAUNCH(gather_wkey_kernel, m, w, w2, perm, k64, k32, m);
        if (w) FHG_TRY(radix_sort_u64(tmp, k64, perm, m, 0, 64));
        else FHG_TRY(radix_sort_u32(tmp, k32, perm, m, 0, 32));
    }
    int32_t *A, *B;
    FHG_TRY(ws.alloc(&out->ssrc, (size_t)m));
    FHG_TRY(ws.alloc(&out->sdst, (size_t)m));
    FHG_TRY(ws.alloc(&out->w, (size_t)m));
    FHG_TRY(ws.alloc(&A, (size_t)m));
    FHG_TRY(ws.alloc(&B, (size_t)m));
    LAUNCH(apply_perm_kernel, m, perm, src, dst, w, w2, out->ssrc, out->sdst, out->w, A, B, m);

    Stage stage(s, "linkage");
    // ---- point renumbering by first edge rank
    int32_t *first, *newid, *inv;
    uint32_t *slot_flag, *slot_pos, *slot_cnt;
    FHG_TRY(ws.alloc(&first, (size_t)n));
    FHG_TRY(ws.alloc(&newid, (size_t)n));
    FHG_TRY(ws.alloc(&inv, (size_t)n));
    {
        Workspace tmp(s);
        FHG_TRY(tmp.alloc(&slot_flag, (size_t)(2 * m)));
        FHG_TRY(tmp.alloc(&slot_pos, (size_t)(2 * m)));
        FHG_TRY(tmp.alloc(&slot_cnt, 1));
        LAUNCH(fill_i32_kernel, n, first, n, INT32_MAX);
        LAUNCH(first_rank_kernel, m, m, A, B, first);
        FHG_CUDA(cudaMemsetAsync(slot_flag, 0, sizeof(uint32_t) * 2 * m, s));
        LAUNCH(slot_flags_kernel, n, n, first, B, slot_flag);
        FHG_TRY(scan_exclusive_u32(tmp, slot_flag, slot_pos, 2 * m, slot_cnt));
        LAUNCH(new_labels_kernel, n, n, first, B, slot_pos, newid, inv);
        LAUNCH(relabel_edges_kernel, m, m, newid, A, B);
    }

    // ---- rank-halving contraction
    FHG_TRY(contract_ranks(m, n, A, B, R, s));
    FHG_TRY(ws.alloc(&out->left, (size_t)m));
    FHG_TRY(ws.alloc(&out->right, (size_t)m));
    LAUNCH(linkage_rows_kernel, m, m, n, A, B, inv, out->left, out->right);
    LAUNCH(node_sizes_kernel, nodes, nodes, R, out->size);
    return FHG_OK;
}

namespace {
__global__ void split_mst_kernel(int64_t m, const double* __restrict__ mst, int32_t* __restrict__ src,
                                 int32_t* __restrict__ dst, double* __restrict__ w) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    // Endpoints must be point ids in [0, m]; anything else (negative, too
    // large, NaN) is clamped into range so that no node record outside the
    // m + 1 points is ever addressed -- the tree is then meaningless, but
    // memory stays safe.
    const double a = mst[3 * i + 0], b = mst[3 * i + 1];
    src[i] = (a >= 0.0 && a <= (double)m) ? (int32_t)a : 0;
    dst[i] = (b >= 0.0 && b <= (double)m) ? (int32_t)b : 0;
    w[i] = mst[3 * i + 2];
}
__global__ void leaf_sizes_kernel(int64_t n, int32_t* __restrict__ size) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) size[i] = 1;
}
__global__ void split_linkage_kernel(int64_t m, int64_t n, const double* __restrict__ lk,
                                     int32_t* __restrict__ left, int32_t* __restrict__ right,
                                     double* __restrict__ w, int32_t* __restrict__ size) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    left[i] = (int32_t)lk[4 * i + 0];
    right[i] = (int32_t)lk[4 * i + 1];
    w[i] = lk[4 * i + 2];
    size[n + i] = (int32_t)lk[4 * i + 3];
}
}  // namespace

int split_mst_f64(Workspace& ws, const double* mst, int64_t m, int32_t** src, int32_t** dst,
                  double** w) {
    cudaStream_t s = ws.stream();
    FHG_TRY(ws.alloc(src, (size_t)(m > 0 ? m : 1)));
    FHG_TRY(ws.alloc(dst, (size_t)(m > 0 ? m : 1)));
    FHG_TRY(ws.alloc(w, (size_t)(m > 0 ? m : 1)));
    LAUNCH(split_mst_kernel, m, m, mst, *src, *dst, *w);
    return FHG_OK;
}

int linkage_from_f64(Workspace& ws, const double* lk, int64_t m, Linkage* out) {
    cudaStream_t s = ws.stream();
    *out = Linkage();
    const int64_t n = m + 1;
    out->n = n;
    out->m = m;
    FHG_TRY(ws.alloc(&out->size, (size_t)(n + m)));
    FHG_TRY(ws.alloc(&out->left, (size_t)(m > 0 ? m : 1)));
    FHG_TRY(ws.alloc(&out->right, (size_t)(m > 0 ? m : 1)));
    FHG_TRY(ws.alloc(&out->w, (size_t)(m > 0 ? m : 1)));
    LAUNCH(leaf_sizes_kernel, n, n, out->size);
    LAUNCH(split_linkage_kernel, m, m, n, lk, out->left, out->right, out->w, out->size);
    return FHG_OK;
}

int linkage_to_f64(const Linkage& lk, double* out, cudaStream_t s) {
    LAUNCH(linkage_f64_kernel, lk.m, lk.m, lk.left, lk.right, lk.w, lk.size, lk.wsize, lk.n, out);
    return FHG_OK;
}
int sorted_mst_to_f64(const Linkage& lk, double* out, cudaStream_t s) {
    LAUNCH(sorted_mst_f64_kernel, lk.m, lk.m, lk.ssrc, lk.sdst, lk.w, out);
    return FHG_OK;
}

}  // namespace fhg

// ---------------------------------------------------------------------------
// Linkage tree without any device allocation.
//
// Some callers cannot allocate device memory while they run: a process whose
// HBM is entirely reserved up front by its own pool allocator, or a
// latency-critical loop that must never enter the CUDA allocator.  For them,
// fhg_mst_to_linkage_tree_noalloc builds the same linkage tree as
// fhg_mst_to_linkage_tree (presorted input) using only the scratch array
// below, a file-scope device array of fixed size that every GPU loading this
// library holds until the process exits.  Inputs and outputs stay the
// caller's buffers.
// ---------------------------------------------------------------------------
#include <mutex>

namespace fhg {
namespace {

constexpr int64_t kNoAllocMaxEdges = FHG_NOALLOC_MAX_EDGES;
constexpr int64_t kNoAllocAlign = 256;

constexpr int64_t noalloc_round(int64_t b) { return (b + kNoAllocAlign - 1) / kNoAllocAlign * kNoAllocAlign; }

// src, dst, A, B, left, right: int32[m]; w: double[m]; node records:
// NodeRec[2m + 1]; node sizes: int32[2m + 1]
constexpr int64_t noalloc_bytes(int64_t m) {
    return 6 * noalloc_round(4 * m) + noalloc_round(8 * m) +
           noalloc_round((int64_t)sizeof(NodeRec) * (2 * m + 1)) + noalloc_round(4 * (2 * m + 1));
}

constexpr int64_t kNoAllocScratchBytes = noalloc_bytes(kNoAllocMaxEdges);

// The scratch array.  Its contents persist from call to call; every buffer
// carved from it is initialised by the kernels of each call before use.
static __device__ __align__(256) unsigned char g_linkage_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_base[kNoAllocMaxDevices] = {};

// Device address of g_linkage_scratch on the current device.  In host code the
// array's name only stands for the device symbol, so the address is asked of
// the runtime once per device (with that device current) and cached.
int noalloc_scratch_base(unsigned char** out) {
    int dev = -1;
    FHG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        set_error("fhg_mst_to_linkage_tree_noalloc: device %d out of range", dev);
        return FHG_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_base[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_linkage_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_error("cudaGetSymbolAddress(g_linkage_scratch) failed on device %d: %s", dev,
                      cudaGetErrorString(e));
            return FHG_ERR_CUDA;
        }
        g_noalloc_base[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_base[dev]);
    return FHG_OK;
}

template <class T>
T* carve(unsigned char*& cur, int64_t count) {
    T* p = reinterpret_cast<T*>(cur);
    cur += noalloc_round((int64_t)sizeof(T) * count);
    return p;
}

int link_presorted_noalloc(const double* smst, int64_t m, double* out, cudaStream_t s) {
    unsigned char* base = nullptr;
    FHG_TRY(noalloc_scratch_base(&base));
    const int64_t n = m + 1, nodes = n + m;
    unsigned char* cur = base;
    int32_t* src = carve<int32_t>(cur, m);
    int32_t* dst = carve<int32_t>(cur, m);
    int32_t* A = carve<int32_t>(cur, m);
    int32_t* B = carve<int32_t>(cur, m);
    int32_t* left = carve<int32_t>(cur, m);
    int32_t* right = carve<int32_t>(cur, m);
    double* w = carve<double>(cur, m);
    NodeRec* R = carve<NodeRec>(cur, nodes);
    int32_t* size = carve<int32_t>(cur, nodes);

    LAUNCH(split_mst_kernel, m, m, smst, src, dst, w);
    LAUNCH(node_init_kernel, nodes, nodes, n, R);
    FHG_CUDA(cudaMemcpyAsync(A, src, sizeof(int32_t) * m, cudaMemcpyDeviceToDevice, s));
    FHG_CUDA(cudaMemcpyAsync(B, dst, sizeof(int32_t) * m, cudaMemcpyDeviceToDevice, s));
    FHG_TRY(contract_ranks(m, n, A, B, R, s));
    LAUNCH(linkage_rows_kernel, m, m, n, A, B, (const int32_t*)nullptr, left, right);
    LAUNCH(node_sizes_kernel, nodes, nodes, R, size);
    LAUNCH(linkage_f64_kernel, m, m, left, right, w, size, (const float*)nullptr, n, out);
    return FHG_OK;
}

}  // namespace
}  // namespace fhg

extern "C" __attribute__((visibility("default"))) int fhg_mst_to_linkage_tree_noalloc(
    const double* sorted_mst_dev, int64_t m, double* linkage_dev, void* stream) {
    if (m <= 0) return FHG_OK;
    if (m > fhg::kNoAllocMaxEdges) {
        fhg::set_error("fhg_mst_to_linkage_tree_noalloc: %lld edges exceed the fixed scratch "
                       "limit of %lld edges (FHG_NOALLOC_MAX_EDGES); use "
                       "fhg_mst_to_linkage_tree",
                       (long long)m, (long long)fhg::kNoAllocMaxEdges);
        return FHG_ERR_INVALID;
    }
    if (!sorted_mst_dev || !linkage_dev) {
        fhg::set_error("fhg_mst_to_linkage_tree_noalloc: null pointer argument");
        return FHG_ERR_INVALID;
    }
    return fhg::link_presorted_noalloc(sorted_mst_dev, m, linkage_dev,
                                       reinterpret_cast<cudaStream_t>(stream));
}
