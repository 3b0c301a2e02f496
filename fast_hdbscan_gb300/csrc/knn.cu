// Exact k-nearest-neighbour search (core distances), warp-cooperative.
//
// One warp owns one bucket of 32 Morton-consecutive query points (lane =
// query).  The warp walks the bucket tree depth-first with a shared stack in
// shared memory; a node is entered when ANY lane's lower bound is within
// that lane's current k-th distance.  At a leaf, lane t loads candidate t of
// the bucket (one coalesced 16/32-byte load per lane) and the 32 candidates
// are broadcast with warp shuffles, so every query sees every candidate of
// the leaf without divergent global loads.  Each lane keeps a sorted top-K
// list in registers (fully unrolled compare-exchange insertion).
//
// Ordering: (squared distance, caller index), ascending -- the reference's
// parallel_tree_query order with equal distances ordered by index.
// Replaces numba_kdtree.py:680-792 (tree_query_recursion, simple_heap_push,
// deheap_sort, parallel_tree_query).
#include "index.cuh"

namespace fhg {
namespace {

constexpr int kKnnWarps = 4;
constexpr int kStack = 64;

template <int P, int K>
__global__ void __launch_bounds__(kKnnWarps * 32) knn_kernel(IndexView ix, int k,
                                                              float* __restrict__ d_s,
                                                              int32_t* __restrict__ i_s,
                                                              float* __restrict__ d_o,
                                                              int32_t* __restrict__ i_o) {
    __shared__ int32_t s_stack[kKnnWarps][kStack];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t leaf = (int64_t)blockIdx.x * kKnnWarps + warp;
    if (leaf >= ix.nleaves) return;
    const int64_t qi = leaf * kLeaf + lane;
    const bool valid = qi < ix.n;
    float q[P];
    if (valid) load_pt<P>(ix.pts, qi, q);
    else
#pragma unroll
        for (int j = 0; j < P; ++j) q[j] = 0.0f;

    // Centre of this bucket's box: orders children (nearer first).
    float ctr[P];
    {
        float b[2 * P];
        load_box<P>(ix.box, ix.slots - 1 + leaf, b);
#pragma unroll
        for (int j = 0; j < P; ++j) ctr[j] = 0.5f * (b[j] + b[P + j]);
    }

    // Slots [0, K-k) hold a -1 sentinel so that the live list has length k.
    float bd[K];
    int32_t bo[K], bs[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        bd[j] = (j < K - k) ? -1.0f : INFINITY;
        bo[j] = INT32_MAX;
        bs[j] = -1;
    }

    // Candidates of one bucket: lane t holds candidate t, broadcast by shuffle.
    auto scan_leaf = [&](int64_t lf, bool need) {
        const int64_t base = lf * kLeaf;
        const int cnt = (int)(ix.n - base < kLeaf ? ix.n - base : kLeaf);
        float c[P];
        int32_t co = INT32_MAX;
        if (lane < cnt) {
            load_pt<P>(ix.pts, base + lane, c);
            co = __ldg(ix.orig + base + lane);
        } else {
#pragma unroll
            for (int j = 0; j < P; ++j) c[j] = 0.0f;
        }
        for (int t = 0; t < cnt; ++t) {
            float cc[P];
#pragma unroll
            for (int j = 0; j < P; ++j) cc[j] = __shfl_sync(kFull, c[j], t);
            const int32_t o = __shfl_sync(kFull, co, t);
            const float dd = rdist_rn<P>(q, cc);
            if (need && (dd < bd[K - 1] || (dd == bd[K - 1] && o < bo[K - 1]))) {
                bd[K - 1] = dd;
                bo[K - 1] = o;
                bs[K - 1] = (int32_t)(base + t);
#pragma unroll
                for (int j = K - 1; j > 0; --j) {
                    const bool sw = bd[j] < bd[j - 1] || (bd[j] == bd[j - 1] && bo[j] < bo[j - 1]);
                    if (sw) {
                        float tf = bd[j]; bd[j] = bd[j - 1]; bd[j - 1] = tf;
                        int32_t ti = bo[j]; bo[j] = bo[j - 1]; bo[j - 1] = ti;
                        ti = bs[j]; bs[j] = bs[j - 1]; bs[j - 1] = ti;
                    }
                }
            }
        }
    };

    // Seed with the warp's own bucket (it holds the queries themselves), so
    // that the walk below starts with a tight k-th distance; the walk then
    // skips this bucket.
    scan_leaf(leaf, valid);

    int32_t* st = s_stack[warp];
    int sp = 1;
    if (lane == 0) st[0] = 0;
    __syncwarp();
    const int64_t first_leaf_node = ix.slots - 1;
    const int64_t home_node = first_leaf_node + leaf;
    while (sp > 0) {
        --sp;
        const int32_t node = st[sp];
        __syncwarp();
        if (node == home_node) continue;
        float b[2 * P];
        load_box<P>(ix.box, node, b);
        const float lb = box_lb<P>(b, q);
        const bool need = valid && lb <= bd[K - 1];
        if (!__any_sync(kFull, need)) continue;
        if (node >= first_leaf_node) {
            scan_leaf(node - first_leaf_node, need);
        } else {
            const int32_t l = 2 * node + 1, r = l + 1;
            float bl[2 * P], br[2 * P];
            load_box<P>(ix.box, l, bl);
            load_box<P>(ix.box, r, br);
            const float ll = box_lb<P>(bl, ctr), lr = box_lb<P>(br, ctr);
            const int32_t near = ll <= lr ? l : r, far = ll <= lr ? r : l;
            if (lane == 0) {
                st[sp] = far;
                st[sp + 1] = near;
            }
            sp += 2;
            __syncwarp();
        }
    }
    if (!valid) return;
    const int64_t o_row = ix.orig[qi];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        if (j < K - k) continue;
        const int jj = j - (K - k);
        const bool have = bs[j] >= 0;
        if (d_s) {
            d_s[qi * k + jj] = bd[j];
            i_s[qi * k + jj] = bs[j];
        }
        if (d_o) {
            d_o[o_row * k + jj] = bd[j];
            i_o[o_row * k + jj] = have ? bo[j] : -1;
        }
    }
}

template <int P, int K>
int launch_knn(const fhg_index& ix, int k, float* d_s, int32_t* i_s, float* d_o, int32_t* i_o,
               cudaStream_t s) {
    unsigned g = grid_for(ix.nleaves, kKnnWarps);
    ::fhg::note_launch();
    knn_kernel<P, K><<<g, kKnnWarps * 32, 0, s>>>(view_of(ix), k, d_s, i_s, d_o, i_o);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

template <int P>
int dispatch_k(const fhg_index& ix, int k, float* d_s, int32_t* i_s, float* d_o, int32_t* i_o,
               cudaStream_t s) {
    if (k <= 8) return launch_knn<P, 8>(ix, k, d_s, i_s, d_o, i_o, s);
    if (k <= 16) return launch_knn<P, 16>(ix, k, d_s, i_s, d_o, i_o, s);
    if (k <= 32) return launch_knn<P, 32>(ix, k, d_s, i_s, d_o, i_o, s);
    return launch_knn<P, 64>(ix, k, d_s, i_s, d_o, i_o, s);
}

}  // namespace

int index_knn(const fhg_index& ix, int k, float* d_s, int32_t* i_s, float* d_o, int32_t* i_o,
              cudaStream_t s) {
    if (k < 1 || k > 64) {
        set_error("knn: k must be in [1, 64] (got %d)", k);
        return FHG_ERR_INVALID;
    }
    if ((d_s == nullptr) != (i_s == nullptr) || (d_o == nullptr) != (i_o == nullptr)) {
        set_error("knn: distance and index outputs must be given together");
        return FHG_ERR_INVALID;
    }
    Stage stage(s, "knn");
    return ix.pad == 4 ? dispatch_k<4>(ix, k, d_s, i_s, d_o, i_o, s)
                       : dispatch_k<8>(ix, k, d_s, i_s, d_o, i_o, s);
}

}  // namespace fhg
