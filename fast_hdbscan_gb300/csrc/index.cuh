// The spatial index shared by the kNN and Boruvka kernels.
//
// HBM layout (n points, p = 4 floats per point for d <= 4, 8 for d <= 8):
//   pts   [n][p]  float32  points in Morton order, padded with zeros
//   orig  [n]     int32    Morton position -> caller index
//   rank  [n]     int32    caller index -> Morton position
//   box   [nodes][2][p]    float32 lower / upper corner of every tree node
// Buckets of kLeaf = 32 consecutive Morton positions are the leaves of an
// implicit complete binary tree with `slots` (a power of two) leaf slots:
// node i has children 2i+1 and 2i+2, and leaf slot s is node slots-1+s.
// Slots past the last bucket carry an empty box (lo = +inf, hi = -inf).
#pragma once
#include "fhg_common.cuh"

struct fhg_index {
    int64_t n = 0;
    int32_t d = 0;
    int32_t pad = 4;
    int64_t nleaves = 0, slots = 0, nnodes = 0;
    float* pts = nullptr;
    int32_t* orig = nullptr;
    int32_t* rank = nullptr;
    float* box = nullptr;
};

namespace fhg {

struct IndexView {
    int64_t n, nleaves, slots;
    const float* __restrict__ pts;
    const int32_t* __restrict__ orig;
    const int32_t* __restrict__ rank;
    const float* __restrict__ box;
};

inline IndexView view_of(const fhg_index& ix) {
    return IndexView{ix.n, ix.nleaves, ix.slots, ix.pts, ix.orig, ix.rank, ix.box};
}

// Squared float32 distance with every multiply and add rounded separately,
// in dimension order (the reference's rdist).
template <int P>
__device__ __forceinline__ float rdist_rn(const float* a, const float* b) {
    float r = 0.0f;
#pragma unroll
    for (int j = 0; j < P; ++j) {
        float df = __fsub_rn(a[j], b[j]);
        r = __fadd_rn(r, __fmul_rn(df, df));
    }
    return r;
}

// Squared distance from a point to a box (the reference's
// point_to_node_lower_bound_rdist); never exceeds rdist_rn to any point
// inside the box.
template <int P>
__device__ __forceinline__ float box_lb(const float* __restrict__ box, const float* q) {
    float r = 0.0f;
#pragma unroll
    for (int j = 0; j < P; ++j) {
        float lo = box[j], hi = box[P + j];
        float dlo = lo > q[j] ? __fsub_rn(lo, q[j]) : 0.0f;
        float dhi = q[j] > hi ? __fsub_rn(q[j], hi) : 0.0f;
        float dd = __fadd_rn(dlo, dhi);
        r = __fadd_rn(r, __fmul_rn(dd, dd));
    }
    return r;
}

// box_lb over the first DIM coordinates of a box stored with SP floats per
// corner (padded coordinates are zero on both sides and contribute nothing).
template <int DIM, int SP>
__device__ __forceinline__ float box_lb_n(const float* __restrict__ box, const float* q) {
    float r = 0.0f;
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
        float lo = box[j], hi = box[SP + j];
        float dlo = lo > q[j] ? __fsub_rn(lo, q[j]) : 0.0f;
        float dhi = q[j] > hi ? __fsub_rn(q[j], hi) : 0.0f;
        float dd = __fadd_rn(dlo, dhi);
        r = __fadd_rn(r, __fmul_rn(dd, dd));
    }
    return r;
}

template <int P>
__device__ __forceinline__ void load_pt(const float* __restrict__ pts, int64_t i, float* out) {
    const float4* p4 = reinterpret_cast<const float4*>(pts) + (P / 4) * i;
#pragma unroll
    for (int h = 0; h < P / 4; ++h) {
        const float4 v = __ldg(p4 + h);
        out[4 * h] = v.x; out[4 * h + 1] = v.y; out[4 * h + 2] = v.z; out[4 * h + 3] = v.w;
    }
}

template <int P>
__device__ __forceinline__ void load_box(const float* __restrict__ box, int64_t node, float* out) {
    const float4* b4 = reinterpret_cast<const float4*>(box + node * 2 * P);
#pragma unroll
    for (int j = 0; j < 2 * P / 4; ++j) {
        float4 v = __ldg(b4 + j);
        out[4 * j] = v.x; out[4 * j + 1] = v.y; out[4 * j + 2] = v.z; out[4 * j + 3] = v.w;
    }
}

int index_build(const float* X, int64_t n, int32_t d, cudaStream_t s, fhg_index** out);
int index_free(fhg_index* ix, cudaStream_t s);

// kNN over the index.  Outputs (all nullable):
//   d_s/i_s : rows in Morton order, neighbour ids as Morton positions
//   d_o/i_o : rows in caller order, neighbour ids as caller indices (i_o may
//             be given alone; then its rows may have their own stride and
//             drop their first io_skip columns -- the neighbours[:, 1:]
//             matrix of the fit)
//   tie_s   : per point (Morton order), 1 when some point outside its list
//             lies at exactly its k-th distance
// A capped kNN pass (all members nullable, Morton order): cap2 = every
// query's squared search radius; queries with fewer than k points within it
// get fail = 1 (and fail_count, if given, counts them) and no output.
// redo: only these queries search (uncapped).  scan_count (nullable, any
// pass): adds the number of buckets the pass scanned.
struct KnnCap {
    const float* cap2 = nullptr;
    const uint8_t* redo = nullptr;
    uint8_t* fail = nullptr;
    unsigned long long* fail_count = nullptr;
    unsigned long long* scan_count = nullptr;
};
// Longest kNN list: lists of up to 64 are kept in registers, longer ones (a
// warp per query) in shared memory.
constexpr int kKnnMaxK = 2048;
int index_knn(const fhg_index& ix, int k, float* d_s, int32_t* i_s, float* d_o, int32_t* i_o,
              cudaStream_t s, int8_t* tie_s = nullptr, int io_stride = 0, int io_skip = 0,
              const KnnCap& cap = KnnCap());

}  // namespace fhg
