// Spatial index build: Morton keys -> radix sort -> bucketed points ->
// bottom-up bounding boxes.  Replaces the reference's single-threaded
// median-split KD-tree build (numba_kdtree.py:410-521); the tree here only
// serves as a pruning structure, so its shape does not affect results.
#include "index.cuh"
#include "primitives.cuh"

namespace fhg {
namespace {

constexpr int kBBThreads = 256;
constexpr int kMaxDim = 32;  // bounding box layout: lo[0..32), hi[32..64)

// Per-block min/max of every dimension: partial[block][2][kMaxDim].  MAXD is
// 8 or kMaxDim; the loops are unrolled and predicated on d (no local memory).
template <int MAXD>
__global__ void bbox_partial_kernel(const float* __restrict__ X, int64_t n, int d,
                                    float* __restrict__ partial) {
    float lo[MAXD], hi[MAXD];
#pragma unroll
    for (int j = 0; j < MAXD; ++j) {
        lo[j] = INFINITY;
        hi[j] = -INFINITY;
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int j = 0; j < MAXD; ++j) {
            if (j < d) {
                float v = X[i * d + j];
                lo[j] = fminf(lo[j], v);
                hi[j] = fmaxf(hi[j], v);
            }
        }
    }
    __shared__ float s_lo[kBBThreads / 32][MAXD], s_hi[kBBThreads / 32][MAXD];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < MAXD; ++j) {
        float a = lo[j], b = hi[j];
        for (int o = 16; o; o >>= 1) {
            a = fminf(a, __shfl_xor_sync(kFull, a, o));
            b = fmaxf(b, __shfl_xor_sync(kFull, b, o));
        }
        if (lane == 0) {
            s_lo[w][j] = a;
            s_hi[w][j] = b;
        }
    }
    __syncthreads();
    if (threadIdx.x < MAXD) {
        float a = INFINITY, b = -INFINITY;
        for (int ww = 0; ww < kBBThreads / 32; ++ww) {
            a = fminf(a, s_lo[ww][threadIdx.x]);
            b = fmaxf(b, s_hi[ww][threadIdx.x]);
        }
        partial[blockIdx.x * 2 * kMaxDim + threadIdx.x] = a;
        partial[blockIdx.x * 2 * kMaxDim + kMaxDim + threadIdx.x] = b;
    }
}

__global__ void bbox_final_kernel(const float* __restrict__ partial, int nb, int d, float* bb) {
    int j = threadIdx.x;  // 2 * kMaxDim threads: lo then hi
    if (j >= 2 * kMaxDim) return;
    bool is_lo = j < kMaxDim;
    float acc = is_lo ? INFINITY : -INFINITY;
    if ((j % kMaxDim) < d)
        for (int b = 0; b < nb; ++b) {
            float v = partial[b * 2 * kMaxDim + j];
            acc = is_lo ? fminf(acc, v) : fmaxf(acc, v);
        }
    bb[j] = acc;
}

// 63-bit (or less) Morton key from a common-scale quantisation of all axes
// (bits per axis = min(63 / d, 31); at least one).
template <int MAXD>
__global__ void morton_kernel(const float* __restrict__ X, int64_t n, int d,
                              const float* __restrict__ bb, int bits,
                              uint64_t* __restrict__ keys, int32_t* __restrict__ vals) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float ext = 0.0f;
#pragma unroll
    for (int j = 0; j < MAXD; ++j)
        if (j < d) ext = fmaxf(ext, bb[kMaxDim + j] - bb[j]);
    const float qmax = (float)((1ull << bits) - 1ull);
    const float scale = ext > 0.0f ? qmax / ext : 0.0f;
    uint32_t q[MAXD];
#pragma unroll
    for (int j = 0; j < MAXD; ++j) {
        q[j] = 0;
        if (j < d) {
            float t = (X[i * d + j] - bb[j]) * scale;
            t = fminf(fmaxf(t, 0.0f), qmax);
            q[j] = (uint32_t)t;
        }
    }
    uint64_t key = 0;
    for (int b = 0; b < bits; ++b) {
#pragma unroll
        for (int j = 0; j < MAXD; ++j)
            if (j < d) key |= (uint64_t)((q[j] >> b) & 1u) << (b * d + j);
    }
    keys[i] = key;
    vals[i] = (int32_t)i;
}

__global__ void gather_points_kernel(const float* __restrict__ X, int64_t n, int d, int pad,
                                     const int32_t* __restrict__ orig, float* __restrict__ pts,
                                     int32_t* __restrict__ rank) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int32_t o = orig[s];
    for (int j = 0; j < pad; ++j) pts[s * pad + j] = j < d ? X[(int64_t)o * d + j] : 0.0f;
    rank[o] = (int32_t)s;
}

// One warp per leaf slot; box[node] = bounds of its (up to 32) points.
template <int P>
__global__ void leaf_box_kernel(const float* __restrict__ pts, int64_t n, int64_t nleaves,
                                int64_t slots, float* __restrict__ box) {
    int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (leaf >= slots) return;
    int64_t i = leaf * kLeaf + lane;
    bool valid = leaf < nleaves && i < n;
    float p[P];
    if (valid) load_pt<P>(pts, i, p);
    float* out = box + (slots - 1 + leaf) * 2 * P;
#pragma unroll
    for (int j = 0; j < P; ++j) {
        float a = valid ? p[j] : INFINITY, b = valid ? p[j] : -INFINITY;
        for (int o = 16; o; o >>= 1) {
            a = fminf(a, __shfl_xor_sync(kFull, a, o));
            b = fmaxf(b, __shfl_xor_sync(kFull, b, o));
        }
        if (lane == 0) {
            out[j] = a;
            out[P + j] = b;
        }
    }
}

template <int P>
__global__ void level_box_kernel(float* __restrict__ box, int64_t first, int64_t count) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    int64_t node = first + t;
    const float* l = box + (2 * node + 1) * 2 * P;
    const float* r = box + (2 * node + 2) * 2 * P;
    float* o = box + node * 2 * P;
#pragma unroll
    for (int j = 0; j < P; ++j) {
        o[j] = fminf(l[j], r[j]);
        o[P + j] = fmaxf(l[P + j], r[P + j]);
    }
}

template <int P>
int build_boxes(fhg_index* ix, cudaStream_t s) {
    unsigned g = grid_for(ix->slots * 32, 256);
    ::fhg::note_launch();
    leaf_box_kernel<P><<<g, 256, 0, s>>>(ix->pts, ix->n, ix->nleaves, ix->slots, ix->box);
    FHG_CUDA(cudaGetLastError());
    for (int64_t width = ix->slots / 2; width >= 1; width /= 2) {
        int64_t first = width - 1;
        ::fhg::note_launch();
        level_box_kernel<P><<<grid_for(width, 256), 256, 0, s>>>(ix->box, first, width);
        FHG_CUDA(cudaGetLastError());
    }
    return FHG_OK;
}

int index_alloc(fhg_index* ix, cudaStream_t s) {
    cudaMemPool_t pool;
    FHG_TRY(device_pool(&pool));
    FHG_CUDA(cudaMallocFromPoolAsync(&ix->pts, sizeof(float) * ix->n * ix->pad + 16, pool, s));
    FHG_CUDA(cudaMallocFromPoolAsync(&ix->orig, sizeof(int32_t) * ix->n + 16, pool, s));
    FHG_CUDA(cudaMallocFromPoolAsync(&ix->rank, sizeof(int32_t) * ix->n + 16, pool, s));
    FHG_CUDA(cudaMallocFromPoolAsync(&ix->box, sizeof(float) * ix->nnodes * 2 * ix->pad + 16,
                                     pool, s));
    return FHG_OK;
}

}  // namespace

int index_free(fhg_index* ix, cudaStream_t s) {
    if (!ix) return FHG_OK;
    if (ix->pts) cudaFreeAsync(ix->pts, s);
    if (ix->orig) cudaFreeAsync(ix->orig, s);
    if (ix->rank) cudaFreeAsync(ix->rank, s);
    if (ix->box) cudaFreeAsync(ix->box, s);
    delete ix;
    return FHG_OK;
}

int index_build(const float* X, int64_t n, int32_t d, cudaStream_t s, fhg_index** out) {
    *out = nullptr;
    if (n < 1 || d < 1 || d > kMaxDim) {
        set_error("index_build: need n >= 1 and 1 <= d <= 32 (got n=%lld, d=%d)", (long long)n, d);
        return FHG_ERR_INVALID;
    }
    if (n >= ((int64_t)1 << 31) - 64) {
        set_error("index_build: n must be below 2^31");
        return FHG_ERR_INVALID;
    }
    Stage stage(s, "index_build");
    fhg_index* ix = new fhg_index();
    ix->n = n;
    ix->d = d;
    ix->pad = d <= 4 ? 4 : (d <= 8 ? 8 : (d <= 16 ? 16 : 32));
    ix->nleaves = (n + kLeaf - 1) / kLeaf;
    ix->slots = 1;
    while (ix->slots < ix->nleaves) ix->slots *= 2;
    ix->nnodes = 2 * ix->slots - 1;
    int rc = index_alloc(ix, s);
    if (rc != FHG_OK) {
        index_free(ix, s);
        return rc;
    }
    {
        Workspace ws(s);
        float *partial, *bb;
        uint64_t* keys;
        int nb = (int)std::min<int64_t>(1024, (n + kBBThreads - 1) / kBBThreads);
        rc = ws.alloc(&partial, (size_t)nb * 2 * kMaxDim);
        if (rc == FHG_OK) rc = ws.alloc(&bb, 2 * kMaxDim);
        if (rc == FHG_OK) rc = ws.alloc(&keys, (size_t)n);
        if (rc == FHG_OK) {
            ::fhg::note_launch();
            if (d <= 8) bbox_partial_kernel<8><<<nb, kBBThreads, 0, s>>>(X, n, d, partial);
            else bbox_partial_kernel<kMaxDim><<<nb, kBBThreads, 0, s>>>(X, n, d, partial);
            ::fhg::note_launch();
            bbox_final_kernel<<<1, 2 * kMaxDim, 0, s>>>(partial, nb, d, bb);
            int bits = std::max(1, std::min(63 / d, 31));
            ::fhg::note_launch();
            if (d <= 8)
                morton_kernel<8><<<grid_for(n, 256), 256, 0, s>>>(X, n, d, bb, bits, keys,
                                                                   ix->orig);
            else
                morton_kernel<kMaxDim><<<grid_for(n, 256), 256, 0, s>>>(X, n, d, bb, bits, keys,
                                                                        ix->orig);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) {
                set_error("morton kernels: %s", cudaGetErrorString(e));
                rc = FHG_ERR_CUDA;
            } else {
                rc = radix_sort_u64(ws, keys, ix->orig, n, 0, bits * d);
            }
        }
        if (rc == FHG_OK) {
            ::fhg::note_launch();
            gather_points_kernel<<<grid_for(n, 256), 256, 0, s>>>(X, n, d, ix->pad, ix->orig,
                                                                  ix->pts, ix->rank);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) {
                set_error("gather kernel: %s", cudaGetErrorString(e));
                rc = FHG_ERR_CUDA;
            }
        }
        if (rc == FHG_OK) {
            switch (ix->pad) {
                case 4: rc = build_boxes<4>(ix, s); break;
                case 8: rc = build_boxes<8>(ix, s); break;
                case 16: rc = build_boxes<16>(ix, s); break;
                default: rc = build_boxes<32>(ix, s); break;
            }
        }
    }
    if (rc != FHG_OK) {
        index_free(ix, s);
        return rc;
    }
    *out = ix;
    return FHG_OK;
}

}  // namespace fhg
