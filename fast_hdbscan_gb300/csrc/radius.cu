// Learned kNN search radius.  A small network predicts every point's log
// core distance (the log of its k-th neighbour distance) from where it sits
// in the spatial index; the kNN kernel then starts each query with that
// radius (times a safety margin) as its bound and certifies the answer: a
// query with fewer than k points inside its radius is searched again without
// a bound.  The kNN output is therefore exactly the plain one whatever the
// prediction; a good prediction only prunes the search earlier.
//
// Features (11 per point): the first three coordinates scaled to the index's
// bounding box, and for the point's bucket and the 7 tree nodes above it the
// log point density (log points - log box volume).  The network standardises
// them with its own means and deviations.
//
// Network 11 -> 64 -> 64 -> 1 with ReLU, bfloat16 operands and float32
// accumulation, defined as
//   x  = bf16((f - mu) / sigma)                       (11, padded to 16)
//   h1 = bf16(relu(bf16(W1) x + b1))
//   h2 = relu(bf16(W2) h1 + b2)                        (float32)
//   y  = bf16(w3) . h2 + b3
// The master weights are float32.  Inference runs layers 1 and 2 on the
// tensor cores (mma.sync m16n8k16, 16 points per warp-tile, weights held in
// registers); training runs its own scalar forward, backward, gradient and
// Adam kernels with the same rounding points (gradients pass through the
// bfloat16 roundings unchanged), one step captured in a CUDA graph.
//
// Parameter block (float32, kRadiusParams): W1[64][11] b1[64] W2[64][64]
// b2[64] w3[64] b3 mu[11] sigma[11].
#include <cuda_bf16.h>

#include <algorithm>

#include "radius.cuh"

namespace fhg {

namespace {

constexpr int kRIn = 11, kRHid = 64, kRLevels = 8;
constexpr int kRW1 = 0, kRB1 = kRW1 + kRHid * kRIn, kRW2 = kRB1 + kRHid,
              kRB2 = kRW2 + kRHid * kRHid, kRW3 = kRB2 + kRHid, kRB3 = kRW3 + kRHid,
              kRMu = kRB3 + 1, kRSig = kRMu + kRIn, kRAll = kRSig + kRIn;
constexpr int kRTrain = kRMu;  // trained parameters: everything before mu
static_assert(kRAll == kRadiusParams, "parameter block size");

__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// ------------------------------------------------------------- features
// Per Morton position p; written to row orig[p] when orig is given, else p.
template <int SP>
__global__ void features_kernel(IndexView ix, int d, const int32_t* __restrict__ orig,
                                float* __restrict__ feat) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= ix.n) return;
    float x[SP], root[2 * SP];
    load_pt<SP>(ix.pts, p, x);
    load_box<SP>(ix.box, 0, root);
    float f[kRIn];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const float ext = j < d ? root[SP + j] - root[j] : 0.0f;
        f[j] = (j < d && ext > 0.0f) ? (x[j] - root[j]) / ext : 0.0f;
    }
    const int64_t leaf = p / kLeaf;
    int64_t node = ix.slots - 1 + leaf;
#pragma unroll
    for (int L = 0; L < kRLevels; ++L) {
        float b[2 * SP];
        load_box<SP>(ix.box, node, b);
        const int64_t first = (leaf >> L) << L;  // first leaf slot under the node
        const int64_t pts = min(ix.n, (first + ((int64_t)1 << L)) * kLeaf) - first * kLeaf;
        float logvol = 0.0f;
#pragma unroll
        for (int j = 0; j < SP; ++j)
            if (j < d) logvol += logf(fmaxf(b[SP + j] - b[j], 1e-6f));
        f[3 + L] = logf((float)max(pts, (int64_t)1)) - logvol;
        if (node > 0) node = (node - 1) >> 1;
    }
    const int64_t row = orig ? orig[p] : p;
#pragma unroll
    for (int j = 0; j < kRIn; ++j) feat[row * kRIn + j] = f[j];
}

// ------------------------------------------------------------- inference
__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One warp per tile of 16 points (grid-stride).  Fragment layout of
// m16n8k16 (g = lane / 4, t = lane % 4): A holds rows g and g + 8 at columns
// 2t, 2t+1 and 2t+8, 2t+9; B holds column g at rows 2t, 2t+1 and 2t+8, 2t+9;
// C holds rows g and g + 8 at columns 2t, 2t+1.  A layer's C tiles for
// columns [16kb, 16kb+16) are the next layer's A fragment for k-block kb.
// Output: y (log radius, nullable) and cap2 = (exp(y) margin)^2 (nullable).
__global__ void __launch_bounds__(128) predict_kernel(int64_t n, const float* __restrict__ prm,
                                                      const float* __restrict__ feat, float margin,
                                                      float* __restrict__ out_y,
                                                      float* __restrict__ cap2) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    // the weights as B fragments, once per warp
    uint32_t w1[8][2], w2[4][8][2];
    float b1v[8][2], b2v[8][2], w3v[8][2];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int o = nt * 8 + g;
        const int k0 = 2 * t, k1 = 2 * t + 8;
        w1[nt][0] = pack_bf2(k0 < kRIn ? prm[kRW1 + o * kRIn + k0] : 0.0f,
                             k0 + 1 < kRIn ? prm[kRW1 + o * kRIn + k0 + 1] : 0.0f);
        w1[nt][1] = pack_bf2(k1 < kRIn ? prm[kRW1 + o * kRIn + k1] : 0.0f,
                             k1 + 1 < kRIn ? prm[kRW1 + o * kRIn + k1 + 1] : 0.0f);
#pragma unroll
        for (int kb = 0; kb < 4; ++kb) {
            const float* r = prm + kRW2 + o * kRHid + kb * 16;
            w2[kb][nt][0] = pack_bf2(r[2 * t], r[2 * t + 1]);
            w2[kb][nt][1] = pack_bf2(r[2 * t + 8], r[2 * t + 9]);
        }
        const int c = nt * 8 + 2 * t;
        b1v[nt][0] = prm[kRB1 + c];
        b1v[nt][1] = prm[kRB1 + c + 1];
        b2v[nt][0] = prm[kRB2 + c];
        b2v[nt][1] = prm[kRB2 + c + 1];
        w3v[nt][0] = bf(prm[kRW3 + c]);
        w3v[nt][1] = bf(prm[kRW3 + c + 1]);
    }
    const float b3 = prm[kRB3];
    float mu[4], sg[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int j = (e < 2 ? 2 * t : 2 * t + 8) + (e & 1);
        mu[e] = j < kRIn ? prm[kRMu + j] : 0.0f;
        sg[e] = j < kRIn ? prm[kRSig + j] : 1.0f;
    }
    const int64_t tiles = (n + 15) / 16;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t tile = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile < tiles;
         tile += warps) {
        const int64_t r0 = tile * 16 + g, r1 = r0 + 8;
        float xv[2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int64_t r = h ? r1 : r0;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int j = (e < 2 ? 2 * t : 2 * t + 8) + (e & 1);
                xv[h][e] = (r < n && j < kRIn) ? (feat[r * kRIn + j] - mu[e]) / sg[e] : 0.0f;
            }
        }
        const uint32_t a1[4] = {pack_bf2(xv[0][0], xv[0][1]), pack_bf2(xv[1][0], xv[1][1]),
                                pack_bf2(xv[0][2], xv[0][3]), pack_bf2(xv[1][2], xv[1][3])};
        float h1[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            h1[nt][0] = b1v[nt][0];
            h1[nt][1] = b1v[nt][1];
            h1[nt][2] = b1v[nt][0];
            h1[nt][3] = b1v[nt][1];
            mma_bf16(h1[nt], a1, w1[nt][0], w1[nt][1]);
        }
        uint32_t a2[4][4];
#pragma unroll
        for (int kb = 0; kb < 4; ++kb) {
            const float* lo = h1[2 * kb];
            const float* hi = h1[2 * kb + 1];
            a2[kb][0] = pack_bf2(fmaxf(lo[0], 0.0f), fmaxf(lo[1], 0.0f));
            a2[kb][1] = pack_bf2(fmaxf(lo[2], 0.0f), fmaxf(lo[3], 0.0f));
            a2[kb][2] = pack_bf2(fmaxf(hi[0], 0.0f), fmaxf(hi[1], 0.0f));
            a2[kb][3] = pack_bf2(fmaxf(hi[2], 0.0f), fmaxf(hi[3], 0.0f));
        }
        float y0 = 0.0f, y1 = 0.0f;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            float acc[4] = {b2v[nt][0], b2v[nt][1], b2v[nt][0], b2v[nt][1]};
#pragma unroll
            for (int kb = 0; kb < 4; ++kb) mma_bf16(acc, a2[kb], w2[kb][nt][0], w2[kb][nt][1]);
            y0 += w3v[nt][0] * fmaxf(acc[0], 0.0f) + w3v[nt][1] * fmaxf(acc[1], 0.0f);
            y1 += w3v[nt][0] * fmaxf(acc[2], 0.0f) + w3v[nt][1] * fmaxf(acc[3], 0.0f);
        }
        y0 += __shfl_xor_sync(0xffffffffu, y0, 1);
        y0 += __shfl_xor_sync(0xffffffffu, y0, 2);
        y1 += __shfl_xor_sync(0xffffffffu, y1, 1);
        y1 += __shfl_xor_sync(0xffffffffu, y1, 2);
        if (t == 0) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int64_t r = h ? r1 : r0;
                if (r >= n) continue;
                const float y = (h ? y1 : y0) + b3;
                if (out_y) out_y[r] = y;
                if (cap2) {
                    const float rad = expf(y) * margin;
                    const float c = rad * rad;
                    cap2[r] = c >= 0.0f ? c : INFINITY;  // NaN: no cap
                }
            }
        }
    }
}

// ------------------------------------------------------------- training
// Sample s of a step takes point hash(seed, step, s) mod n (splitmix64).
__device__ __forceinline__ int64_t sample_of(uint64_t seed, int64_t step, int64_t s, int64_t n) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(step * 1000003 + s + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (int64_t)(z % (uint64_t)n);
}

// Forward pass of a batch, one thread per sample: keeps x, h1 (bf16 values),
// h2 and the loss gradient dy = 2 (y - target) / B; adds the batch's mean
// squared error to *loss.  rows (nullable): the batch's sample indices.
__global__ void train_fwd_kernel(int64_t B, int64_t n, const float* __restrict__ prm,
                                 const float* __restrict__ feat, const float* __restrict__ tgt,
                                 const int64_t* __restrict__ step, uint64_t seed,
                                 const int32_t* __restrict__ rows, float* __restrict__ X,
                                 float* __restrict__ H1, float* __restrict__ H2,
                                 float* __restrict__ DY, float* __restrict__ loss) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B) return;
    const int64_t i = rows ? rows[s] : sample_of(seed, *step, s, n);
    float x[kRIn], h1[kRHid];
    for (int j = 0; j < kRIn; ++j) {
        x[j] = bf((feat[i * kRIn + j] - prm[kRMu + j]) / prm[kRSig + j]);
        X[s * kRIn + j] = x[j];
    }
    for (int o = 0; o < kRHid; ++o) {
        float a = prm[kRB1 + o];
        for (int j = 0; j < kRIn; ++j) a += bf(prm[kRW1 + o * kRIn + j]) * x[j];
        h1[o] = bf(fmaxf(a, 0.0f));
        H1[s * kRHid + o] = h1[o];
    }
    float y = prm[kRB3];
    for (int o = 0; o < kRHid; ++o) {
        float a = prm[kRB2 + o];
        for (int j = 0; j < kRHid; ++j) a += bf(prm[kRW2 + o * kRHid + j]) * h1[j];
        const float h2 = fmaxf(a, 0.0f);
        H2[s * kRHid + o] = h2;
        y += bf(prm[kRW3 + o]) * h2;
    }
    const float e = y - tgt[i];
    DY[s] = 2.0f * e / (float)B;
    atomicAdd(loss, e * e / (float)B);
}

// Backward per sample: the deltas at the second and first hidden layers.
__global__ void train_bwd_kernel(int64_t B, const float* __restrict__ prm,
                                 const float* __restrict__ H1, const float* __restrict__ H2,
                                 const float* __restrict__ DY, float* __restrict__ D2,
                                 float* __restrict__ D1) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B) return;
    const float dy = DY[s];
    float d2[kRHid];
    for (int o = 0; o < kRHid; ++o) {
        d2[o] = H2[s * kRHid + o] > 0.0f ? dy * bf(prm[kRW3 + o]) : 0.0f;
        D2[s * kRHid + o] = d2[o];
    }
    for (int j = 0; j < kRHid; ++j) {
        float a = 0.0f;
        for (int o = 0; o < kRHid; ++o) a += bf(prm[kRW2 + o * kRHid + j]) * d2[o];
        D1[s * kRHid + j] = H1[s * kRHid + j] > 0.0f ? a : 0.0f;
    }
}

// Every trained parameter's gradient summed over the batch: one warp per
// parameter, lanes over samples, a fixed reduction order.
__global__ void train_grad_kernel(int64_t B, const float* __restrict__ X,
                                  const float* __restrict__ H1, const float* __restrict__ H2,
                                  const float* __restrict__ DY, const float* __restrict__ D2,
                                  const float* __restrict__ D1, float* __restrict__ G) {
    const int t = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (t >= kRTrain) return;
    float g = 0.0f;
    if (t < kRB1) {  // W1[o][j]
        const int o = t / kRIn, j = t % kRIn;
        for (int64_t s = lane; s < B; s += 32) g += D1[s * kRHid + o] * X[s * kRIn + j];
    } else if (t < kRW2) {
        const int o = t - kRB1;
        for (int64_t s = lane; s < B; s += 32) g += D1[s * kRHid + o];
    } else if (t < kRB2) {  // W2[o][j]
        const int o = (t - kRW2) / kRHid, j = (t - kRW2) % kRHid;
        for (int64_t s = lane; s < B; s += 32) g += D2[s * kRHid + o] * H1[s * kRHid + j];
    } else if (t < kRW3) {
        const int o = t - kRB2;
        for (int64_t s = lane; s < B; s += 32) g += D2[s * kRHid + o];
    } else if (t < kRB3) {
        const int o = t - kRW3;
        for (int64_t s = lane; s < B; s += 32) g += DY[s] * H2[s * kRHid + o];
    } else {
        for (int64_t s = lane; s < B; s += 32) g += DY[s];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) g += __shfl_xor_sync(0xffffffffu, g, o);
    if (lane == 0) G[t] = g;
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8) at step *step + 1; the counter is
// advanced by the next kernel so that every thread here sees the same step.
__global__ void adam_kernel(float* __restrict__ prm, const float* __restrict__ G,
                            float* __restrict__ M, float* __restrict__ V,
                            const int64_t* __restrict__ step, float lr) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kRTrain) return;
    const float k = (float)(*step + 1);
    const float m = 0.9f * M[t] + 0.1f * G[t];
    const float v = 0.999f * V[t] + 0.001f * G[t] * G[t];
    M[t] = m;
    V[t] = v;
    const float mh = m / (1.0f - powf(0.9f, k)), vh = v / (1.0f - powf(0.999f, k));
    prm[t] -= lr * mh / (sqrtf(vh) + 1e-8f);
}
__global__ void step_advance_kernel(int64_t* step, const float* loss, float* curve) {
    if (curve) curve[*step] = *loss;
    *step += 1;
}

// Initial parameters: the feature means and deviations and the target mean
// over all n rows (one block per column, a fixed summation order).
__global__ void __launch_bounds__(256) init_stats_kernel(int64_t n, const float* __restrict__ feat,
                                                         const float* __restrict__ tgt,
                                                         float* __restrict__ prm) {
    __shared__ double s1[256], s2[256];
    const int col = blockIdx.x;  // 0..10 features, 11 the target
    double a = 0.0, b = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = col < kRIn ? feat[i * kRIn + col] : tgt[i];
        a += v;
        b += v * v;
    }
    s1[threadIdx.x] = a;
    s2[threadIdx.x] = b;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            s1[threadIdx.x] += s1[threadIdx.x + w];
            s2[threadIdx.x] += s2[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double mean = s1[0] / (double)n;
        const double var = fmax(s2[0] / (double)n - mean * mean, 0.0);
        if (col < kRIn) {
            prm[kRMu + col] = (float)mean;
            prm[kRSig + col] = (float)fmax(sqrt(var), 1e-3);
        } else {
            prm[kRB3] = (float)mean;
        }
    }
}
// He-normal weights (Box-Muller on counter-hashed uniforms), zero biases.
__global__ void init_weights_kernel(float* __restrict__ prm, uint64_t seed) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kRB3) return;
    float scale = 0.0f;
    if (t < kRB1) scale = sqrtf(2.0f / kRIn);
    else if (t >= kRW2 && t < kRB2) scale = sqrtf(2.0f / kRHid);
    else if (t >= kRW3) scale = sqrtf(1.0f / kRHid);
    if (scale == 0.0f) {
        prm[t] = 0.0f;
        return;
    }
    const int64_t u = sample_of(seed, 0, 2 * t, 1ll << 24), v = sample_of(seed, 0, 2 * t + 1, 1ll << 24);
    const float u1 = ((float)u + 0.5f) / 16777216.0f, u2 = (float)v / 16777216.0f;
    prm[t] = scale * sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

__global__ void log_core_kernel(int64_t n, int k, const float* __restrict__ rdist,
                                float* __restrict__ tgt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    tgt[i] = 0.5f * logf(fmaxf(rdist[i * k + k - 1], 1e-30f));
}

struct TrainBufs {
    float *X, *H1, *H2, *DY, *D2, *D1;
    int alloc(Workspace& ws, int64_t B) {
        FHG_TRY(ws.alloc(&X, (size_t)(B * kRIn)));
        FHG_TRY(ws.alloc(&H1, (size_t)(B * kRHid)));
        FHG_TRY(ws.alloc(&H2, (size_t)(B * kRHid)));
        FHG_TRY(ws.alloc(&D2, (size_t)(B * kRHid)));
        FHG_TRY(ws.alloc(&D1, (size_t)(B * kRHid)));
        FHG_TRY(ws.alloc(&DY, (size_t)B));
        return FHG_OK;
    }
};

thread_local RadiusUse t_use;
thread_local unsigned long long* t_fallbacks = nullptr;  // the thread's device counter

}  // namespace

const RadiusUse* radius_in_use() { return t_use.params ? &t_use : nullptr; }
void radius_set_use(const float* params, float margin) {
    t_use.params = params;
    t_use.margin = margin;
}

int radius_features(const fhg_index& ix, const int32_t* orig, float* feat, cudaStream_t s) {
    if (ix.n <= 0) return FHG_OK;
    const unsigned g = grid_for(ix.n, 256);
    ::fhg::note_launch();
    switch (ix.pad) {
        case 4: features_kernel<4><<<g, 256, 0, s>>>(view_of(ix), ix.d, orig, feat); break;
        case 8: features_kernel<8><<<g, 256, 0, s>>>(view_of(ix), ix.d, orig, feat); break;
        case 16: features_kernel<16><<<g, 256, 0, s>>>(view_of(ix), ix.d, orig, feat); break;
        default: features_kernel<32><<<g, 256, 0, s>>>(view_of(ix), ix.d, orig, feat); break;
    }
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

int radius_predict(const float* prm, const float* feat, int64_t n, float margin, float* out_y,
                   float* cap2, cudaStream_t s) {
    if (n <= 0) return FHG_OK;
    const int64_t tiles = (n + 15) / 16;
    const int64_t blocks = std::min<int64_t>((tiles + 3) / 4, 152 * 8);
    ::fhg::note_launch();
    predict_kernel<<<(unsigned)blocks, 128, 0, s>>>(n, prm, feat, margin, out_y, cap2);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

int radius_init(float* prm, const float* feat, const float* tgt, int64_t n, uint64_t seed,
                cudaStream_t s) {
    if (n <= 0) {
        set_error("radius_init: no training rows");
        return FHG_ERR_INVALID;
    }
    ::fhg::note_launch();
    init_weights_kernel<<<grid_for(kRB3, 256), 256, 0, s>>>(prm, seed);
    ::fhg::note_launch();
    init_stats_kernel<<<kRIn + 1, 256, 0, s>>>(n, feat, tgt, prm);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

int radius_targets(const fhg_index& ix, int k, float* tgt, cudaStream_t s) {
    if (ix.n <= 0) return FHG_OK;
    Workspace ws(s);
    float* rd;
    int32_t* id;
    FHG_TRY(ws.alloc(&rd, (size_t)(ix.n * k)));
    FHG_TRY(ws.alloc(&id, (size_t)(ix.n * k)));
    FHG_TRY(index_knn(ix, k, nullptr, nullptr, rd, id, s));
    ::fhg::note_launch();
    log_core_kernel<<<grid_for(ix.n, 256), 256, 0, s>>>(ix.n, k, rd, tgt);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

int radius_grad(const float* prm, const float* feat, const float* tgt, const int32_t* rows,
                int64_t B, float* grad, float* loss, cudaStream_t s) {
    if (B <= 0) {
        set_error("radius_grad: empty batch");
        return FHG_ERR_INVALID;
    }
    Workspace ws(s);
    TrainBufs tb;
    FHG_TRY(tb.alloc(ws, B));
    FHG_CUDA(cudaMemsetAsync(loss, 0, sizeof(float), s));
    const unsigned gb = grid_for(B, 128);
    ::fhg::note_launch();
    train_fwd_kernel<<<gb, 128, 0, s>>>(B, 1, prm, feat, tgt, nullptr, 0, rows, tb.X, tb.H1,
                                        tb.H2, tb.DY, loss);
    ::fhg::note_launch();
    train_bwd_kernel<<<gb, 128, 0, s>>>(B, prm, tb.H1, tb.H2, tb.DY, tb.D2, tb.D1);
    ::fhg::note_launch();
    train_grad_kernel<<<grid_for((int64_t)kRTrain * 32, 256), 256, 0, s>>>(
        B, tb.X, tb.H1, tb.H2, tb.DY, tb.D2, tb.D1, grad);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

int radius_train(float* prm, const float* feat, const float* tgt, int64_t n, int32_t steps,
                 int32_t B, float lr, uint64_t seed, float* loss_curve, cudaStream_t s) {
    if (n <= 0 || steps <= 0 || B <= 0) {
        set_error("radius_train: needs rows, steps and a batch size");
        return FHG_ERR_INVALID;
    }
    Workspace ws(s);
    TrainBufs tb;
    float *G, *M, *V, *loss;
    int64_t* step;
    FHG_TRY(tb.alloc(ws, B));
    FHG_TRY(ws.alloc(&G, (size_t)kRTrain));
    FHG_TRY(ws.alloc(&M, (size_t)kRTrain));
    FHG_TRY(ws.alloc(&V, (size_t)kRTrain));
    FHG_TRY(ws.alloc(&loss, 1));
    FHG_TRY(ws.alloc(&step, 1));
    FHG_CUDA(cudaMemsetAsync(M, 0, sizeof(float) * kRTrain, s));
    FHG_CUDA(cudaMemsetAsync(V, 0, sizeof(float) * kRTrain, s));
    FHG_CUDA(cudaMemsetAsync(step, 0, sizeof(int64_t), s));
    FHG_CUDA(cudaStreamSynchronize(s));
    // One Adam step as a graph on a private stream, replayed `steps` times;
    // each replay reads its step number from the device counter.
    cudaStream_t cs;
    FHG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const unsigned gb = grid_for(B, 128);
    int rc = FHG_OK;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        set_error("radius_train: cannot begin graph capture");
        rc = FHG_ERR_CUDA;
    } else {
        cudaMemsetAsync(loss, 0, sizeof(float), cs);
        train_fwd_kernel<<<gb, 128, 0, cs>>>(B, n, prm, feat, tgt, step, seed, nullptr, tb.X,
                                             tb.H1, tb.H2, tb.DY, loss);
        train_bwd_kernel<<<gb, 128, 0, cs>>>(B, prm, tb.H1, tb.H2, tb.DY, tb.D2, tb.D1);
        train_grad_kernel<<<grid_for((int64_t)kRTrain * 32, 256), 256, 0, cs>>>(
            B, tb.X, tb.H1, tb.H2, tb.DY, tb.D2, tb.D1, G);
        adam_kernel<<<grid_for(kRTrain, 256), 256, 0, cs>>>(prm, G, M, V, step, lr);
        step_advance_kernel<<<1, 1, 0, cs>>>(step, loss, loss_curve);
        const cudaError_t e = cudaStreamEndCapture(cs, &graph);
        if (e != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
            set_error("radius_train: graph capture failed");
            rc = FHG_ERR_CUDA;
        }
    }
    for (int32_t k = 0; k < steps && rc == FHG_OK; ++k) {
        ::fhg::note_launch();
        if (cudaGraphLaunch(exec, cs) != cudaSuccess) {
            set_error("radius_train: graph launch failed");
            rc = FHG_ERR_CUDA;
        }
    }
    const cudaError_t e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess && rc == FHG_OK) {
        set_error("radius_train: %s", cudaGetErrorString(e));
        rc = FHG_ERR_CUDA;
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    return rc;
}

// Certified kNN with a learned radius: features and the predicted radius per
// Morton position, a capped pass, then the uncapped pass over the queries the
// capped pass could not certify.  Same outputs as index_knn.
int knn_with_radius(const fhg_index& ix, int k, const RadiusUse& use, float* d_s, int32_t* i_s,
                    float* d_o, int32_t* i_o, cudaStream_t s, int8_t* tie_s, int io_stride,
                    int io_skip, unsigned long long* scans) {
    const int64_t n = ix.n;
    if (n <= 0) return index_knn(ix, k, d_s, i_s, d_o, i_o, s, tie_s, io_stride, io_skip);
    if (!t_fallbacks) FHG_CUDA(cudaMalloc(&t_fallbacks, sizeof(unsigned long long)));
    Workspace ws(s);
    float *feat, *cap2;
    uint8_t* fail;
    FHG_TRY(ws.alloc(&feat, (size_t)(n * kRIn)));
    FHG_TRY(ws.alloc(&cap2, (size_t)n));
    FHG_TRY(ws.alloc(&fail, (size_t)n));
    FHG_TRY(radius_features(ix, nullptr, feat, s));
    FHG_TRY(radius_predict(use.params, feat, n, use.margin, nullptr, cap2, s));
    FHG_CUDA(cudaMemsetAsync(fail, 0, (size_t)n, s));
    FHG_CUDA(cudaMemsetAsync(t_fallbacks, 0, sizeof(unsigned long long), s));
    KnnCap capped;
    capped.cap2 = cap2;
    capped.fail = fail;
    capped.fail_count = t_fallbacks;
    capped.scan_count = scans;
    FHG_TRY(index_knn(ix, k, d_s, i_s, d_o, i_o, s, tie_s, io_stride, io_skip, capped));
    KnnCap redo;
    redo.redo = fail;
    redo.scan_count = scans;
    return index_knn(ix, k, d_s, i_s, d_o, i_o, s, tie_s, io_stride, io_skip, redo);
}

// Buckets scanned by the kNN of every point with (params != nullptr) or
// without the learned radius; the kNN output itself is discarded.
int knn_scan_count(const fhg_index& ix, int k, const float* params, float margin, int64_t* scans,
                   int64_t* fallbacks, cudaStream_t s) {
    Workspace ws(s);
    float* rd;
    int32_t* id;
    unsigned long long* cnt;
    FHG_TRY(ws.alloc(&rd, (size_t)(std::max<int64_t>(ix.n, 1) * k)));
    FHG_TRY(ws.alloc(&id, (size_t)(std::max<int64_t>(ix.n, 1) * k)));
    FHG_TRY(ws.alloc(&cnt, 1));
    FHG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
    if (params) {
        RadiusUse use;
        use.params = params;
        use.margin = margin;
        FHG_TRY(knn_with_radius(ix, k, use, nullptr, nullptr, rd, id, s, nullptr, 0, 0, cnt));
    } else {
        KnnCap c;
        c.scan_count = cnt;
        FHG_TRY(index_knn(ix, k, nullptr, nullptr, rd, id, s, nullptr, 0, 0, c));
    }
    unsigned long long v = 0;
    FHG_CUDA(cudaMemcpyAsync(&v, cnt, sizeof(v), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    *scans = (int64_t)v;
    if (fallbacks) {
        if (params) FHG_TRY(radius_last_fallbacks(fallbacks, s));
        else *fallbacks = 0;
    }
    return FHG_OK;
}

int radius_last_fallbacks(int64_t* out, cudaStream_t s) {
    unsigned long long v = 0;
    if (t_fallbacks) {
        FHG_CUDA(cudaMemcpyAsync(&v, t_fallbacks, sizeof(v), cudaMemcpyDeviceToHost, s));
        FHG_CUDA(cudaStreamSynchronize(s));
    }
    *out = (int64_t)v;
    return FHG_OK;
}

}  // namespace fhg
