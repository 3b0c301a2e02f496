// Exact kNN for high-dimensional points (d up to 96) by brute force on the
// tensor cores, behind the reference's d > 30 route (hdbscan.py:447 ->
// nndescent.py:179 compute_mst_from_knn_graph, whose kNN graph pynndescent
// approximates; here it is exact).
//
// 1. Candidates.  The centred points c = x - mean are split into two
//    bfloat16 terms, hi = bf16(c) and lo = bf16(c - hi), and every query's
//    squared distance to every point is estimated as
//        D~ = |y_i|^2 + |y_j|^2 - 2 (hi_i.hi_j + hi_i.lo_j + lo_i.hi_j)
//    (y = hi + lo) with one bf16 GEMM of depth 3 * dp (mma.sync m16n8k16,
//    float32 accumulation).  A CTA holds 128 queries (8 warps of 16, operands
//    in registers; 64 when the buffers below need the room) and streams all
//    points through shared memory in chunks of 64 (cp.async,
//    double-buffered).  Each query keeps the L = k + 32 points
//    of smallest D~ in a shared-memory buffer: an estimate below the query's
//    current L-th value is appended, and a buffer that fills is cut back to
//    its L smallest by ranking.
// 2. Re-rank and certificate.  The L candidates' exact float32 squared
//    distances (each difference, square and sum rounded in dimension order,
//    as every kNN of the engine computes them) give the k nearest in
//    (distance, index) order.  Every other point has D~ >= T, the L-th
//    estimate, and the rounding analysis bounds the estimate's error:
//      |c - y| <= (2^-16 + 2^-23) |c|  per point (two bf16 terms),
//      |D~ - |y_i - y_j|^2| <= eta_i = (2 K + 4 dp + 16) 2^-24 (|y_i| + Ymax)^2
//                                    + 2^-15 |c_i| Cmax
//    (K = 3 dp float32 accumulations, which may truncate; the dropped
//    lo_i.lo_j term).  So every non-candidate lies at true distance at least
//      lb = sqrt(T - eta_i) - (2^-16 + 2^-23)(|c_i| + Cmax),
//    and its float32 squared distance at least lb^2 (1 - (d + 8) 2^-23).  A
//    query whose k-th exact candidate distance is below that bound is
//    certified; the others (and none is assumed rare) are searched again.
// 3. Fallback.  A warp per uncertified query scans every point in exact
//    float32 with the same buffer-and-rank selection.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <type_traits>

#include "highd.cuh"
#include "primitives.cuh"
#include "tc.cuh"

namespace fhg {
namespace {

constexpr int kHdRows = 16;     // queries per warp
constexpr int kHdChunk = 64;    // points per streamed chunk
constexpr int kHdCap = 192;     // largest candidate buffer per query (L + kHdChunk)
constexpr int kHdMaxL = 128;    // candidates kept (k + 32)
constexpr int kHdSmemMax = 227 * 1024;

__device__ __forceinline__ unsigned long long hd_key(float dist, int32_t j) {
    return ((unsigned long long)__float_as_uint(dist) << 32) | (uint32_t)j;
}
__device__ __forceinline__ float hd_dist(unsigned long long key) {
    return __uint_as_float((uint32_t)(key >> 32));
}

// Column means (one block per dimension, a fixed summation order).
__global__ void __launch_bounds__(256) hd_mean_kernel(const float* __restrict__ X, int64_t n,
                                                      int d, float* __restrict__ mu) {
    __shared__ double part[256];
    const int col = blockIdx.x;
    double a = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) a += X[i * d + col];
    part[threadIdx.x] = a;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) mu[col] = (float)(part[0] / (double)n);
}

// Per point: the operand rows A = [hi, hi, lo] and B = [hi, lo, hi] (dp
// columns each, zero-padded), |y|^2 (float32, dimension order), |c|, and the
// running maxima of |y| and |c| (float bit patterns, non-negative).
// Rows are kw >= 3 dp elements long (zero-padded: the tensor-core pipeline
// takes whole 64-element row segments).
__global__ void hd_split_kernel(const float* __restrict__ X, int64_t n, int d, int dp, int kw,
                                const float* __restrict__ mu, __nv_bfloat16* __restrict__ A,
                                __nv_bfloat16* __restrict__ B, float* __restrict__ ny,
                                float* __restrict__ cn, unsigned* __restrict__ maxes) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 3 * dp; k < kw; ++k) {
        A[i * kw + k] = __float2bfloat16_rn(0.0f);
        B[i * kw + k] = __float2bfloat16_rn(0.0f);
    }
    float y2 = 0.0f, c2 = 0.0f;
    for (int k = 0; k < dp; ++k) {
        __nv_bfloat16 hi = __float2bfloat16_rn(0.0f), lo = hi;
        if (k < d) {
            const float c = __fsub_rn(X[i * d + k], mu[k]);
            hi = __float2bfloat16_rn(c);
            lo = __float2bfloat16_rn(__fsub_rn(c, __bfloat162float(hi)));
            const float y = __fadd_rn(__bfloat162float(hi), __bfloat162float(lo));
            y2 = __fadd_rn(y2, __fmul_rn(y, y));
            c2 = __fadd_rn(c2, __fmul_rn(c, c));
        }
        A[i * kw + k] = hi;
        A[i * kw + dp + k] = hi;
        A[i * kw + 2 * dp + k] = lo;
        B[i * kw + k] = hi;
        B[i * kw + dp + k] = lo;
        B[i * kw + 2 * dp + k] = hi;
    }
    ny[i] = y2;
    const float c = sqrtf(c2);
    cn[i] = c;
    atomicMax(maxes, __float_as_uint(sqrtf(y2)));
    atomicMax(maxes + 1, __float_as_uint(c));
}

__device__ __forceinline__ void hd_mma(float (&c)[4], const uint32_t (&a)[4], uint32_t b0,
                                       uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Cuts a buffer of cnt unique keys back to its `keep` smallest, sorted: every
// lane ranks its keys against the whole buffer, then writes the kept ones at
// their ranks.  Returns the new count.
__device__ __forceinline__ int hd_cut(unsigned long long* buf, int cnt, int keep, int lane) {
    constexpr int kPer = kHdCap / 32;
    unsigned long long mine[kPer];
    int rank[kPer];
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
        const int e = lane + 32 * m;
        mine[m] = e < cnt ? buf[e] : ~0ull;
        rank[m] = 0;
    }
    for (int e = 0; e < cnt; ++e) {
        const unsigned long long o = buf[e];
#pragma unroll
        for (int m = 0; m < kPer; ++m) rank[m] += o < mine[m] ? 1 : 0;
    }
    __syncwarp();
#pragma unroll
    for (int m = 0; m < kPer; ++m)
        if (lane + 32 * m < cnt && rank[m] < keep) buf[rank[m]] = mine[m];
    __syncwarp();
    return cnt < keep ? cnt : keep;
}

// KB: k-blocks of 16 in the operand depth 3 * dp; W warps of MT m-tiles of
// 16 queries (every staged B fragment feeds MT tensor-core ops).
// cap: candidate buffer entries per query (L + kHdChunk rounded up, <= kHdCap):
// after a cut to L a buffer always has room for one chunk's estimates.
template <int KB, int W, int MT>
__global__ void __launch_bounds__(W * 32) hd_cand_kernel(
    int64_t n, int L, int cap, const __nv_bfloat16* __restrict__ A,
    const __nv_bfloat16* __restrict__ B, const float* __restrict__ ny, int32_t* __restrict__ cand,
    float* __restrict__ T) {
    constexpr int kWRows = kHdRows * MT;  // queries per warp (<= 32)
    constexpr int kHdQ = W * kWRows;
    constexpr int KW = KB * 16;
    constexpr int RS = KW + 8;  // shared row stride (bf16): conflict-free fragment loads
    static_assert(kWRows <= 32, "one lane per warp row checks its buffer");
    extern __shared__ __align__(16) unsigned char hd_smem[];
    __nv_bfloat16* Bs = reinterpret_cast<__nv_bfloat16*>(hd_smem);  // [2][kHdChunk][RS]
    unsigned long long* bufs =
        reinterpret_cast<unsigned long long*>(Bs + 2 * kHdChunk * RS);  // [kHdQ][cap]
    float* npj = reinterpret_cast<float*>(bufs + kHdQ * cap);          // [2][kHdChunk]
    int* cnt = reinterpret_cast<int*>(npj + 2 * kHdChunk);              // [kHdQ]
    float* tau = reinterpret_cast<float*>(cnt + kHdQ);                  // [kHdQ]

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int64_t q0 = (int64_t)blockIdx.x * kHdQ + warp * kWRows;
    for (int i = threadIdx.x; i < kHdQ; i += W * 32) {
        cnt[i] = 0;
        tau[i] = INFINITY;
    }
    // this warp's query rows as A fragments: m-tile mt holds rows 16 mt + g
    // (index 0) and 16 mt + g + 8 (index 1)
    uint32_t a[MT][KB][4];
    float nq[MT][2], tq[MT][2];
    unsigned long long* bq[MT][2];
    int* cq[MT][2];
#pragma unroll
    for (int mt = 0; mt < MT; ++mt) {
        const int64_t ra = q0 + 16 * mt + g, rb = ra + 8;
#pragma unroll
        for (int kb = 0; kb < KB; ++kb) {
            const int c0 = kb * 16 + 2 * t;
            a[mt][kb][0] = ra < n ? *reinterpret_cast<const uint32_t*>(A + ra * KW + c0) : 0u;
            a[mt][kb][1] = rb < n ? *reinterpret_cast<const uint32_t*>(A + rb * KW + c0) : 0u;
            a[mt][kb][2] = ra < n ? *reinterpret_cast<const uint32_t*>(A + ra * KW + c0 + 8) : 0u;
            a[mt][kb][3] = rb < n ? *reinterpret_cast<const uint32_t*>(A + rb * KW + c0 + 8) : 0u;
        }
        nq[mt][0] = ra < n ? ny[ra] : 0.0f;
        nq[mt][1] = rb < n ? ny[rb] : 0.0f;
        tq[mt][0] = tq[mt][1] = INFINITY;
        const int r0 = warp * kWRows + 16 * mt + g;
        bq[mt][0] = bufs + r0 * cap;
        bq[mt][1] = bufs + (r0 + 8) * cap;
        cq[mt][0] = cnt + r0;
        cq[mt][1] = cnt + r0 + 8;
    }

    const int64_t nchunks = (n + kHdChunk - 1) / kHdChunk;
    constexpr int kSeg = KW * 2 / 16;  // 16-byte segments per point row
    auto stage = [&](int64_t chunk, int slot) {
        __nv_bfloat16* dst = Bs + slot * kHdChunk * RS;
        constexpr int kPerThr = (kHdChunk * kSeg + W * 32 - 1) / (W * 32);
#pragma unroll
        for (int i = 0; i < kPerThr; ++i) {
            const int e = threadIdx.x + i * W * 32;
            if (kHdChunk * kSeg % (W * 32) != 0 && e >= kHdChunk * kSeg) break;
            const int r = e / kSeg, sgm = e % kSeg;
            const int64_t j = chunk * kHdChunk + r;
            __nv_bfloat16* d16 = dst + r * RS + sgm * 8;
            if (j < n) {
                const unsigned sa = (unsigned)__cvta_generic_to_shared(d16);
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa),
                             "l"(B + j * KW + sgm * 8));
            } else {
                *reinterpret_cast<uint4*>(d16) = make_uint4(0u, 0u, 0u, 0u);
            }
        }
        asm volatile("cp.async.commit_group;\n" ::);
        if (threadIdx.x < kHdChunk) {
            const int64_t j = chunk * kHdChunk + threadIdx.x;
            npj[slot * kHdChunk + threadIdx.x] = j < n ? ny[j] : 0.0f;
        }
    };
    stage(0, 0);
    for (int64_t c = 0; c < nchunks; ++c) {
        const int slot = (int)(c & 1);
        asm volatile("cp.async.wait_group 0;\n" ::);
        __syncthreads();  // chunk c visible; every warp is done with chunk c - 1
        if (c + 1 < nchunks) stage(c + 1, slot ^ 1);
        const __nv_bfloat16* bs = Bs + slot * kHdChunk * RS;
        float acc[MT][8][4];
#pragma unroll
        for (int mt = 0; mt < MT; ++mt)
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
                acc[mt][nt][0] = acc[mt][nt][1] = acc[mt][nt][2] = acc[mt][nt][3] = 0.0f;
#pragma unroll
        for (int kb = 0; kb < KB; ++kb) {
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const __nv_bfloat16* row = bs + (nt * 8 + g) * RS + kb * 16 + 2 * t;
                const uint32_t b0 = *reinterpret_cast<const uint32_t*>(row);
                const uint32_t b1 = *reinterpret_cast<const uint32_t*>(row + 8);
#pragma unroll
                for (int mt = 0; mt < MT; ++mt) hd_mma(acc[mt][nt], a[mt][kb], b0, b1);
            }
        }
        // estimates below the row's current L-th value join its buffer; a row
        // whose buffer cannot take this chunk's passing estimates is first cut
        // back to its L smallest (which can only tighten its threshold)
        const int64_t jb = c * kHdChunk;
        const bool whole = jb + kHdChunk <= n;
        int pc[MT][2];
#pragma unroll
        for (int mt = 0; mt < MT; ++mt) {
            pc[mt][0] = pc[mt][1] = 0;
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int col = nt * 8 + 2 * t + (e & 1);
                    const int h = e >> 1;
                    const float dd =
                        (whole || jb + col < n)
                            ? fmaxf(__fsub_rn(__fadd_rn(nq[mt][h], npj[slot * kHdChunk + col]),
                                              __fmul_rn(2.0f, acc[mt][nt][e])),
                                    0.0f)
                            : INFINITY;
                    acc[mt][nt][e] = dd;
                    pc[mt][h] += dd < tq[mt][h] ? 1 : 0;
                }
            }
        }
        unsigned rows = 0;  // bit r: warp row r must be cut before inserting
        int any = 0;
#pragma unroll
        for (int mt = 0; mt < MT; ++mt) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                int v = pc[mt][h];
                v += __shfl_xor_sync(0xffffffffu, v, 1);
                v += __shfl_xor_sync(0xffffffffu, v, 2);
                pc[mt][h] = v;
                any += v;
                // lane 4g answers for row 16 mt + 8 h + g
                const unsigned over = __ballot_sync(0xffffffffu, t == 0 && *cq[mt][h] + v > cap);
#pragma unroll
                for (int r = 0; r < 8; ++r)
                    rows |= ((over >> (4 * r)) & 1u) << (16 * mt + 8 * h + r);
            }
        }
        if (rows) {
            while (rows) {
                const int r = __ffs(rows) - 1;
                rows &= rows - 1u;
                const int qr = warp * kWRows + r;
                unsigned long long* b = bufs + qr * cap;
                const int kept = hd_cut(b, cnt[qr], L, lane);
                if (lane == 0) {
                    cnt[qr] = kept;
                    tau[qr] = kept >= L ? hd_dist(b[L - 1]) : INFINITY;
                }
                __syncwarp();
            }
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                tq[mt][0] = tau[warp * kWRows + 16 * mt + g];
                tq[mt][1] = tau[warp * kWRows + 16 * mt + g + 8];
            }
        }
        if (any > 0) {  // quad-uniform: the quad's rows have passing estimates
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
#pragma unroll
                for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int h = e >> 1;
                        const float dd = acc[mt][nt][e];
                        if (dd < tq[mt][h]) {
                            const int p = atomicAdd(cq[mt][h], 1);
                            bq[mt][h][p] = hd_key(dd, (int32_t)(jb + nt * 8 + 2 * t + (e & 1)));
                        }
                    }
                }
            }
        }
        __syncwarp();
    }
    // final cut: the L smallest estimates of every row, and the L-th estimate
    for (int r = 0; r < kWRows; ++r) {
        const int qr = warp * kWRows + r;
        const int64_t q = q0 + r;
        unsigned long long* b = bufs + qr * cap;
        const int kept = hd_cut(b, cnt[qr], L, lane);
        if (q < n) {
            for (int e = lane; e < L; e += 32)
                cand[q * L + e] = e < kept ? (int32_t)(uint32_t)b[e] : -1;
            if (lane == 0) T[q] = kept >= L ? hd_dist(b[L - 1]) : INFINITY;
        }
        __syncwarp();
    }
}

// Exact float32 squared distance in dimension order (each difference, square
// and sum rounded), from shared-memory query coordinates.
__device__ __forceinline__ float hd_rdist(const float* __restrict__ q,
                                          const float* __restrict__ x, int d) {
    float r = 0.0f;
    for (int k = 0; k < d; ++k) {
        const float df = __fsub_rn(q[k], x[k]);
        r = __fadd_rn(r, __fmul_rn(df, df));
    }
    return r;
}

// ------------------------------------------------- tcgen05 candidate GEMM
// The same candidates as hd_cand_kernel, from a Blackwell pipeline: a CTA of
// 128 queries holds their operand rows in shared memory (one TMA load), and
// every point tile of 128 rows streams through a two-stage ring of shared
// memory by TMA (cp.async.bulk.tensor, 128-byte swizzle); one thread issues
// the 128 x 128 x 16 bf16 tcgen05.mma steps into a float32 accumulator in
// tensor memory (two accumulators, so the next tile's products accumulate
// while the last one is read); four warps read the accumulator rows
// (tcgen05.ld, lane = query) and run the selection of hd_cand_kernel on them.
//   warp 0  TMA producer        warp 1  MMA issuer (allocates TMEM)
//   warps 4-7  epilogue: query row = 32 (warp - 4) + lane, the TMEM lane
// Operand rows are padded to a multiple of 64 bf16 (KA atoms of 128 bytes).
// The points' |y|^2 travel in their own four-slot ring, released by the
// epilogue (the operand ring is released by the MMA, which runs ahead).
constexpr int kTcBM = 128;       // queries per CTA (TMEM lanes)
constexpr int kTcBN = 128;       // points per tile (accumulator columns)
constexpr int kTcStages = 2;     // operand ring (gated by the MMA)
constexpr int kTcNyStages = 4;   // |y|^2 ring (gated by the epilogue, which trails the MMA by
                                 // at most two tiles: it never holds the producer back)
constexpr int kTcSub = 8;        // estimates inserted between buffer checks
constexpr int kTcStatic = 1024;  // room for the kernel's static shared memory (barriers)
constexpr int kTcThreads = 256;
constexpr int kTcTmemCols = 2 * kTcBN;
constexpr int kTcAtom = 128;     // bytes per swizzled operand row segment (64 bf16)

__host__ __device__ constexpr int tc_cap(int L) { return (L + kTcSub + 7) / 8 * 8; }
__host__ __device__ constexpr size_t tc_smem(int ka, int L) {
    return (size_t)ka * kTcBM * kTcAtom                       // A
           + (size_t)kTcStages * ka * kTcBN * kTcAtom         // B ring
           + (size_t)kTcNyStages * kTcBN * sizeof(float)      // |y|^2 of the ring's points
           + (size_t)kTcBM * tc_cap(L) * sizeof(unsigned long long)  // candidate buffers
           + 1024;                                            // 1024-byte alignment slack
}

// Sort keys of the points by |y|^2 (non-negative: its float bits order it).
__global__ void hd_norm_keys_kernel(int64_t n, const float* __restrict__ ny,
                                    uint32_t* __restrict__ key, int32_t* __restrict__ perm) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    key[i] = __float_as_uint(ny[i]);
    perm[i] = (int32_t)i;
}

// The nearest of `marks` landmarks (points 0, stride, 2 stride, ...) of every
// point, in float32 (first landmark wins ties), with perm = identity.
constexpr int kLandmarks = 256;
__global__ void __launch_bounds__(256) hd_landmark_kernel(int64_t n, int d,
                                                          const float* __restrict__ X, int marks,
                                                          int64_t stride, uint32_t* __restrict__ key,
                                                          int32_t* __restrict__ perm) {
    __shared__ float lm[32][kHighdMaxDim];
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float best = INFINITY;
    int bi = 0;
    for (int c0 = 0; c0 < marks; c0 += 32) {
        __syncthreads();
        for (int t = threadIdx.x; t < 32 * d; t += blockDim.x) {
            const int l = t / d, j = t - (t / d) * d;
            lm[l][j] = c0 + l < marks ? X[(int64_t)(c0 + l) * stride * d + j] : 0.0f;
        }
        __syncthreads();
        if (p < n) {
            float acc[32];
#pragma unroll
            for (int l = 0; l < 32; ++l) acc[l] = 0.0f;
            for (int j = 0; j < d; ++j) {
                const float x = X[p * d + j];
#pragma unroll
                for (int l = 0; l < 32; ++l) {
                    const float t = x - lm[l][j];
                    acc[l] = fmaf(t, t, acc[l]);
                }
            }
#pragma unroll
            for (int l = 0; l < 32; ++l)
                if (c0 + l < marks && acc[l] < best) {
                    best = acc[l];
                    bi = c0 + l;
                }
        }
    }
    if (p < n) {
        key[p] = (uint32_t)bi;
        perm[p] = (int32_t)p;
    }
}

// Row r of Bp (vw 16-byte vectors) and nyp[r] from point perm[r].
__global__ void hd_permute_kernel(int64_t n, int vw, const int32_t* __restrict__ perm,
                                  const uint4* __restrict__ B, const float* __restrict__ ny,
                                  uint4* __restrict__ Bp, float* __restrict__ nyp) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * vw) return;
    const int64_t r = t / vw;
    const int c = (int)(t - r * vw);
    const int64_t j = perm[r];
    Bp[t] = B[j * vw + c];
    if (c == 0) nyp[r] = ny[j];
}

// hd_cut for buffers of up to 32 * PER entries (kept out of line: the
// epilogue calls it rarely, from several places).
template <int PER>
__device__ __noinline__ int tc_cut(unsigned long long* buf, int cnt, int keep, int lane) {
    unsigned long long mine[PER];
    int rank[PER];
#pragma unroll
    for (int m = 0; m < PER; ++m) {
        const int e = lane + 32 * m;
        mine[m] = e < cnt ? buf[e] : ~0ull;
        rank[m] = 0;
    }
    for (int e = 0; e < cnt; ++e) {
        const unsigned long long o = buf[e];
#pragma unroll
        for (int m = 0; m < PER; ++m) rank[m] += o < mine[m] ? 1 : 0;
    }
    __syncwarp();
#pragma unroll
    for (int m = 0; m < PER; ++m)
        if (lane + 32 * m < cnt && rank[m] < keep) buf[rank[m]] = mine[m];
    __syncwarp();
    return cnt < keep ? cnt : keep;
}

template <int KA, int PER>
__global__ void __launch_bounds__(kTcThreads, 1) hd_cand_tc_kernel(
    const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
    int64_t n, int L, int cap, const float* __restrict__ ny, const float* __restrict__ nyq,
    const int32_t* __restrict__ perm, const int32_t* __restrict__ qperm,
    int32_t* __restrict__ cand, float* __restrict__ T, int* __restrict__ err) {
    constexpr int kABytes = KA * kTcBM * kTcAtom;
    constexpr int kBBytes = KA * kTcBN * kTcAtom;  // one stage
    constexpr uint32_t kIdesc = tc::idesc_bf16_f32(kTcBM, kTcBN);
    extern __shared__ unsigned char tc_smem_raw[];
    // full: a stage's operand rows and |y|^2 landed; empty: the MMA read the
    // stage's rows; nempty: the epilogue read a slot's |y|^2; tfull /
    // tempty: an accumulator was written / read
    __shared__ __align__(8) uint64_t full[kTcStages], empty[kTcStages], nempty[kTcNyStages],
        tfull[2], tempty[2], afull, done;
    __shared__ uint32_t tmem_slot;
    unsigned char* base = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~(uintptr_t)1023);
    unsigned char* As = base;
    unsigned char* Bs = As + kABytes;
    float* nys = reinterpret_cast<float*>(Bs + kTcStages * kBBytes);
    unsigned long long* bufs = reinterpret_cast<unsigned long long*>(nys + kTcNyStages * kTcBN);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t q0 = (int64_t)blockIdx.x * kTcBM;
    const int64_t ntiles = (n + kTcBN - 1) / kTcBN;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int u = 0; u < kTcNyStages; ++u) tc::mbar_init(&nempty[u], 4 * 32);
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&tfull[b], 1);
            tc::mbar_init(&tempty[b], 4 * 32);
        }
        tc::mbar_init(&afull, 1);
        tc::mbar_init(&done, 1);
        tc::fence_mbar_init();
    }
    if (warp == 1) {
        tc::tmem_alloc(&tmem_slot, kTcTmemCols);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        // ------------------------------------------------------ TMA producer
        if (tc::elect_one()) {
            tc::prefetch_tmap(&mapA);
            tc::prefetch_tmap(&mapB);
            tc::mbar_arrive_expect_tx(&afull, kABytes);
            for (int a = 0; a < KA; ++a)
                tc::tma_load_2d(As + a * kTcBM * kTcAtom, &mapA, a * 64, (int32_t)q0, &afull);
            int64_t issued = 0;
            for (int64_t t = 0; t < ntiles; ++t) {
                const int s = (int)(t % kTcStages);
                const int u = (int)(t % kTcNyStages);
                const uint32_t ph = (uint32_t)((t / kTcStages) & 1);
                // the operand stage is free once the MMA has read tile
                // t - kTcStages; the |y|^2 slot once the epilogue has read
                // tile t - kTcNyStages
                if (!tc::mbar_wait(&empty[s], ph ^ 1u, err, 1)) break;
                if (!tc::mbar_wait(&nempty[u], (uint32_t)(((t / kTcNyStages) & 1) ^ 1), err, 7))
                    break;
                tc::mbar_arrive_expect_tx(&full[s], kBBytes + kTcBN * (uint32_t)sizeof(float));
                unsigned char* dst = Bs + s * kBBytes;
                for (int a = 0; a < KA; ++a)
                    tc::tma_load_2d(dst + a * kTcBN * kTcAtom, &mapB, a * 64,
                                    (int32_t)(t * kTcBN), &full[s]);
                // |y|^2 of the tile's points (ny is padded to whole tiles)
                tc::bulk_load(nys + u * kTcBN, ny + t * kTcBN, kTcBN * (uint32_t)sizeof(float),
                              &full[s]);
                issued = t + 1;
            }
            // no copy may still be in flight when the block exits
            for (int64_t t = issued > kTcStages ? issued - kTcStages : 0; t < issued; ++t)
                tc::mbar_drain(&full[t % kTcStages], (uint32_t)((t / kTcStages) & 1));
            tc::mbar_drain(&afull, 0);
        }
    } else if (warp == 1) {
        // ------------------------------------------------------- MMA issuer
        if (tc::elect_one()) {
            if (tc::mbar_wait(&afull, 0, err, 2)) {
                for (int64_t t = 0; t < ntiles; ++t) {
                    const int s = (int)(t % kTcStages);
                    const int b = (int)(t & 1);
                    if (!tc::mbar_wait(&full[s], (uint32_t)((t / kTcStages) & 1), err, 3)) break;
                    if (!tc::mbar_wait(&tempty[b], (uint32_t)(((t >> 1) & 1) ^ 1), err, 4)) break;
                    tc::tc_fence_after();
                    const uint32_t d = tmem + (uint32_t)(b * kTcBN);
                    const uint32_t a0 = tc::smem_u32(As), b0 = tc::smem_u32(Bs + s * kBBytes);
#pragma unroll
                    for (int a = 0; a < KA; ++a)
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk)
                            tc::mma_bf16(d,
                                         tc::smem_desc_sw128(a0 + a * kTcBM * kTcAtom + kk * 32),
                                         tc::smem_desc_sw128(b0 + a * kTcBN * kTcAtom + kk * 32),
                                         kIdesc, (a | kk) != 0);
                    tc::mma_commit(&empty[s]);
                    tc::mma_commit(&tfull[b]);
                }
            }
            // every issued product has landed before the accumulators are freed
            tc::mma_commit(&done);
            tc::mbar_drain(&done, 0);
        }
    } else if (warp >= 4) {
        // -------------------------------------------------------- epilogue
        const int quarter = warp & 3;
        const int r = quarter * 32 + lane;
        const int64_t q = q0 + r;
        const float nq = q < n ? nyq[q] : 0.0f;
        unsigned long long* row = bufs + (size_t)r * cap;
        float tq = INFINITY;
        int cnt = 0;
        const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
        for (int64_t t = 0; t < ntiles; ++t) {
            const int b = (int)(t & 1);
            if (!tc::mbar_wait(&tfull[b], (uint32_t)((t >> 1) & 1), err, 6)) break;
            tc::tc_fence_after();
            const int u = (int)(t % kTcNyStages);
            const float* hy = nys + u * kTcBN;
            const int64_t jb = t * kTcBN;
            // 32 accumulator columns at a time; the accumulator is handed back
            // to the MMA as soon as its last columns are in registers
#pragma unroll 1
            for (int c = 0; c < kTcBN / 32; ++c) {
                uint32_t acc[32];
                tc::tmem_ld32(tmem + lane_base + (uint32_t)(b * kTcBN + c * 32), acc);
                tc::tmem_wait_ld();
                if (c == kTcBN / 32 - 1) {
                    tc::tc_fence_before();
                    tc::mbar_arrive(&tempty[b]);
                }
                // estimates of 32 columns, 8 between buffer checks; only the
                // last tile has columns past the points
                auto columns = [&](auto whole_tag) {
                    constexpr bool whole = decltype(whole_tag)::value;
                    const float* h = hy + c * 32;
                    const int64_t j0 = jb + c * 32;
#pragma unroll
                    for (int sub = 0; sub < 32 / kTcSub; ++sub) {
                        float e[kTcSub];
                        int pass = 0;
#pragma unroll
                        for (int i = 0; i < kTcSub; ++i) {
                            const int col = sub * kTcSub + i;
                            const float dot = __uint_as_float(acc[col]);
                            e[i] = fmaxf(__fsub_rn(__fadd_rn(nq, h[col]), __fmul_rn(2.0f, dot)),
                                         0.0f);
                            if (!whole && j0 + col >= n) e[i] = INFINITY;
                            pass += e[i] < tq ? 1 : 0;
                        }
                        // a row whose buffer cannot take these is first cut
                        // back to its L smallest (which only tightens its
                        // threshold)
                        unsigned rows = __ballot_sync(0xffffffffu, cnt + pass > cap);
                        if (rows) {
                            __syncwarp();  // every lane's buffer writes visible to the warp
                            do {
                                const int rr = __ffs(rows) - 1;
                                rows &= rows - 1u;
                                const int cc = __shfl_sync(0xffffffffu, cnt, rr);
                                unsigned long long* rb = bufs + (size_t)(quarter * 32 + rr) * cap;
                                const int kept = tc_cut<PER>(rb, cc, L, lane);
                                if (lane == rr) {
                                    cnt = kept;
                                    tq = kept >= L ? hd_dist(rb[L - 1]) : INFINITY;
                                }
                            } while (rows);
                        }
                        if (pass) {
#pragma unroll
                            for (int i = 0; i < kTcSub; ++i)
                                if (e[i] < tq)
                                    row[cnt++] = hd_key(e[i], (int32_t)(j0 + sub * kTcSub + i));
                        }
                    }
                };
                if (jb + kTcBN <= n) {
                    // the points run in increasing |y|^2, so h[c * 32] is the
                    // least of the chunk and, rounding being monotone, no
                    // estimate of the chunk is below
                    // fl(fl(nq + h[c * 32]) - 2 max dot): a chunk whose bound
                    // reaches every row's threshold holds no candidate
                    float dmax = __uint_as_float(acc[0]);
#pragma unroll
                    for (int i = 1; i < 32; ++i) dmax = fmaxf(dmax, __uint_as_float(acc[i]));
                    const float lb =
                        __fsub_rn(__fadd_rn(nq, hy[c * 32]), __fmul_rn(2.0f, dmax));
                    if (__any_sync(0xffffffffu, lb < tq)) columns(std::true_type{});
                } else {
                    columns(std::false_type{});
                }
            }
            tc::mbar_arrive(&nempty[u]);  // this tile's |y|^2 are read
        }
        // the L smallest estimates of every row, and its L-th estimate
        __syncwarp();
        for (int rr = 0; rr < 32; ++rr) {
            const int cc = __shfl_sync(0xffffffffu, cnt, rr);
            unsigned long long* rb = bufs + (size_t)(quarter * 32 + rr) * cap;
            const int kept = tc_cut<PER>(rb, cc, L, lane);
            const int64_t qr = q0 + quarter * 32 + rr;
            if (qr < n) {
                const int64_t qq = qperm[qr];
                for (int e2 = lane; e2 < L; e2 += 32)
                    cand[qq * L + e2] = e2 < kept ? perm[(uint32_t)rb[e2]] : -1;
                if (lane == 0) T[qq] = kept >= L ? hd_dist(rb[L - 1]) : INFINITY;
            }
            __syncwarp();
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 1) tc::tmem_dealloc(tmem, kTcTmemCols);
}

// Re-rank: a warp per query.  Writes the certified queries' k nearest (rows
// of k, (distance, index) order) and lists the others.
__global__ void __launch_bounds__(128) hd_rerank_kernel(
    int64_t n, int d, int dp, int k, int L, const float* __restrict__ X,
    const int32_t* __restrict__ cand, const float* __restrict__ T, const float* __restrict__ ny,
    const float* __restrict__ cn, const unsigned* __restrict__ maxes, float* __restrict__ rd_o,
    int32_t* __restrict__ ix_o, int32_t* __restrict__ fail_list,
    unsigned long long* __restrict__ fail_count) {
    __shared__ float qs[4][96];
    __shared__ unsigned long long keys[4][kHdMaxL];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t q = (int64_t)blockIdx.x * 4 + warp;
    if (q >= n) return;
    for (int e = lane; e < d; e += 32) qs[warp][e] = X[q * d + e];
    __syncwarp();
    int cntc = 0;
    for (int e = lane; e < L; e += 32) {
        const int32_t j = cand[q * L + e];
        keys[warp][e] = j >= 0 ? hd_key(hd_rdist(qs[warp], X + (int64_t)j * d, d), j) : ~0ull;
    }
    __syncwarp();
    for (int e = 0; e < L; ++e) cntc += keys[warp][e] != ~0ull ? 1 : 0;
    // ranks of this lane's keys among the L
    constexpr int kPer = kHdMaxL / 32;
    unsigned long long mine[kPer];
    int rank[kPer];
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
        const int e = lane + 32 * m;
        mine[m] = e < L ? keys[warp][e] : ~0ull;
        rank[m] = 0;
    }
    for (int e = 0; e < L; ++e) {
        const unsigned long long o = keys[warp][e];
#pragma unroll
        for (int m = 0; m < kPer; ++m) rank[m] += o < mine[m] ? 1 : 0;
    }
    __syncwarp();
#pragma unroll
    for (int m = 0; m < kPer; ++m)
        if (lane + 32 * m < L && rank[m] < L) keys[warp][rank[m]] = mine[m];
    __syncwarp();
    // certificate
    const float Tq = T[q];
    bool ok = true;
    if (cntc < k) {
        ok = !(Tq < INFINITY);  // fewer than k points exist only when every point is a candidate
    } else if (Tq < INFINITY) {
        const float dk = hd_dist(keys[warp][k - 1]);
        const float ymax = __uint_as_float(maxes[0]), cmax = __uint_as_float(maxes[1]);
        const float yq = sqrtf(ny[q]), cq = cn[q];
        const float kw = 3.0f * (float)dp;
        const float eta = (2.0f * kw + 4.0f * (float)dp + 16.0f) * 5.9604645e-8f *
                              (yq + ymax) * (yq + ymax) * 1.0001f +
                          3.0517578e-5f * cq * cmax * 1.0001f;
        const float a2 = Tq - eta;
        if (!(a2 > 0.0f)) {
            ok = false;
        } else {
            const float aa = sqrtf(a2) * (1.0f - 9.5367432e-7f);
            const float E = (1.5258789e-5f + 1.1920929e-7f) * (cq + cmax) * 1.0001f;
            const float lb = aa - E;
            ok = lb > 0.0f && lb * lb * (1.0f - (float)(d + 8) * 1.1920929e-7f) > dk;
        }
    }
    if (!ok) {
        if (lane == 0) {
            const unsigned long long p = atomicAdd(fail_count, 1ull);
            fail_list[p] = (int32_t)q;
        }
        return;
    }
    for (int e = lane; e < k; e += 32) {
        const unsigned long long key = keys[warp][e];
        const bool have = e < cntc;
        rd_o[q * k + e] = have ? hd_dist(key) : INFINITY;
        ix_o[q * k + e] = have ? (int32_t)(uint32_t)key : -1;
    }
}

// Fallback: a warp per listed query scans every point in exact float32.
__global__ void __launch_bounds__(128) hd_exact_kernel(
    int64_t n, int d, int k, const float* __restrict__ X, const int32_t* __restrict__ list,
    const unsigned long long* __restrict__ count, float* __restrict__ rd_o,
    int32_t* __restrict__ ix_o) {
    __shared__ float qs[4][96];
    __shared__ unsigned long long bufs[4][kHdCap];
    __shared__ int cnts[4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t total = (int64_t)*count;
    for (int64_t w = (int64_t)blockIdx.x * 4 + warp; w < total; w += (int64_t)gridDim.x * 4) {
        const int64_t q = list[w];
        for (int e = lane; e < d; e += 32) qs[warp][e] = X[q * d + e];
        if (lane == 0) cnts[warp] = 0;
        __syncwarp();
        unsigned long long* buf = bufs[warp];
        float tau = INFINITY;
        for (int64_t j0 = 0; j0 < n; j0 += 32) {
            const int64_t j = j0 + lane;
            if (j < n) {
                const float r = hd_rdist(qs[warp], X + j * d, d);
                if (r <= tau) {
                    const int p = atomicAdd(&cnts[warp], 1);
                    buf[p] = hd_key(r, (int32_t)j);
                }
            }
            __syncwarp();
            const int c = cnts[warp];
            if (c > kHdCap - 32) {
                const int kept = hd_cut(buf, c, k, lane);
                tau = kept >= k ? hd_dist(buf[k - 1]) : INFINITY;
                __syncwarp();
                if (lane == 0) cnts[warp] = kept;
            }
            __syncwarp();
        }
        const int kept = hd_cut(buf, cnts[warp], k, lane);
        for (int e = lane; e < k; e += 32) {
            const bool have = e < kept;
            rd_o[q * k + e] = have ? hd_dist(buf[e]) : INFINITY;
            ix_o[q * k + e] = have ? (int32_t)(uint32_t)buf[e] : -1;
        }
        __syncwarp();
    }
}

size_t cand_smem(int kb, int queries, int cap) {
    const int rs = kb * 16 + 8;
    return (size_t)2 * kHdChunk * rs * sizeof(__nv_bfloat16) +
           (size_t)queries * cap * sizeof(unsigned long long) + 2 * kHdChunk * sizeof(float) +
           queries * (sizeof(int) + sizeof(float));
}

template <int KB, int W, int MT>
int launch_cand_w(int64_t n, int L, int cap, const __nv_bfloat16* A, const __nv_bfloat16* B,
                  const float* ny, int32_t* cand, float* T, cudaStream_t s) {
    constexpr int Q = W * kHdRows * MT;
    const size_t smem = cand_smem(KB, Q, cap);
    FHG_CUDA(cudaFuncSetAttribute(hd_cand_kernel<KB, W, MT>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t blocks = (n + Q - 1) / Q;
    Stage stage(s, "hd_cand_kernel");
    ::fhg::note_launch();
    hd_cand_kernel<KB, W, MT><<<(unsigned)blocks, W * 32, smem, s>>>(n, L, cap, A, B, ny, cand,
                                                                       T);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

// 128 queries share every staged chunk when their buffers fit in shared
// memory (64 otherwise), as 8 (4) warps of one m-tile: two m-tiles per warp
// (each B fragment feeding two tensor-core ops, half the warps) measured
// slower at 1M x 64-D (2.34 s against 1.92 s per kNN).
template <int KB>
int launch_cand(int64_t n, int L, const __nv_bfloat16* A, const __nv_bfloat16* B,
                const float* ny, int32_t* cand, float* T, cudaStream_t s) {
    const int cap = std::min(kHdCap, (L + kHdChunk + 31) / 32 * 32);
    if (cand_smem(KB, 128, cap) <= (size_t)kHdSmemMax)
        return launch_cand_w<KB, 8, 1>(n, L, cap, A, B, ny, cand, T, s);
    return launch_cand_w<KB, 4, 1>(n, L, cap, A, B, ny, cand, T, s);
}

// cuTensorMapEncodeTiled from the driver, without linking libcuda.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
int tensor_map_rows(CUtensorMap* map, const __nv_bfloat16* base, int64_t rows, int kw,
                    int box_rows) {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        FHG_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                  cudaEnableDefault, &q));
        if (!p || q != cudaDriverEntryPointSuccess) {
            set_error("cuTensorMapEncodeTiled is not available from the driver");
            return FHG_ERR_CUDA;
        }
        fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    const cuuint64_t gdim[2] = {(cuuint64_t)kw, (cuuint64_t)rows};
    const cuuint64_t gstride[1] = {(cuuint64_t)kw * sizeof(__nv_bfloat16)};
    const cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
    const cuuint32_t estride[2] = {1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                          const_cast<__nv_bfloat16*>(base), gdim, gstride, box, estride,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return FHG_ERR_CUDA;
    }
    return FHG_OK;
}

template <int KA, int PER>
int launch_cand_tc(int64_t n, int L, const __nv_bfloat16* A, const __nv_bfloat16* B,
                   const float* ny_padded, const float* nyq, const int32_t* perm,
                   const int32_t* qperm, int32_t* cand, float* T, int* err, cudaStream_t s) {
    CUtensorMap ma, mb;
    FHG_TRY(tensor_map_rows(&ma, A, n, KA * 64, kTcBM));
    FHG_TRY(tensor_map_rows(&mb, B, n, KA * 64, kTcBN));
    const size_t smem = tc_smem(KA, L);
    FHG_CUDA(cudaFuncSetAttribute(hd_cand_tc_kernel<KA, PER>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t blocks = (n + kTcBM - 1) / kTcBM;
    Stage stage(s, "hd_cand_kernel");
    ::fhg::note_launch();
    hd_cand_tc_kernel<KA, PER><<<(unsigned)blocks, kTcThreads, smem, s>>>(
        ma, mb, n, L, tc_cap(L), ny_padded, nyq, perm, qperm, cand, T, err);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

// The tensor-core pipeline's operand atoms for (dp, L), or 0 when the
// mma.sync kernel must run (rows of 96 dimensions, or buffers too large for
// shared memory).
int tc_atoms(int dp, int L) {
    const int ka = dp == 32 ? 2 : (dp == 64 ? 3 : 0);
    if (ka == 0 || tc_cap(L) > 32 * 4 || tc_smem(ka, L) + kTcStatic > (size_t)kHdSmemMax)
        return 0;
    return ka;
}

int launch_cand_tc_any(int ka, int64_t n, int L, const __nv_bfloat16* A, const __nv_bfloat16* B,
                       const float* ny_padded, const float* nyq, const int32_t* perm,
                       const int32_t* qperm, int32_t* cand, float* T, int* err,
                       cudaStream_t s) {
    const int per = (tc_cap(L) + 31) / 32;
#define FHG_TC(KA, PER)                                                                     \
    if (ka == KA && per == PER)                                                             \
        return launch_cand_tc<KA, PER>(n, L, A, B, ny_padded, nyq, perm, qperm, cand, T, err, \
                                       s);
    FHG_TC(2, 1) FHG_TC(2, 2) FHG_TC(2, 3) FHG_TC(2, 4)
    FHG_TC(3, 1) FHG_TC(3, 2) FHG_TC(3, 3) FHG_TC(3, 4)
#undef FHG_TC
    set_error("tensor-core kNN: no pipeline for %d atoms, %d-entry buffers", ka, tc_cap(L));
    return FHG_ERR_UNSUPPORTED;
}

}  // namespace

// Which candidate kernel the calling thread's high-dimensional kNN uses: the
// tcgen05 pipeline (default) or the mma.sync kernel.
static thread_local int t_hd_legacy = 0;
int highd_use_legacy(int on) {
    const int old = t_hd_legacy;
    t_hd_legacy = on;
    return old;
}

int highd_knn(const float* X, int64_t n, int d, int k, float* rd_o, int32_t* ix_o,
              int64_t* fallbacks, cudaStream_t s) {
    if (d < 1 || d > kHighdMaxDim) {
        set_error("high-dimensional kNN: d must be in [1, %d] (got %d)", kHighdMaxDim, d);
        return d < 1 ? FHG_ERR_INVALID : FHG_ERR_UNSUPPORTED;
    }
    if (k < 1 || k + 32 > kHdMaxL) {
        set_error("high-dimensional kNN: k must be in [1, %d] (got %d)", kHdMaxL - 32, k);
        return FHG_ERR_INVALID;
    }
    if (n > 0x7fffffffLL) {
        set_error("high-dimensional kNN: more than 2^31 - 1 points");
        return FHG_ERR_UNSUPPORTED;
    }
    if (fallbacks) *fallbacks = 0;
    if (n <= 0) return FHG_OK;
    Stage stage(s, "highd_knn");
    const int dp = d <= 32 ? 32 : (d <= 64 ? 64 : 96);
    const int L = k + 32;
    const int ka = t_hd_legacy ? 0 : tc_atoms(dp, L);
    const int kw = ka ? 64 * ka : 3 * dp;
    const int64_t n_pad = (n + kTcBN - 1) / kTcBN * kTcBN;
    Workspace ws(s);
    float *mu, *ny, *cn, *T;
    unsigned* maxes;
    __nv_bfloat16 *A, *B;
    int32_t *cand, *flist;
    unsigned long long* fcount;
    FHG_TRY(ws.alloc(&mu, (size_t)d));
    FHG_TRY(ws.alloc(&ny, (size_t)n_pad));  // whole point tiles for the bulk copies
    FHG_TRY(ws.alloc(&cn, (size_t)n));
    FHG_TRY(ws.alloc(&T, (size_t)n));
    FHG_TRY(ws.alloc(&maxes, 2));
    FHG_TRY(ws.alloc(&A, (size_t)(n * kw)));
    FHG_TRY(ws.alloc(&B, (size_t)(n * kw)));
    FHG_TRY(ws.alloc(&cand, (size_t)(n * L)));
    FHG_TRY(ws.alloc(&flist, (size_t)n));
    FHG_TRY(ws.alloc(&fcount, 1));
    FHG_CUDA(cudaMemsetAsync(maxes, 0, 2 * sizeof(unsigned), s));
    FHG_CUDA(cudaMemsetAsync(fcount, 0, sizeof(unsigned long long), s));
    if (n_pad > n) FHG_CUDA(cudaMemsetAsync(ny + n, 0, sizeof(float) * (size_t)(n_pad - n), s));
    ::fhg::note_launch();
    hd_mean_kernel<<<d, 256, 0, s>>>(X, n, d, mu);
    ::fhg::note_launch();
    hd_split_kernel<<<grid_for(n, 128), 128, 0, s>>>(X, n, d, dp, kw, mu, A, B, ny, cn, maxes);
    FHG_CUDA(cudaGetLastError());
    if (ka) {
        // the points (B rows, |y|^2) in increasing |y|^2, for the chunk
        // bound of the epilogue; candidates map back through perm.  The
        // queries (A rows) grouped by their nearest landmark, so that the
        // rows of a CTA tend to need the same chunks; results go back to
        // the query's own row through qperm.
        uint32_t *nkey, *qkey;
        int32_t *perm, *qperm;
        float *nyp, *nyq;
        __nv_bfloat16 *Ap, *Bp;
        int* err;
        FHG_TRY(ws.alloc(&nkey, (size_t)n));
        FHG_TRY(ws.alloc(&qkey, (size_t)n));
        FHG_TRY(ws.alloc(&perm, (size_t)n));
        FHG_TRY(ws.alloc(&qperm, (size_t)n));
        FHG_TRY(ws.alloc(&nyp, (size_t)n_pad));
        FHG_TRY(ws.alloc(&nyq, (size_t)n));
        FHG_TRY(ws.alloc(&Ap, (size_t)(n * kw)));
        FHG_TRY(ws.alloc(&Bp, (size_t)(n * kw)));
        FHG_TRY(ws.alloc(&err, 1));
        ::fhg::note_launch();
        hd_norm_keys_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, ny, nkey, perm);
        FHG_CUDA(cudaGetLastError());
        FHG_TRY(radix_sort_u32(ws, nkey, perm, n, 0, 32));
        const int marks = (int)std::min<int64_t>(kLandmarks, n);
        ::fhg::note_launch();
        hd_landmark_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, d, X, marks, n / marks, qkey,
                                                             qperm);
        FHG_CUDA(cudaGetLastError());
        FHG_TRY(radix_sort_u32(ws, qkey, qperm, n, 0, 8));
        const int64_t vecs = n * (kw / 8);
        ::fhg::note_launch();
        hd_permute_kernel<<<grid_for(vecs, 256), 256, 0, s>>>(
            n, kw / 8, perm, reinterpret_cast<const uint4*>(B), ny,
            reinterpret_cast<uint4*>(Bp), nyp);
        ::fhg::note_launch();
        hd_permute_kernel<<<grid_for(vecs, 256), 256, 0, s>>>(
            n, kw / 8, qperm, reinterpret_cast<const uint4*>(A), ny,
            reinterpret_cast<uint4*>(Ap), nyq);
        FHG_CUDA(cudaGetLastError());
        if (n_pad > n)
            FHG_CUDA(cudaMemsetAsync(nyp + n, 0, sizeof(float) * (size_t)(n_pad - n), s));
        FHG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
        FHG_TRY(launch_cand_tc_any(ka, n, L, Ap, Bp, nyp, nyq, perm, qperm, cand, T, err, s));
        int h_err = 0;
        FHG_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
        FHG_CUDA(cudaStreamSynchronize(s));
        if (h_err) {
            set_error("tensor-core kNN pipeline: a wait ran out (stage %d)", h_err);
            return FHG_ERR_CUDA;
        }
    } else {
        switch (dp) {
            case 32: FHG_TRY(launch_cand<6>(n, L, A, B, ny, cand, T, s)); break;
            case 64: FHG_TRY(launch_cand<12>(n, L, A, B, ny, cand, T, s)); break;
            default: FHG_TRY(launch_cand<18>(n, L, A, B, ny, cand, T, s)); break;
        }
    }
    {
        Stage st(s, "hd_rerank_kernel");
        ::fhg::note_launch();
        hd_rerank_kernel<<<(unsigned)((n + 3) / 4), 128, 0, s>>>(
            n, d, dp, k, L, X, cand, T, ny, cn, maxes, rd_o, ix_o, flist, fcount);
        FHG_CUDA(cudaGetLastError());
    }
    unsigned long long nf = 0;
    FHG_CUDA(cudaMemcpyAsync(&nf, fcount, sizeof(nf), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    if (nf > 0) {
        Stage st(s, "hd_exact_kernel");
        const int64_t blocks = std::min<int64_t>(((int64_t)nf + 3) / 4, 152 * 16);
        ::fhg::note_launch();
        hd_exact_kernel<<<(unsigned)blocks, 128, 0, s>>>(n, d, k, X, flist, fcount, rd_o, ix_o);
        FHG_CUDA(cudaGetLastError());
    }
    if (fallbacks) *fallbacks = (int64_t)nf;
    return FHG_OK;
}

}  // namespace fhg
