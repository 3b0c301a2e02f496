// Exclusive scan and LSD radix sort (8-bit digits, stable) for sm_103a.
//
// Radix pass = histogram kernel (one 4096-item tile per block, shared-memory
// counters) + exclusive scan of the digit-major [256][tiles] count table +
// scatter kernel.  The scatter keeps LSD stability by letting each warp rank
// its 512 items in order (warp match on the digit, per-warp running counters)
// and adding the per-warp prefix of each digit.
#include <algorithm>

#include "primitives.cuh"

namespace fhg {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanIPT = 4;
constexpr int kScanTile = kScanThreads * kScanIPT;

template <class T>
__device__ T block_exclusive_scan(T v, T* total) {
    __shared__ T warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        T w = lane < nw ? warp_sums[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(kFull, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) warp_sums[lane] = w;  // inclusive
    }
    __syncthreads();
    T warp_prefix = warp == 0 ? T(0) : warp_sums[warp - 1];
    if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
    T res = warp_prefix + x - v;
    __syncthreads();
    return res;
}

template <class T>
__global__ void __launch_bounds__(kScanThreads) scan_tile_kernel(const T* in, T* out,
                                                                 T* tile_sums, int64_t n) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanIPT;
    T v[kScanIPT];
    T s = 0;
#pragma unroll
    for (int i = 0; i < kScanIPT; ++i) {
        v[i] = (base + i < n) ? in[base + i] : T(0);
        s += v[i];
    }
    __shared__ T tot;
    T run = block_exclusive_scan<T>(s, threadIdx.x == 0 ? &tot : nullptr);
#pragma unroll
    for (int i = 0; i < kScanIPT; ++i) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
    __syncthreads();
    if (threadIdx.x == 0 && tile_sums) tile_sums[blockIdx.x] = tot;
}

template <class T>
__global__ void scan_add_kernel(T* out, const T* tile_offsets, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_offsets[i / kScanTile];
}

template <class T>
int scan_exclusive(Workspace& ws, const T* in, T* out, int64_t n, T* total) {
    cudaStream_t s = ws.stream();
    if (n <= 0) {
        if (total) FHG_CUDA(cudaMemsetAsync(total, 0, sizeof(T), s));
        return FHG_OK;
    }
    int64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 1) {
        ::fhg::note_launch();
        scan_tile_kernel<T><<<1, kScanThreads, 0, s>>>(in, out, total, n);
        FHG_CUDA(cudaGetLastError());
        return FHG_OK;
    }
    T* sums;
    FHG_TRY(ws.alloc(&sums, (size_t)tiles));
    ::fhg::note_launch();
    scan_tile_kernel<T><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, sums, n);
    FHG_CUDA(cudaGetLastError());
    FHG_TRY(scan_exclusive<T>(ws, sums, sums, tiles, total));
    ::fhg::note_launch();
    scan_add_kernel<T><<<grid_for(n, 256), 256, 0, s>>>(out, sums, n);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

// ---------------------------------------------------------------- radix sort
constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsChunks = 8;                        // 32-item chunks per warp
constexpr int kRsTile = kRsWarps * kRsChunks * 32;  // 2048 items per block

template <class K>
__global__ void __launch_bounds__(kRsThreads) rs_hist_kernel(const K* __restrict__ keys,
                                                             int64_t n, int shift,
                                                             uint32_t* __restrict__ hist,
                                                             int64_t tiles) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kRsTile;
    for (int i = threadIdx.x; i < kRsTile; i += kRsThreads) {
        int64_t idx = base + i;
        if (idx < n) atomicAdd(&h[(unsigned)(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one 8-bit digit.  Each warp ranks its 16 chunks of 32
// items per digit (lanes by __match_any_sync); the tile's items are then laid
// out in digit order in shared memory and written out so that consecutive
// threads store consecutive positions of one digit's run (coalesced), in the
// same stable order as a direct scatter.
template <class K>
__global__ void __launch_bounds__(kRsThreads) rs_scatter_kernel(
    const K* __restrict__ kin, const int32_t* __restrict__ vin, K* __restrict__ kout,
    int32_t* __restrict__ vout, int64_t n, int shift, const uint32_t* __restrict__ offs,
    int64_t tiles) {
    __shared__ uint32_t wcnt[kRsWarps][256];
    __shared__ uint32_t tstart[256];
    __shared__ K skey[kRsTile];
    __shared__ int32_t sval[kRsTile];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kRsWarps * 256; i += kRsThreads) (&wcnt[0][0])[i] = 0;
    __syncthreads();
    const unsigned lt_mask = (1u << lane) - 1u;
    const int64_t tile0 = (int64_t)blockIdx.x * kRsTile;
    const int64_t base = tile0 + (int64_t)w * (kRsChunks * 32);
    K key[kRsChunks];
    int32_t val[kRsChunks];
    uint32_t pos[kRsChunks];
    int dig[kRsChunks];
#pragma unroll
    for (int c = 0; c < kRsChunks; ++c) {
        int64_t idx = base + c * 32 + lane;
        bool valid = idx < n;
        K k = valid ? kin[idx] : K(0);
        int32_t v = valid ? vin[idx] : 0;
        int d = valid ? (int)((unsigned)(k >> shift) & 255u) : 256;
        unsigned peers = __match_any_sync(kFull, d);
        int r = __popc(peers & lt_mask);
        uint32_t pre = valid ? wcnt[w][d] : 0u;
        __syncwarp();
        if (valid && r == 0) wcnt[w][d] = pre + (uint32_t)__popc(peers);
        __syncwarp();
        key[c] = k;
        val[c] = v;
        pos[c] = pre + (uint32_t)r;
        dig[c] = d;
    }
    __syncthreads();
    {   // per digit: warps' offsets inside the digit, then the digit's start in the tile
        uint32_t sum = 0;
        for (int ww = 0; ww < kRsWarps; ++ww) {
            uint32_t c = wcnt[ww][threadIdx.x];
            wcnt[ww][threadIdx.x] = sum;
            sum += c;
        }
        tstart[threadIdx.x] = block_exclusive_scan<uint32_t>(sum, nullptr);
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < kRsChunks; ++c) {
        if (dig[c] < 256) {
            const uint32_t lp = tstart[dig[c]] + wcnt[w][dig[c]] + pos[c];
            skey[lp] = key[c];
            sval[lp] = val[c];
        }
    }
    __syncthreads();
    const int cnt = (int)(n - tile0 < kRsTile ? n - tile0 : kRsTile);
    for (int i = threadIdx.x; i < cnt; i += kRsThreads) {
        const K k = skey[i];
        const int d = (int)((unsigned)(k >> shift) & 255u);
        const uint32_t dst = offs[(int64_t)d * tiles + blockIdx.x] + (uint32_t)i - tstart[d];
        kout[dst] = k;
        vout[dst] = sval[i];
    }
}

// The same sort for n <= kRsTile in one launch: a bitonic sort in shared
// memory of (digits, position) pairs, where digits are the key bits the LSD
// passes cover ([begin, end) rounded up to whole 8-bit digits), so the order
// is the stable one the passes give.
constexpr int kRsSmallThreads = 1024;
template <class K>
__global__ void __launch_bounds__(kRsSmallThreads) rs_small_kernel(K* keys, int32_t* vals, int n,
                                                                   int shift, int bits) {
    __shared__ K sk[kRsTile];
    __shared__ uint16_t si[kRsTile];
    __shared__ int32_t sv[kRsTile];
    const K mask = bits >= (int)(8 * sizeof(K)) ? ~K(0) : ((K(1) << bits) - K(1));
    int m2 = 1;
    while (m2 < n) m2 <<= 1;
    for (int i = threadIdx.x; i < m2; i += blockDim.x) {
        sk[i] = i < n ? keys[i] : ~K(0);
        si[i] = i < n ? (uint16_t)i : (uint16_t)0xffffu;  // padding sorts last
        if (i < n) sv[i] = vals ? vals[i] : 0;
    }
    __syncthreads();
    for (int size = 2; size <= m2; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = threadIdx.x; i < m2; i += blockDim.x) {
                const int j = i ^ stride;
                if (j > i) {
                    const K da = (sk[i] >> shift) & mask, db = (sk[j] >> shift) & mask;
                    const bool greater = da > db || (da == db && si[i] > si[j]);
                    if (greater == ((i & size) == 0)) {
                        const K tk = sk[i];
                        sk[i] = sk[j];
                        sk[j] = tk;
                        const uint16_t ti = si[i];
                        si[i] = si[j];
                        si[j] = ti;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        keys[i] = sk[i];
        if (vals) vals[i] = sv[si[i]];
    }
}

template <class K>
int radix_sort(Workspace& ws, K* keys, int32_t* vals, int64_t n, int begin_bit, int end_bit) {
    if (n <= 1 || end_bit <= begin_bit) return FHG_OK;
    if (n >= ((int64_t)1 << 32)) {
        set_error("radix sort: n too large");
        return FHG_ERR_INVALID;
    }
    cudaStream_t s = ws.stream();
    if (n <= kRsTile) {
        const int bits = std::min(((end_bit - begin_bit + 7) / 8) * 8,
                                  (int)(8 * sizeof(K)) - begin_bit);
        ::fhg::note_launch();
        rs_small_kernel<K><<<1, kRsSmallThreads, 0, s>>>(keys, vals, (int)n, begin_bit, bits);
        FHG_CUDA(cudaGetLastError());
        return FHG_OK;
    }
    const int64_t tiles = (n + kRsTile - 1) / kRsTile;
    K* kalt;
    int32_t* valt;
    uint32_t* hist;
    FHG_TRY(ws.alloc(&kalt, (size_t)n));
    FHG_TRY(ws.alloc(&valt, (size_t)n));
    FHG_TRY(ws.alloc(&hist, (size_t)(256 * tiles)));
    K *ka = keys, *kb = kalt;
    int32_t *va = vals, *vb = valt;
    for (int shift = begin_bit; shift < end_bit; shift += 8) {
        ::fhg::note_launch();
        rs_hist_kernel<K><<<(unsigned)tiles, kRsThreads, 0, s>>>(ka, n, shift, hist, tiles);
        FHG_CUDA(cudaGetLastError());
        FHG_TRY(scan_exclusive<uint32_t>(ws, hist, hist, 256 * tiles, nullptr));
        ::fhg::note_launch();
        rs_scatter_kernel<K><<<(unsigned)tiles, kRsThreads, 0, s>>>(ka, va, kb, vb, n, shift,
                                                                   hist, tiles);
        FHG_CUDA(cudaGetLastError());
        K* tk = ka; ka = kb; kb = tk;
        int32_t* tv = va; va = vb; vb = tv;
    }
    if (ka != keys) {
        FHG_CUDA(cudaMemcpyAsync(keys, ka, sizeof(K) * n, cudaMemcpyDeviceToDevice, s));
        FHG_CUDA(cudaMemcpyAsync(vals, va, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
    }
    return FHG_OK;
}

__global__ void iota_kernel(int32_t* p, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = (int32_t)i;
}

}  // namespace

int scan_exclusive_u32(Workspace& ws, const uint32_t* in, uint32_t* out, int64_t n,
                       uint32_t* total) {
    return scan_exclusive<uint32_t>(ws, in, out, n, total);
}
int scan_exclusive_i64(Workspace& ws, const int64_t* in, int64_t* out, int64_t n,
                       int64_t* total) {
    return scan_exclusive<int64_t>(ws, in, out, n, total);
}
int scan_exclusive_f64(Workspace& ws, const double* in, double* out, int64_t n, double* total) {
    return scan_exclusive<double>(ws, in, out, n, total);
}
int radix_sort_u64(Workspace& ws, uint64_t* keys, int32_t* vals, int64_t n, int begin_bit,
                   int end_bit) {
    return radix_sort<uint64_t>(ws, keys, vals, n, begin_bit, end_bit);
}
int radix_sort_u32(Workspace& ws, uint32_t* keys, int32_t* vals, int64_t n, int begin_bit,
                   int end_bit) {
    return radix_sort<uint32_t>(ws, keys, vals, n, begin_bit, end_bit);
}
int fill_iota_i32(int32_t* p, int64_t n, cudaStream_t s) {
    if (n <= 0) return FHG_OK;
    ::fhg::note_launch();
    iota_kernel<<<grid_for(n, 256), 256, 0, s>>>(p, n);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

}  // namespace fhg
