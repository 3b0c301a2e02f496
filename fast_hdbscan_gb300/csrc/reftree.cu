// The reference's KD-tree, built exactly, on the GPU.
//
// The reference builds a median-split KD-tree (numba_kdtree.py:410-521):
// node ranges halve an index array, each internal node splits on the axis of
// largest spread (:129-158) by an introselect of its range around the
// median (:372-413: median-of-three pivot :282, a Hoare partition :316,
// insertion sort at 16 elements or fewer :186, heapsort after 2 log2(size)
// partitions :247), and leaves keep the order those partitions leave behind.
// The Boruvka search visits points in that tree's depth-first order, so
// among candidates of equal weight the reference keeps the one this order
// meets first.  The engine's own spatial index cannot reproduce that order;
// this tree can, and the reference tie mode uses it as the tie-breaker.
//
// Every step of the build is reproduced, not just its result:
//   * compare = (coordinate, index) lexicographic (:164-183), a total order;
//     it is packed as one 64-bit key (order-preserving float bits << 32 |
//     index), so one unsigned comparison decides;
//   * a Hoare partition swaps the k-th element above the pivot counted from
//     the left with the k-th element below it counted from the right, as long
//     as the first lies left of the second, and puts the pivot at
//     left + (elements below it).  That is a prefix count and a pairing, so a
//     thread block runs each partition in parallel with the same result;
//   * insertion sort and heapsort both leave their range in ascending order,
//     which under a total order is unique: a block sorts the range instead.
// One thread block per node of a level runs that node's introselect; while a
// node's active range is long (the top levels), its partition steps run on
// the whole GPU instead, every such node of the level in the same launches.
// The levels run one after another.
#include <cmath>

#include "index.cuh"
#include "primitives.cuh"
#include "reftree.cuh"

namespace fhg {
namespace {

constexpr int kSelThreads = 512;
constexpr int kSelV = 8;                          // consecutive keys per thread and tile
constexpr int kSelTile = kSelThreads * kSelV;     // keys per scan tile
constexpr int kBlockSortMax = 4096;               // ranges a block sorts in shared memory
constexpr int64_t kWideMin = 32768;               // longer ranges partition device-wide

// The saved introselect state of a node partitioned device-wide.
constexpr int kWideActive = 0, kWideBlock = 1, kWideDone = 2;
struct WideNode {
    int64_t l, r, B;
    uint64_t pivot;
    int32_t depth, state;
    uint32_t c, K;
};

#define LAUNCH(kernel, count, ...)                                                   \
    do {                                                                             \
        if ((count) > 0) {                                                           \
            ::fhg::note_launch();                                                    \
            kernel<<<grid_for((count), 256), 256, 0, s>>>(__VA_ARGS__);              \
            FHG_CUDA(cudaGetLastError());                                            \
        }                                                                            \
    } while (0)

// Order-preserving bits of a float (-0 and +0 compare equal, as in the
// reference's `<` / `>` tests).
__device__ __forceinline__ uint32_t ordered_bits(float f) {
    uint32_t u = __float_as_uint(f);
    if (u == 0x80000000u) u = 0u;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float from_ordered(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void init_root_kernel(int64_t n, int32_t* __restrict__ idx, int32_t* __restrict__ nodeof,
                                 int64_t* __restrict__ rs, int64_t* __restrict__ re) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) {
        idx[p] = (int32_t)p;
        nodeof[p] = 0;
    }
    if (p == 0) {
        rs[0] = 0;
        re[0] = n;
    }
}

// Ranges of the next level: the left child takes the first half (rounded
// down) of its parent's range (numba_kdtree.py:486-509).
__global__ void child_ranges_kernel(int64_t first, int64_t count, int64_t* rs, int64_t* re) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int64_t v = first + t;
    const int64_t s = rs[v], e = re[v], mid = s + (e - s) / 2;
    rs[2 * v + 1] = s;
    re[2 * v + 1] = mid;
    rs[2 * v + 2] = mid;
    re[2 * v + 2] = e;
}

__global__ void box_init_kernel(int64_t first, int64_t count, int d, uint32_t* __restrict__ lo,
                                uint32_t* __restrict__ hi) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count * d) return;
    const int64_t v = first + t / d;
    const int j = (int)(t % d);
    lo[v * d + j] = 0xff800000u;  // ordered bits of +inf
    hi[v * d + j] = 0x007fffffu;  // ordered bits of -inf
}

// Per node of the level: the bounding box of its points (_init_node,
// numba_kdtree.py:67).  Positions of one node are contiguous, so a warp
// reduces each run of lanes that share a node (a segmented shuffle
// reduction) and the run's first lane takes the atomics; a block whose
// threads all share one node (the top levels) combines its warps first and
// takes one atomic per dimension.  pts: the points in caller order, pad
// floats per row.
constexpr int kBoxThreads = 256;
__global__ void __launch_bounds__(kBoxThreads) box_level_kernel(
    int64_t n, int d, int pad, const int32_t* __restrict__ idx, const int32_t* __restrict__ nodeof,
    const float* __restrict__ pts, uint32_t* lo, uint32_t* hi) {
    __shared__ int32_t s_v0;
    __shared__ uint32_t s_lo[kBoxThreads / 32][32], s_hi[kBoxThreads / 32][32];
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const bool valid = p < n;
    const int32_t v = valid ? nodeof[p] : -1;
    const int64_t row = valid ? (int64_t)idx[p] * pad : 0;
    if (threadIdx.x == 0) s_v0 = v;
    __syncthreads();
    const bool block_uniform = __syncthreads_and(valid && v == s_v0);
    // lanes of the same node above this one, for each shuffle distance
    unsigned same = 0;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const int32_t other = __shfl_down_sync(kFull, v, 1 << k);
        if (lane + (1 << k) < 32 && other == v) same |= 1u << k;
    }
    const int32_t v_prev = __shfl_up_sync(kFull, v, 1);  // every lane takes part
    const bool head = valid && (lane == 0 || v_prev != v);
    for (int j = 0; j < d; ++j) {
        const uint32_t o = valid ? ordered_bits(pts[row + j]) : 0u;
        uint32_t a = valid ? o : 0xffffffffu, b = o;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const uint32_t a2 = __shfl_down_sync(kFull, a, 1 << k);
            const uint32_t b2 = __shfl_down_sync(kFull, b, 1 << k);
            if (same & (1u << k)) {
                a = min(a, a2);
                b = max(b, b2);
            }
        }
        if (block_uniform) {
            if (lane == 0) {
                s_lo[w][j] = a;
                s_hi[w][j] = b;
            }
        } else if (head) {
            atomicMin(&lo[(int64_t)v * d + j], a);
            atomicMax(&hi[(int64_t)v * d + j], b);
        }
    }
    if (block_uniform) {
        __syncthreads();
        if (threadIdx.x < d) {
            const int j = threadIdx.x;
            uint32_t a = s_lo[0][j], b = s_hi[0][j];
            for (int k = 1; k < kBoxThreads / 32; ++k) {
                a = min(a, s_lo[k][j]);
                b = max(b, s_hi[k][j]);
            }
            atomicMin(&lo[(int64_t)v * d + j], a);
            atomicMax(&hi[(int64_t)v * d + j], b);
        }
    }
}

// The split axis of every internal node of the level: the first dimension
// of largest spread hi - lo, 0 when every spread is 0 (_find_node_split_dim,
// numba_kdtree.py:129: `spread > max_spread`, max_spread starting at 0).
// Also writes the node's box as float32 (lower then upper corner).
__global__ void axis_level_kernel(int64_t first, int64_t count, int d,
                                  const uint32_t* __restrict__ lo, const uint32_t* __restrict__ hi,
                                  float* __restrict__ box, int32_t* __restrict__ axis) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int64_t v = first + t;
    float best = 0.0f;
    int32_t a = 0;
    for (int j = 0; j < d; ++j) {
        const float l = from_ordered(lo[v * d + j]), h = from_ordered(hi[v * d + j]);
        box[v * 2 * d + j] = l;
        box[v * 2 * d + d + j] = h;
        const float spread = __fsub_rn(h, l);
        if (spread > best) {
            best = spread;
            a = j;
        }
    }
    if (axis) axis[t] = a;
}

// key[p] = (ordered bits of the point's split coordinate) << 32 | index.
__global__ void keys_level_kernel(int64_t n, int64_t first, int pad,
                                  const int32_t* __restrict__ idx,
                                  const int32_t* __restrict__ nodeof,
                                  const int32_t* __restrict__ axis, const float* __restrict__ pts,
                                  uint64_t* __restrict__ keys) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int32_t c = idx[p];
    const float x = pts[(int64_t)c * pad + axis[nodeof[p] - first]];
    keys[p] = ((uint64_t)ordered_bits(x) << 32) | (uint32_t)c;
}

// The index's points (Morton order) back in caller order.
__global__ void caller_order_kernel(int64_t n, int pad, const int32_t* __restrict__ orig,
                                    const float* __restrict__ pts, float* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * pad) return;
    const int64_t r = t / pad;
    out[(int64_t)orig[r] * pad + (t - r * pad)] = pts[t];
}

__global__ void unpack_level_kernel(int64_t n, const uint64_t* __restrict__ keys,
                                    const int64_t* __restrict__ rs, const int64_t* __restrict__ re,
                                    int32_t* __restrict__ idx, int32_t* __restrict__ nodeof) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    idx[p] = (int32_t)(keys[p] & 0xffffffffu);
    const int32_t v = nodeof[p];
    const int64_t mid = rs[v] + (re[v] - rs[v]) / 2;
    nodeof[p] = 2 * v + 1 + (p >= mid ? 1 : 0);
}

__global__ void inverse_kernel(int64_t n, const int32_t* __restrict__ idx, int32_t* __restrict__ pos) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) pos[idx[p]] = (int32_t)p;
}

__device__ __forceinline__ void swap_keys(uint64_t* k, int64_t a, int64_t b) {
    const uint64_t t = k[a];
    k[a] = k[b];
    k[b] = t;
}

// Exclusive block prefix of one value per thread; returns the block total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* out, uint32_t* s_warp) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    if (w == 0) {
        uint32_t x = lane < kSelThreads / 32 ? s_warp[lane] : 0u;
        uint32_t y = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, y, o);
            if (lane >= o) y += t;
        }
        if (lane < kSelThreads / 32) s_warp[32 + lane] = y - x;  // exclusive warp offsets
        if (lane == 31) s_warp[64] = y;
    }
    __syncthreads();
    *out = s_warp[32 + w] + incl - v;
    const uint32_t total = s_warp[64];
    __syncthreads();
    return total;
}

// Sorts keys[l, r) ascending (r - l <= kBlockSortMax) in shared memory:
// bitonic sort over the next power of two, padded with the largest key.
__device__ void block_sort(uint64_t* keys, int64_t l, int64_t r, uint64_t* s_buf) {
    const int m = (int)(r - l);
    int m2 = 1;
    while (m2 < m) m2 <<= 1;
    for (int i = threadIdx.x; i < m2; i += blockDim.x) s_buf[i] = i < m ? keys[l + i] : ~0ull;
    __syncthreads();
    for (int size = 2; size <= m2; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = threadIdx.x; i < m2; i += blockDim.x) {
                const int j = i ^ stride;
                if (j > i) {
                    const bool up = (i & size) == 0;
                    const uint64_t a = s_buf[i], b = s_buf[j];
                    if ((a > b) == up) {
                        s_buf[i] = b;
                        s_buf[j] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < m; i += blockDim.x) keys[l + i] = s_buf[i];
    __syncthreads();
}

// ------------------------------------------------ device-wide partitions
// A level with few nodes leaves most of the GPU idle while one block per
// node partitions millions of keys.  While a node's active range is longer
// than kWideMin, its partitions run on the whole GPU instead: the same
// median-of-three, the same pairing of misplaced elements, with the prefix
// counts taken over tiles of kSelTile keys, every such node of the level in
// the same launches.  The block kernel then continues from the saved state.
__device__ __forceinline__ int wide_node_of(const int64_t* __restrict__ tile_off, int count,
                                            int64_t tile) {
    int lo = 0, hi = count - 1;  // last node whose first tile <= tile
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tile_off[mid] <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One block: per node, start (init) or continue a partition step; tiles of
// the step's range, their prefix over nodes, and in ctl the total of tiles
// and the number of nodes partitioned in this step.
__global__ void __launch_bounds__(kSelThreads) wide_setup_kernel(
    int64_t first, int count, const int64_t* __restrict__ rs, const int64_t* __restrict__ re,
    int64_t n_nodes, int init, uint64_t* keys, WideNode* wide, int64_t* __restrict__ tile_off,
    int64_t* __restrict__ ctl) {
    __shared__ uint32_t s_warp[65];
    __shared__ int64_t s_carry;
    __shared__ int s_active;
    if (threadIdx.x == 0) {
        s_carry = 0;
        s_active = 0;
    }
    __syncthreads();
    for (int base = 0; base < count; base += kSelThreads) {
        const int t = base + threadIdx.x;
        int64_t tiles = 0;
        if (t < count) {
            WideNode w = wide[t];
            if (init) {
                const int64_t v = first + t, s0 = rs[v], e0 = re[v], m = e0 - s0;
                w.l = s0;
                w.r = e0;
                w.depth = m > 16 ? 2 * (63 - __clzll((unsigned long long)m)) : 0;
                w.state = (2 * v + 1 >= n_nodes || m < 2) ? kWideDone : kWideActive;
            }
            if (w.state == kWideActive) {
                const int64_t l = w.l, r = w.r, m = r - l;
                if (m <= kWideMin || w.depth == 0) {
                    w.state = kWideBlock;  // the block kernel takes over (or sorts)
                } else {
                    --w.depth;
                    const int64_t mid = (l + r - 1) / 2;  // numba_kdtree.py:282
                    if (keys[l] > keys[mid]) swap_keys(keys, l, mid);
                    if (keys[mid] > keys[r - 1]) {
                        swap_keys(keys, mid, r - 1);
                        if (keys[l] > keys[mid]) swap_keys(keys, l, mid);
                    }
                    swap_keys(keys, mid, r - 1);
                    w.pivot = keys[r - 1];
                    w.K = 0;
                    tiles = (m - 1 + kSelTile - 1) / kSelTile;
                    atomicAdd(&s_active, 1);
                }
            }
            wide[t] = w;
        }
        uint32_t before;
        const uint32_t sum = block_exclusive((uint32_t)tiles, &before, s_warp);
        if (t < count) tile_off[t] = s_carry + before;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += sum;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        ctl[0] = s_carry;   // tiles of this step, over all nodes
        ctl[1] = s_active;  // nodes partitioned in this step
    }
}

// Elements below the pivot in one tile of a node's step range [l, r - 1).
__global__ void __launch_bounds__(kSelThreads) wide_count_kernel(
    int count, const int64_t* __restrict__ tile_off, const WideNode* __restrict__ wide,
    const uint64_t* __restrict__ keys, uint32_t* __restrict__ tile_small) {
    __shared__ uint32_t s_warp[65];
    const int64_t tile = blockIdx.x;
    const int t = wide_node_of(tile_off, count, tile);
    const WideNode w = wide[t];
    const int64_t p0 = w.l + (tile - tile_off[t]) * kSelTile + (int64_t)threadIdx.x * kSelV;
    uint32_t cnt = 0;
#pragma unroll
    for (int j = 0; j < kSelV; ++j) {
        const int64_t p = p0 + j;
        cnt += (p < w.r - 1 && keys[p] < w.pivot) ? 1u : 0u;
    }
    uint32_t dummy;
    const uint32_t total = block_exclusive(cnt, &dummy, s_warp);
    if (threadIdx.x == 0) tile_small[tile] = total;
}

// One block per node: the tiles' exclusive prefix of their counts, the
// node's count c and the pivot's final place B = l + c.
__global__ void __launch_bounds__(kSelThreads) wide_scan_kernel(
    int count, const int64_t* __restrict__ tile_off, const int64_t* __restrict__ ctl,
    WideNode* wide, const uint32_t* __restrict__ tile_small, uint32_t* __restrict__ tile_base) {
    __shared__ uint32_t s_warp[65];
    const int t = blockIdx.x;
    const WideNode w = wide[t];
    if (w.state != kWideActive) return;
    const int64_t a = tile_off[t], b = t + 1 < count ? tile_off[t + 1] : ctl[0];
    uint32_t carry = 0;
    for (int64_t i0 = a; i0 < b; i0 += kSelThreads) {
        const int64_t i = i0 + threadIdx.x;
        uint32_t before;
        const uint32_t sum = block_exclusive(i < b ? tile_small[i] : 0u, &before, s_warp);
        if (i < b) tile_base[i] = carry + before;
        carry += sum;
    }
    if (threadIdx.x == 0) {
        wide[t].c = carry;
        wide[t].B = w.l + carry;
    }
}

// select_level_kernel's pairing, over tiles: elements above the pivot left
// of B, ranked from the left, and elements below it from B on, ranked from
// the right; K counts the pairs.
__global__ void __launch_bounds__(kSelThreads) wide_rank_kernel(
    int count, const int64_t* __restrict__ tile_off, WideNode* wide,
    const uint64_t* __restrict__ keys, const uint32_t* __restrict__ tile_base,
    int32_t* __restrict__ pos_big, int32_t* __restrict__ pos_small) {
    __shared__ uint32_t s_warp[65];
    const int64_t tile = blockIdx.x;
    const int t = wide_node_of(tile_off, count, tile);
    const WideNode w = wide[t];
    const int64_t l = w.l, r = w.r, B = w.B;
    const uint32_t c = w.c;
    const int64_t p0 = l + (tile - tile_off[t]) * kSelTile + (int64_t)threadIdx.x * kSelV;
    uint64_t kv[kSelV];
    uint32_t cnt = 0;
#pragma unroll
    for (int j = 0; j < kSelV; ++j) {
        const int64_t p = p0 + j;
        kv[j] = p < r - 1 ? keys[p] : 0ull;
        cnt += (p < r - 1 && kv[j] < w.pivot) ? 1u : 0u;
    }
    uint32_t before;
    block_exclusive(cnt, &before, s_warp);
    before += tile_base[tile];
    uint32_t kb = 0;
#pragma unroll
    for (int j = 0; j < kSelV; ++j) {
        const int64_t p = p0 + j;
        if (p >= r - 1) break;
        const bool small = kv[j] < w.pivot;
        if (p < B && !small) {
            pos_big[l + (p - l) - before] = (int32_t)p;
            ++kb;
        } else if (p >= B && small) {
            pos_small[l + (c - 1 - before)] = (int32_t)p;
        }
        before += small ? 1u : 0u;
    }
    kb = __reduce_add_sync(kFull, kb);
    if ((threadIdx.x & 31) == 0 && kb) atomicAdd(&wide[t].K, kb);
}

__global__ void __launch_bounds__(kSelThreads) wide_swap_kernel(
    int count, const int64_t* __restrict__ tile_off, const WideNode* __restrict__ wide,
    uint64_t* keys, const int32_t* __restrict__ pos_big, const int32_t* __restrict__ pos_small) {
    const int64_t tile = blockIdx.x;
    const int t = wide_node_of(tile_off, count, tile);
    const WideNode w = wide[t];
    const int64_t k0 = (tile - tile_off[t]) * kSelTile;
    for (int64_t k = k0 + threadIdx.x; k < k0 + kSelTile && k < (int64_t)w.K; k += kSelThreads)
        swap_keys(keys, pos_big[w.l + k], pos_small[w.l + k]);
}

// The pivot to its place; the range narrows to the side holding the median.
__global__ void wide_finish_kernel(int count, WideNode* wide, uint64_t* keys, int64_t first,
                                   const int64_t* __restrict__ rs, const int64_t* __restrict__ re) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    WideNode w = wide[t];
    if (w.state != kWideActive) return;
    swap_keys(keys, w.B, w.r - 1);
    const int64_t v = first + t, nth = rs[v] + (re[v] - rs[v]) / 2;
    if (nth < w.B) w.r = w.B;
    else if (nth > w.B) w.l = w.B + 1;
    else w.state = kWideDone;
    wide[t] = w;
}

// The introselect of keys[l, r) around nth (l <= nth < r), continued in
// shared memory once the active range fits (r - l <= kBlockSortMax): the
// range is read once, every later partition and the final sort run on s_buf,
// and it is written back once.  The pairing positions are 12-bit offsets in
// s_big / s_small (a partition pairs at most (r - l - 1) / 2 elements).
__device__ void select_in_smem(uint64_t* keys, int64_t l, int64_t r, int64_t nth, int depth,
                               uint64_t* s_buf, uint16_t* s_big, uint16_t* s_small,
                               uint32_t* s_warp, uint32_t* s_K) {
    const int m = (int)(r - l), target = (int)(nth - l);
    for (int i = threadIdx.x; i < m; i += blockDim.x) s_buf[i] = keys[l + i];
    __syncthreads();
    int L = 0, R = m;
    while (true) {
        const int mm = R - L;
        if (mm <= 16) {
            // insertion sort (numba_kdtree.py:186): ascending, by ranks
            uint64_t x = 0;
            int rank = 0;
            if (threadIdx.x < mm) {
                x = s_buf[L + threadIdx.x];
                for (int j = 0; j < mm; ++j) rank += s_buf[L + j] < x ? 1 : 0;
            }
            __syncthreads();
            if (threadIdx.x < mm) s_buf[L + rank] = x;
            __syncthreads();
            break;
        }
        if (depth == 0) {
            // the heapsort fallback (numba_kdtree.py:247): ascending
            for (int i = threadIdx.x; i < m; i += blockDim.x) keys[l + i] = s_buf[i];
            __syncthreads();
            block_sort(keys, l + L, l + R, s_buf);
            return;
        }
        --depth;
        if (threadIdx.x == 0) {
            // median of three (numba_kdtree.py:282), the pivot to the end
            const int mid = (L + R - 1) / 2;
            uint64_t a = s_buf[L], b = s_buf[mid], c = s_buf[R - 1], t;
            if (a > b) { t = a; a = b; b = t; }
            if (b > c) {
                t = b; b = c; c = t;
                if (a > b) { t = a; a = b; b = t; }
            }
            s_buf[L] = a;
            s_buf[mid] = c;
            s_buf[R - 1] = b;
            *s_K = 0;
        }
        __syncthreads();
        const uint64_t pivot = s_buf[R - 1];
        const int p0 = L + (int)threadIdx.x * kSelV;
        uint64_t kv[kSelV];
        uint32_t cnt = 0;
#pragma unroll
        for (int j = 0; j < kSelV; ++j) {
            const int p = p0 + j;
            kv[j] = p < R - 1 ? s_buf[p] : 0ull;
            cnt += (p < R - 1 && kv[j] < pivot) ? 1u : 0u;
        }
        uint32_t before;
        const uint32_t c = block_exclusive(cnt, &before, s_warp);
        const int B = L + (int)c;
        uint32_t kb = 0;
#pragma unroll
        for (int j = 0; j < kSelV; ++j) {
            const int p = p0 + j;
            if (p >= R - 1) break;
            const bool small = kv[j] < pivot;
            if (p < B && !small) {
                s_big[(p - L) - before] = (uint16_t)p;
                ++kb;
            } else if (p >= B && small) {
                s_small[c - 1 - before] = (uint16_t)p;
            }
            before += small ? 1u : 0u;
        }
        if (kb) atomicAdd(s_K, kb);
        __syncthreads();
        const uint32_t K = *s_K;
        for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) {
            const int a = s_big[k], b = s_small[k];
            const uint64_t t = s_buf[a];
            s_buf[a] = s_buf[b];
            s_buf[b] = t;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint64_t t = s_buf[B];
            s_buf[B] = s_buf[R - 1];
            s_buf[R - 1] = t;
        }
        __syncthreads();
        if (target < B) R = B;
        else if (target > B) L = B + 1;
        else break;
    }
    for (int i = threadIdx.x; i < m; i += blockDim.x) keys[l + i] = s_buf[i];
}

// One block per internal node of the level: the reference's introselect of
// the node's range around its median position (numba_kdtree.py:395
// _introselect, :372 _introselect_impl).  pos_big / pos_small: per-node
// scratch (the node's own range of two n-long arrays) pairing the swaps of a
// partition while the range is longer than a block holds.  A range that
// reaches the depth limit while longer than a block can sort is recorded in
// big_sort (its bounds) for a device-wide sort after the launch.  wide
// (nullable): the state the device-wide partitions left for each node.
__global__ void __launch_bounds__(kSelThreads) select_level_kernel(
    int64_t first, const int64_t* __restrict__ rs, const int64_t* __restrict__ re,
    int64_t n_nodes, uint64_t* keys, int32_t* __restrict__ pos_big,
    int32_t* __restrict__ pos_small, int64_t* __restrict__ big_sort, int* big_sort_count,
    const WideNode* __restrict__ wide) {
    __shared__ uint64_t s_buf[kBlockSortMax];
    __shared__ uint16_t s_big[kBlockSortMax / 2], s_small[kBlockSortMax / 2];
    __shared__ uint32_t s_warp[65];
    __shared__ int64_t s_l, s_r;
    __shared__ uint64_t s_pivot;
    __shared__ int s_done;
    __shared__ uint32_t s_K;
    const int64_t v = first + blockIdx.x;
    const int64_t s0 = rs[v], e0 = re[v];
    // a node is a leaf when it has no children slots or fewer than 2 points
    if (2 * v + 1 >= n_nodes || e0 - s0 < 2) return;
    const int64_t nth = s0 + (e0 - s0) / 2;
    if (threadIdx.x == 0) {
        s_l = s0;
        s_r = e0;
        s_done = 0;
    }
    const int64_t size0 = e0 - s0;
    // 2 * int(log2(size)) (numba_kdtree.py:411), exact for integers
    int depth = size0 > 16 ? 2 * (63 - __clzll((unsigned long long)size0)) : 0;
    if (wide) {  // the device-wide partitions already ran the first steps
        const WideNode w = wide[blockIdx.x];
        if (w.state == kWideDone) return;
        if (threadIdx.x == 0) {
            s_l = w.l;
            s_r = w.r;
        }
        depth = w.depth;
    }
    __syncthreads();
    while (true) {
        const int64_t l = s_l, r = s_r;
        if (r - l <= kBlockSortMax) {
            select_in_smem(keys, l, r, nth, depth, s_buf, s_big, s_small, s_warp, &s_K);
            return;
        }
        if (depth == 0) {
            // the heapsort fallback on a range longer than a block sorts:
            // sorted ascending on the device after the launch
            if (threadIdx.x == 0) {
                const int slot = atomicAdd(big_sort_count, 1);
                big_sort[2 * slot] = l;
                big_sort[2 * slot + 1] = r;
            }
            return;
        }
        --depth;
        if (threadIdx.x == 0) {
            // median of three (numba_kdtree.py:282), then the pivot to the
            // end (:316)
            const int64_t mid = (l + r - 1) / 2;
            if (keys[l] > keys[mid]) swap_keys(keys, l, mid);
            if (keys[mid] > keys[r - 1]) {
                swap_keys(keys, mid, r - 1);
                if (keys[l] > keys[mid]) swap_keys(keys, l, mid);
            }
            swap_keys(keys, mid, r - 1);
            s_pivot = keys[r - 1];
            s_K = 0;
        }
        __syncthreads();
        const uint64_t pivot = s_pivot;
        // elements below the pivot in [l, r - 1)
        uint32_t c_loc = 0;
        for (int64_t p = l + threadIdx.x; p < r - 1; p += blockDim.x) c_loc += keys[p] < pivot;
        uint32_t dummy;
        const uint32_t c = block_exclusive(c_loc, &dummy, s_warp);
        const int64_t B = l + c;
        // pair the elements above the pivot left of B (ranked from the left)
        // with those below it from B on (ranked from the right)
        uint32_t carry = 0;
        for (int64_t base = l; base < r - 1; base += kSelTile) {
            const int64_t p0 = base + (int64_t)threadIdx.x * kSelV;
            uint64_t kv[kSelV];
            uint32_t cnt = 0;
#pragma unroll
            for (int j = 0; j < kSelV; ++j) {
                const int64_t p = p0 + j;
                kv[j] = p < r - 1 ? keys[p] : 0ull;
                cnt += (p < r - 1 && kv[j] < pivot) ? 1u : 0u;
            }
            uint32_t before;
            const uint32_t tile_total = block_exclusive(cnt, &before, s_warp);
            before += carry;
            uint32_t kb = 0;
#pragma unroll
            for (int j = 0; j < kSelV; ++j) {
                const int64_t p = p0 + j;
                if (p >= r - 1) break;
                const bool small = kv[j] < pivot;
                if (p < B && !small) {
                    pos_big[l + (p - l) - before] = (int32_t)p;
                    ++kb;
                } else if (p >= B && small) {
                    pos_small[l + (c - 1 - before)] = (int32_t)p;
                }
                before += small ? 1u : 0u;
            }
            if (kb) atomicAdd(&s_K, kb);
            carry += tile_total;
        }
        __syncthreads();
        const uint32_t K = s_K;
        for (uint32_t k = threadIdx.x; k < K; k += blockDim.x)
            swap_keys(keys, pos_big[l + k], pos_small[l + k]);
        __syncthreads();
        if (threadIdx.x == 0) {
            swap_keys(keys, B, r - 1);
            if (nth < B) s_r = B;
            else if (nth > B) s_l = B + 1;
            else s_done = 1;
        }
        __syncthreads();
        if (s_done) return;
    }
}

// ----------------------------------------------- the reference's kNN query
constexpr int kRefKnnMax = 64;  // heap entries
constexpr int kRefStack = 64;   // pending subtrees of the walk (<= levels + 1)

// simple_heap_push (numba_kdtree.py:578): a max-heap of k entries whose root
// is replaced by a smaller priority and sifted down, with its tie rules.
__device__ __forceinline__ void ref_heap_push(float* pri, int32_t* ind, int size, float p,
                                              int32_t x) {
    if (p >= pri[0]) return;
    int i = 0;
    while (true) {
        const int c1 = 2 * i + 1, c2 = c1 + 1;
        int sw;
        if (c1 >= size) break;
        if (c2 >= size) {
            if (pri[c1] > p) sw = c1;
            else break;
        } else if (pri[c1] >= pri[c2]) {
            if (p < pri[c1]) sw = c1;
            else break;
        } else {
            if (p < pri[c2]) sw = c2;
            else break;
        }
        pri[i] = pri[sw];
        ind[i] = ind[sw];
        i = sw;
    }
    pri[i] = p;
    ind[i] = x;
}

// One thread per caller point: tree_query_recursion (numba_kdtree.py:680)
// with an explicit stack -- a subtree is pruned when its bound exceeds the
// heap's largest entry at the time it is visited, a leaf pushes its points in
// tree order, an internal node visits the child of smaller bound first (the
// left one on equal bounds) -- then deheap_sort (:652, siftdown :630).
__global__ void __launch_bounds__(128) ref_knn_kernel(
    RefTreeView t, const int32_t* __restrict__ tidx, const float* __restrict__ pts, int pad,
    const int32_t* __restrict__ rank, const int32_t* __restrict__ orig,
    const int32_t* __restrict__ list, int64_t count, int k, int kk, int sqrt_order,
    float* __restrict__ d_s, int32_t* __restrict__ s_s, int32_t* __restrict__ nbr_o,
    int nbr_cols) {
    const int64_t li = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= count) return;
    const int64_t c = orig[list[li]];  // the query, by caller index
    const int d = t.d;
    float q[32];
    const float* qp = pts + (int64_t)rank[c] * pad;
    for (int j = 0; j < d; ++j) q[j] = qp[j];
    float pri[kRefKnnMax], rd[kRefKnnMax];
    int32_t ind[kRefKnnMax];
    for (int j = 0; j < k; ++j) {
        pri[j] = INFINITY;
        ind[j] = -1;
    }
    int32_t st_v[kRefStack], st_s[kRefStack], st_e[kRefStack];
    float st_lb[kRefStack];
    int sp = 0;
    st_v[0] = 0;
    st_s[0] = 0;
    st_e[0] = (int32_t)t.n;
    st_lb[0] = ref_node_lb(t, 0, q);
    sp = 1;
    while (sp > 0) {
        --sp;
        const int32_t v = st_v[sp], s0 = st_s[sp], e0 = st_e[sp];
        if (st_lb[sp] > pri[0]) continue;
        if (2 * (int64_t)v + 1 >= t.nodes || e0 - s0 < 2) {
            for (int32_t i = s0; i < e0; ++i) {
                const int32_t x = tidx[i];
                const float* xp = pts + (int64_t)rank[x] * pad;
                float r = 0.0f;
                for (int j = 0; j < d; ++j) {
                    const float df = __fsub_rn(q[j], xp[j]);
                    r = __fadd_rn(r, __fmul_rn(df, df));
                }
                if (r < pri[0]) ref_heap_push(pri, ind, k, r, x);
            }
        } else if (sp + 2 <= kRefStack) {
            const int32_t mid = s0 + (e0 - s0) / 2, l = 2 * v + 1, r = l + 1;
            const float bl = ref_node_lb(t, l, q), br = ref_node_lb(t, r, q);
            // the child visited first goes on top
            const bool left_first = bl <= br;
            st_v[sp] = left_first ? r : l;
            st_s[sp] = left_first ? mid : s0;
            st_e[sp] = left_first ? e0 : mid;
            st_lb[sp] = left_first ? br : bl;
            ++sp;
            st_v[sp] = left_first ? l : r;
            st_s[sp] = left_first ? s0 : mid;
            st_e[sp] = left_first ? mid : e0;
            st_lb[sp] = left_first ? bl : br;
            ++sp;
        }
    }
    // deheap_sort on the distances the query returns: squared, or their
    // square roots; the squared values travel with their entries
    for (int j = 0; j < k; ++j) {
        rd[j] = pri[j];
        if (sqrt_order) pri[j] = __fsqrt_rn(pri[j]);
    }
    for (int j = k - 1; j > 0; --j) {
        float tp = pri[0]; pri[0] = pri[j]; pri[j] = tp;
        float tr = rd[0]; rd[0] = rd[j]; rd[j] = tr;
        int32_t ti = ind[0]; ind[0] = ind[j]; ind[j] = ti;
        int e = 0;  // siftdown of [0, j)
        while (e * 2 + 1 < j) {
            const int lc = e * 2 + 1, rc = lc + 1;
            int sw = e;
            if (pri[sw] < pri[lc]) sw = lc;
            if (rc < j && pri[sw] < pri[rc]) sw = rc;
            if (sw == e) break;
            tp = pri[e]; pri[e] = pri[sw]; pri[sw] = tp;
            tr = rd[e]; rd[e] = rd[sw]; rd[sw] = tr;
            ti = ind[e]; ind[e] = ind[sw]; ind[sw] = ti;
            e = sw;
        }
    }
    const int64_t p = rank[c];
    for (int j = 0; j < kk; ++j) {
        d_s[p * kk + j] = rd[j];
        s_s[p * kk + j] = ind[j] >= 0 ? rank[ind[j]] : -1;
        if (nbr_o && j >= 1 && j - 1 < nbr_cols) nbr_o[c * nbr_cols + j - 1] = ind[j];
    }
}

// Rows whose order can differ from the reference's: two entries at the same
// distance (the reference lists them in its query and heap order, the engine
// by index; with sqrt_order, the same square root), or a point outside the
// list at the k-th distance (tie, from the kNN kernel: the reference keeps
// the first one its walk meets).  Elsewhere the k nearest and their order
// are unique.
__global__ void tie_rows_kernel(int64_t n, int kk, int sqrt_order,
                                const float* __restrict__ d_s, const int8_t* __restrict__ tie,
                                uint32_t* __restrict__ flag) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    bool f = tie && tie[p] != 0;
    for (int j = 0; j + 1 < kk && !f; ++j) {
        const float a = d_s[p * kk + j], b = d_s[p * kk + j + 1];
        f = sqrt_order ? __fsqrt_rn(a) == __fsqrt_rn(b) : a == b;
    }
    flag[p] = f ? 1u : 0u;
}
__global__ void tie_list_kernel(int64_t n, const uint32_t* __restrict__ flag,
                                const uint32_t* __restrict__ pos, int32_t* __restrict__ list) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n && flag[p]) list[pos[p]] = (int32_t)p;
}

}  // namespace

int ref_knn(const RefTree& t, const fhg_index& ix, int k, bool sqrt_order, const int8_t* tie,
            float* d_s, int32_t* s_s, int32_t* nbr_o, int nbr_cols, cudaStream_t s) {
    if (k < 1 || k > kRefKnnMax || t.d > 32 || t.levels + 1 > kRefStack) {
        set_error("reference kNN: k = %d, d = %d, %d levels out of range", k, t.d, t.levels);
        return FHG_ERR_UNSUPPORTED;
    }
    const int64_t n = t.n;
    const int kk = (int)(k < n ? k : n);
    Stage stage(s, "ref_knn");
    Workspace tmp(s);
    uint32_t *flag, *pos, *cnt;
    int32_t* list;
    FHG_TRY(tmp.alloc(&flag, (size_t)n));
    FHG_TRY(tmp.alloc(&pos, (size_t)n));
    FHG_TRY(tmp.alloc(&cnt, 1));
    FHG_TRY(tmp.alloc(&list, (size_t)n));
    LAUNCH(tie_rows_kernel, n, n, kk, sqrt_order ? 1 : 0, d_s, tie, flag);
    FHG_TRY(scan_exclusive_u32(tmp, flag, pos, n, cnt));
    LAUNCH(tie_list_kernel, n, n, flag, pos, list);
    uint32_t h_cnt = 0;
    FHG_CUDA(cudaMemcpyAsync(&h_cnt, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    profile_count("ref_knn_rows", (double)h_cnt);
    if (h_cnt == 0) return FHG_OK;
    ::fhg::note_launch();
    ref_knn_kernel<<<grid_for((int64_t)h_cnt, 128), 128, 0, s>>>(
        view_of(t), t.idx, ix.pts, ix.pad, ix.rank, ix.orig, list, (int64_t)h_cnt, k, kk,
        sqrt_order ? 1 : 0, d_s, s_s, nbr_o, nbr_cols);
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

// [nodes][2][d] -> the reference's node_bounds layout [2][nodes][d]
__global__ void bounds_layout_kernel(int64_t nodes, int d, const float* __restrict__ box,
                                     float* __restrict__ out) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nodes * 2 * d) return;
    const int64_t v = t / (2 * d);
    const int side = (int)((t / d) % 2), j = (int)(t % d);
    out[(int64_t)side * nodes * d + v * d + j] = box[t];
}

int ref_tree_export(const RefTree& t, int32_t* idx_array, float* node_bounds, cudaStream_t s) {
    if (idx_array)
        FHG_CUDA(cudaMemcpyAsync(idx_array, t.idx, sizeof(int32_t) * t.n,
                                 cudaMemcpyDeviceToDevice, s));
    if (node_bounds) LAUNCH(bounds_layout_kernel, t.nodes * 2 * t.d, t.nodes, t.d, t.box, node_bounds);
    return FHG_OK;
}

int ref_tree_levels(int64_t n) {
    // numba_kdtree.py:486: int(np.log2(max(1, (n - 1) / leaf_size)) + 1), leaf_size 40
    double x = (double)(n - 1) / 40.0;
    if (x < 1.0) x = 1.0;
    return (int)(std::log2(x) + 1.0);
}

int ref_tree_build(Workspace& ws, const fhg_index& ix, RefTree* out) {
    cudaStream_t s = ws.stream();
    const int64_t n = ix.n;
    const int d = ix.d, pad = ix.pad;
    *out = RefTree();
    out->n = n;
    out->d = d;
    out->levels = ref_tree_levels(n);
    const int64_t nodes = ((int64_t)1 << out->levels) - 1;
    out->nodes = nodes;
    Stage stage(s, "ref_tree_build");
    FHG_TRY(ws.alloc(&out->idx, (size_t)n));
    FHG_TRY(ws.alloc(&out->pos, (size_t)n));
    FHG_TRY(ws.alloc(&out->box, (size_t)(nodes * 2 * d)));
    Workspace tmp(s);
    int32_t *nodeof, *axis, *pos_big, *pos_small, *dummy;
    int64_t *rs, *re, *big_sort;
    uint32_t *lo, *hi;
    uint64_t* keys;
    int* big_count;
    FHG_TRY(tmp.alloc(&nodeof, (size_t)n));
    FHG_TRY(tmp.alloc(&axis, (size_t)((nodes + 1) / 2)));
    FHG_TRY(tmp.alloc(&pos_big, (size_t)n));
    FHG_TRY(tmp.alloc(&pos_small, (size_t)n));
    FHG_TRY(tmp.alloc(&rs, (size_t)nodes));
    FHG_TRY(tmp.alloc(&re, (size_t)nodes));
    FHG_TRY(tmp.alloc(&lo, (size_t)(nodes * d)));
    FHG_TRY(tmp.alloc(&hi, (size_t)(nodes * d)));
    FHG_TRY(tmp.alloc(&keys, (size_t)n));
    FHG_TRY(tmp.alloc(&big_count, 1));
    const int64_t max_level_nodes = (nodes + 1) / 2;
    FHG_TRY(tmp.alloc(&big_sort, (size_t)(2 * max_level_nodes)));
    // device-wide partitions: saved node states, tile offsets, tile counts
    int64_t wide_levels = 0;
    while (wide_levels + 1 < out->levels && ((n + ((int64_t)1 << wide_levels) - 1) >> wide_levels) > kWideMin)
        ++wide_levels;
    WideNode* wide = nullptr;
    int64_t *tile_off = nullptr, *ctl = nullptr;
    uint32_t *tile_small = nullptr, *tile_base = nullptr;
    if (wide_levels > 0) {
        const int64_t wide_nodes = (int64_t)1 << (wide_levels - 1);
        const size_t max_tiles = (size_t)(n / kSelTile + wide_nodes + 1);
        FHG_TRY(tmp.alloc(&wide, (size_t)wide_nodes));
        FHG_TRY(tmp.alloc(&tile_off, (size_t)wide_nodes));
        FHG_TRY(tmp.alloc(&ctl, 2));
        FHG_TRY(tmp.alloc(&tile_small, max_tiles));
        FHG_TRY(tmp.alloc(&tile_base, max_tiles));
    }
    float* ptsc;
    FHG_TRY(tmp.alloc(&ptsc, (size_t)(n * pad)));
    LAUNCH(caller_order_kernel, n * pad, n, pad, ix.orig, ix.pts, ptsc);
    LAUNCH(init_root_kernel, n, n, out->idx, nodeof, rs, re);
    for (int lvl = 0; lvl < out->levels; ++lvl) {
        const int64_t first = ((int64_t)1 << lvl) - 1, count = (int64_t)1 << lvl;
        const bool last = lvl + 1 == out->levels;
        {
            Stage boxes(s, "ref_tree_boxes");
            LAUNCH(box_init_kernel, count * d, first, count, d, lo, hi);
            LAUNCH(box_level_kernel, n, n, d, pad, out->idx, nodeof, ptsc, lo, hi);
            LAUNCH(axis_level_kernel, count, first, count, d, lo, hi, out->box,
                   last ? nullptr : axis);
        }
        if (last) break;
        {
            Stage kst(s, "ref_tree_keys");
            LAUNCH(child_ranges_kernel, count, first, count, rs, re);
            LAUNCH(keys_level_kernel, n, n, first, pad, out->idx, nodeof, axis, ptsc, keys);
        }
        FHG_CUDA(cudaMemsetAsync(big_count, 0, sizeof(int), s));
        const bool wide_level = lvl < wide_levels;  // some node longer than kWideMin
        if (wide_level) {
            Stage sel(s, "ref_tree_select_wide");
            for (int init = 1;; init = 0) {
                ::fhg::note_launch();
                wide_setup_kernel<<<1, kSelThreads, 0, s>>>(first, (int)count, rs, re, nodes, init,
                                                           keys, wide, tile_off, ctl);
                FHG_CUDA(cudaGetLastError());
                int64_t h_ctl[2];
                FHG_CUDA(cudaMemcpyAsync(h_ctl, ctl, sizeof(h_ctl), cudaMemcpyDeviceToHost, s));
                FHG_CUDA(cudaStreamSynchronize(s));
                if (h_ctl[1] == 0) break;
                const unsigned tiles = (unsigned)h_ctl[0];
                ::fhg::note_launch();
                wide_count_kernel<<<tiles, kSelThreads, 0, s>>>((int)count, tile_off, wide, keys,
                                                                tile_small);
                ::fhg::note_launch();
                wide_scan_kernel<<<(unsigned)count, kSelThreads, 0, s>>>((int)count, tile_off, ctl,
                                                                         wide, tile_small, tile_base);
                ::fhg::note_launch();
                wide_rank_kernel<<<tiles, kSelThreads, 0, s>>>((int)count, tile_off, wide, keys,
                                                               tile_base, pos_big, pos_small);
                ::fhg::note_launch();
                wide_swap_kernel<<<tiles, kSelThreads, 0, s>>>((int)count, tile_off, wide, keys,
                                                               pos_big, pos_small);
                FHG_CUDA(cudaGetLastError());
                LAUNCH(wide_finish_kernel, count, (int)count, wide, keys, first, rs, re);
            }
        }
        {
            Stage sel(s, wide_level ? "ref_tree_select_top" : "ref_tree_select_deep");
            ::fhg::note_launch();
            select_level_kernel<<<(unsigned)count, kSelThreads, 0, s>>>(
                first, rs, re, nodes, keys, pos_big, pos_small, big_sort, big_count,
                wide_level ? wide : nullptr);
            FHG_CUDA(cudaGetLastError());
        }
        int h_big = 0;
        FHG_CUDA(cudaMemcpyAsync(&h_big, big_count, sizeof(int), cudaMemcpyDeviceToHost, s));
        FHG_CUDA(cudaStreamSynchronize(s));
        if (h_big > 0) {
            // ranges that hit the depth limit while longer than a block sorts:
            // sorted ascending on the device (the heapsort's result)
            std::vector<int64_t> h_ranges(2 * (size_t)h_big);
            FHG_CUDA(cudaMemcpyAsync(h_ranges.data(), big_sort, sizeof(int64_t) * 2 * h_big,
                                     cudaMemcpyDeviceToHost, s));
            FHG_CUDA(cudaStreamSynchronize(s));
            for (int i = 0; i < h_big; ++i) {
                const int64_t l = h_ranges[2 * i], r = h_ranges[2 * i + 1];
                Workspace one(s);
                FHG_TRY(one.alloc(&dummy, (size_t)(r - l)));
                FHG_TRY(radix_sort_u64(one, keys + l, dummy, r - l, 0, 64));
            }
        }
        LAUNCH(unpack_level_kernel, n, n, keys, rs, re, out->idx, nodeof);
    }
    LAUNCH(inverse_kernel, n, n, out->idx, out->pos);
    return FHG_OK;
}

}  // namespace fhg
