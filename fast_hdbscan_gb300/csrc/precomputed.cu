// Precomputed sparse graphs (metric="precomputed"): precomputed.py:479
// compute_mst_from_precomputed_sparse_kruskal and :410
// compute_mst_from_precomputed_sparse, without cannot-link constraints.
//
// The reference symmetrises the graph by the least weight per undirected pair
// without its diagonal (:70 _symmetrize_min_csr), takes every point's core
// distance as the min_samples-th smallest weight of its row (:148
// _core_distances_csr), gives every stored entry its float64
// mutual-reachability weight max(core_i, core_j, w_ij) and builds the minimum
// spanning forest -- Kruskal over a stable argsort of the entries, or its
// float32 Boruvka -- then joins the components with +inf bridges.
//
// Here every step is a sort or a pass over the entries: the symmetrised
// graph by a stable radix sort of the (min, max) pair keys with a segmented
// minimum, its CSR order (pairs (i, j) with i < j first, then the mirrored
// ones, each stably by row, as the reference's two concatenated halves) by a
// stable radix sort of the row; row order by weight by a two-key LSD sort;
// the forest by the Boruvka rounds over sorted ranks of kruskal.cu.  The
// forest is Kruskal's (float64 weight, then entry position) for both
// algorithms: the reference's Boruvka returns a forest of the same weights,
// whose equal-weight choices and edge order are its own.
#include "mst.cuh"
#include "primitives.cuh"

namespace fhg {
namespace {

#define LAUNCH(kernel, count, ...)                                        \
    do {                                                                  \
        if ((count) > 0) {                                                \
            ::fhg::note_launch();                                         \
            kernel<<<grid_for((count), 256), 256, 0, s>>>(__VA_ARGS__);   \
            FHG_CUDA(cudaGetLastError());                                 \
        }                                                                 \
    } while (0)

__device__ __forceinline__ uint64_t f64_bits(double x) {  // x >= 0 (or +inf)
    return (uint64_t)__double_as_longlong(x);
}

__global__ void pc_offdiag_kernel(int64_t nnz, const int32_t* __restrict__ rows,
                                  const int32_t* __restrict__ cols, uint32_t* __restrict__ flag) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nnz) flag[t] = rows[t] != cols[t] ? 1u : 0u;
}
// (min, max) pair key of every off-diagonal entry, in input order.
__global__ void pc_pairs_kernel(int64_t nnz, int64_t n, const int32_t* __restrict__ rows,
                                const int32_t* __restrict__ cols, const double* __restrict__ data,
                                const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos,
                                uint64_t* __restrict__ key, int32_t* __restrict__ at,
                                double* __restrict__ d0) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnz || !flag[t]) return;
    const int64_t u = min(rows[t], cols[t]), v = max(rows[t], cols[t]);
    const uint32_t o = pos[t];
    key[o] = (uint64_t)u * (uint64_t)n + (uint64_t)v;
    at[o] = (int32_t)o;
    d0[o] = data[t];
}
__global__ void pc_group_flags_kernel(int64_t m0, const uint64_t* __restrict__ key,
                                      uint32_t* __restrict__ flag) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m0) flag[j] = (j == 0 || key[j] != key[j - 1]) ? 1u : 0u;
}
__global__ void pc_fill_u64_kernel(uint64_t* a, int64_t n, uint64_t v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}
// np.minimum.reduceat over each pair's run (the weights are >= 0, so their
// bit patterns order like the values).
__global__ void pc_group_min_kernel(int64_t m0, int64_t n, const uint64_t* __restrict__ key,
                                    const int32_t* __restrict__ at, const double* __restrict__ d0,
                                    const uint32_t* __restrict__ flag,
                                    const uint32_t* __restrict__ gpos,
                                    unsigned long long* __restrict__ gmin,
                                    int32_t* __restrict__ gu, int32_t* __restrict__ gv) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m0) return;
    // group of j: the last group start at or before j
    const int64_t g = (int64_t)gpos[j] + (flag[j] ? 0 : -1);
    atomicMin(&gmin[g], (unsigned long long)f64_bits(d0[at[j]]));
    if (flag[j]) {
        gu[g] = (int32_t)(key[j] / (uint64_t)n);
        gv[g] = (int32_t)(key[j] % (uint64_t)n);
    }
}
// The symmetric entries: pairs (u, v) in pair order, then (v, u) likewise.
__global__ void pc_sym_kernel(int64_t mu, const int32_t* __restrict__ gu,
                              const int32_t* __restrict__ gv, uint32_t* __restrict__ rowkey,
                              int32_t* __restrict__ perm) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * mu) return;
    rowkey[t] = (uint32_t)(t < mu ? gu[t] : gv[t - mu]);
    perm[t] = (int32_t)t;
}
__global__ void pc_csr_kernel(int64_t M, int64_t mu, const int32_t* __restrict__ perm,
                              const int32_t* __restrict__ gu, const int32_t* __restrict__ gv,
                              const unsigned long long* __restrict__ gmin,
                              int32_t* __restrict__ srow, int32_t* __restrict__ scol,
                              double* __restrict__ sd, uint32_t* __restrict__ count) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= M) return;
    const int64_t t = perm[p];
    const int64_t g = t < mu ? t : t - mu;
    const int32_t r = t < mu ? gu[g] : gv[g];
    srow[p] = r;
    scol[p] = t < mu ? gv[g] : gu[g];
    sd[p] = __longlong_as_double((long long)gmin[g]);
    atomicAdd(&count[r], 1u);
}
__global__ void pc_weight_keys_kernel(int64_t M, const double* __restrict__ sd,
                                      uint64_t* __restrict__ key, int32_t* __restrict__ perm) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= M) return;
    key[p] = f64_bits(sd[p]);
    perm[p] = (int32_t)p;
}
__global__ void pc_row_keys_kernel(int64_t M, const int32_t* __restrict__ perm,
                                   const int32_t* __restrict__ srow, uint32_t* __restrict__ key) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < M) key[q] = (uint32_t)srow[perm[q]];
}
__global__ void pc_core_init_kernel(int64_t n, int k, int ms, int32_t* __restrict__ nbrs,
                                    double* __restrict__ core) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n * k) nbrs[t] = -1;
    if (t < n) core[t] = ms > 1 ? INFINITY : 0.0;
}
// :148 _core_distances_csr on the rows ordered by weight (ties by position).
__global__ void pc_core_kernel(int64_t M, int k, int ms, const int32_t* __restrict__ perm,
                               const int32_t* __restrict__ srow, const int32_t* __restrict__ scol,
                               const double* __restrict__ sd, const uint32_t* __restrict__ indptr,
                               int32_t* __restrict__ nbrs, double* __restrict__ core) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= M) return;
    const int32_t p = perm[q];
    const int32_t r = srow[p];
    const int64_t j = q - (int64_t)indptr[r];
    if (j < k) nbrs[(int64_t)r * k + j] = scol[p];
    if (ms > 1 && j == ms - 1) core[r] = sd[p];
}
// kruskal.py:421 _compute_mrd_csr_flat.
__global__ void pc_mrd_kernel(int64_t M, const int32_t* __restrict__ srow,
                              const int32_t* __restrict__ scol, const double* __restrict__ sd,
                              const double* __restrict__ core, uint64_t* __restrict__ key,
                              int32_t* __restrict__ perm) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= M) return;
    double mrd = core[srow[p]];
    const double cj = core[scol[p]];
    if (cj > mrd) mrd = cj;
    if (sd[p] > mrd) mrd = sd[p];
    key[p] = f64_bits(mrd);
    perm[p] = (int32_t)p;
}
__global__ void pc_ranks_kernel(int64_t M, const int32_t* __restrict__ perm,
                                const int32_t* __restrict__ srow, const int32_t* __restrict__ scol,
                                const uint64_t* __restrict__ key, int2* __restrict__ uv,
                                double* __restrict__ w) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= M) return;
    const int32_t p = perm[r];
    uv[r] = make_int2(srow[p], scol[p]);
    w[r] = __longlong_as_double((long long)key[r]);
}

}  // namespace

int precomputed_mst(const int32_t* rows, const int32_t* cols, const double* data, int64_t nnz,
                    int64_t n, int min_samples, double* edges, int32_t* neighbors, double* core,
                    int64_t* n_components, cudaStream_t s) {
    if (nnz > 0x7fffffffLL) {
        set_error("precomputed: %lld stored entries exceed the int32 entry index",
                  (long long)nnz);
        return FHG_ERR_UNSUPPORTED;
    }
    const int k = min_samples > 1 ? min_samples : 1;
    *n_components = n > 0 ? 1 : 0;
    if (n < 1) return FHG_OK;
    Stage stage(s, "precomputed_mst");
    Workspace ws(s);
    uint32_t* cnt;
    FHG_TRY(ws.alloc(&cnt, 2));
    LAUNCH(pc_core_init_kernel, n * k, n, k, min_samples, neighbors, core);

    // ---- _symmetrize_min_csr
    const size_t nz = (size_t)(nnz > 0 ? nnz : 1);
    uint32_t *flag, *pos;
    FHG_TRY(ws.alloc(&flag, nz));
    FHG_TRY(ws.alloc(&pos, nz));
    LAUNCH(pc_offdiag_kernel, nnz, nnz, rows, cols, flag);
    FHG_TRY(scan_exclusive_u32(ws, flag, pos, nnz, cnt));
    uint32_t h = 0;
    FHG_CUDA(cudaMemcpyAsync(&h, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    const int64_t m0 = h;
    const size_t mz = (size_t)(m0 > 0 ? m0 : 1);
    uint64_t* key;
    int32_t* at;
    double* d0;
    FHG_TRY(ws.alloc(&key, mz));
    FHG_TRY(ws.alloc(&at, mz));
    FHG_TRY(ws.alloc(&d0, mz));
    LAUNCH(pc_pairs_kernel, nnz, nnz, n, rows, cols, data, flag, pos, key, at, d0);
    if (m0 > 1) {
        Workspace tmp(s);
        const int kb = 2 * bits_for(n);
        FHG_TRY(radix_sort_u64(tmp, key, at, m0, 0, kb < 64 ? kb : 64));
    }
    uint32_t *gflag, *gpos;
    FHG_TRY(ws.alloc(&gflag, mz));
    FHG_TRY(ws.alloc(&gpos, mz));
    LAUNCH(pc_group_flags_kernel, m0, m0, key, gflag);
    FHG_TRY(scan_exclusive_u32(ws, gflag, gpos, m0, cnt));
    FHG_CUDA(cudaMemcpyAsync(&h, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    FHG_CUDA(cudaStreamSynchronize(s));
    const int64_t mu = m0 > 0 ? h : 0;
    const size_t gz = (size_t)(mu > 0 ? mu : 1);
    unsigned long long* gmin;
    int32_t *gu, *gv;
    FHG_TRY(ws.alloc(&gmin, gz));
    FHG_TRY(ws.alloc(&gu, gz));
    FHG_TRY(ws.alloc(&gv, gz));
    LAUNCH(pc_fill_u64_kernel, mu, reinterpret_cast<uint64_t*>(gmin), mu, ~0ull);
    LAUNCH(pc_group_min_kernel, m0, m0, n, key, at, d0, gflag, gpos, gmin, gu, gv);

    // ---- the symmetric CSR: both halves, stably by row
    const int64_t M = 2 * mu;
    if (M > 0x7fffffffLL) {
        set_error("precomputed: %lld symmetric entries exceed the int32 entry index",
                  (long long)M);
        return FHG_ERR_UNSUPPORTED;
    }
    const size_t Mz = (size_t)(M > 0 ? M : 1);
    uint32_t *rowkey, *count, *indptr;
    int32_t *perm, *srow, *scol;
    double* sd;
    FHG_TRY(ws.alloc(&rowkey, Mz));
    FHG_TRY(ws.alloc(&perm, Mz));
    FHG_TRY(ws.alloc(&srow, Mz));
    FHG_TRY(ws.alloc(&scol, Mz));
    FHG_TRY(ws.alloc(&sd, Mz));
    FHG_TRY(ws.alloc(&count, (size_t)n));
    FHG_TRY(ws.alloc(&indptr, (size_t)n));
    FHG_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t) * n, s));
    LAUNCH(pc_sym_kernel, M, mu, gu, gv, rowkey, perm);
    if (M > 1) {
        Workspace tmp(s);
        FHG_TRY(radix_sort_u32(tmp, rowkey, perm, M, 0, bits_for(n)));
    }
    LAUNCH(pc_csr_kernel, M, M, mu, perm, gu, gv, gmin, srow, scol, sd, count);
    FHG_TRY(scan_exclusive_u32(ws, count, indptr, n, cnt));

    // ---- _core_distances_csr: every row by weight, ties by position
    if (M > 0) {
        uint64_t* wkey;
        FHG_TRY(ws.alloc(&wkey, Mz));
        LAUNCH(pc_weight_keys_kernel, M, M, sd, wkey, perm);
        {
            Workspace tmp(s);
            if (M > 1) FHG_TRY(radix_sort_u64(tmp, wkey, perm, M, 0, 64));
        }
        LAUNCH(pc_row_keys_kernel, M, M, perm, srow, rowkey);
        {
            Workspace tmp(s);
            if (M > 1) FHG_TRY(radix_sort_u32(tmp, rowkey, perm, M, 0, bits_for(n)));
        }
        LAUNCH(pc_core_kernel, M, M, k, min_samples, perm, srow, scol, sd, indptr, neighbors,
               core);
    }

    // ---- mutual-reachability weights, stably sorted, and the forest
    uint64_t* mkey;
    int2* uv;
    double* w;
    FHG_TRY(ws.alloc(&mkey, Mz));
    FHG_TRY(ws.alloc(&uv, Mz));
    FHG_TRY(ws.alloc(&w, Mz));
    LAUNCH(pc_mrd_kernel, M, M, srow, scol, sd, core, mkey, perm);
    if (M > 1) {
        Workspace tmp(s);
        FHG_TRY(radix_sort_u64(tmp, mkey, perm, M, 0, 64));
    }
    LAUNCH(pc_ranks_kernel, M, M, perm, srow, scol, mkey, uv, w);
    if (n < 2) return FHG_OK;
    return sorted_forest_edges(ws, n, M, 0, nullptr, nullptr, uv, nullptr, 0, edges,
                               n_components, w);
}

}  // namespace fhg
