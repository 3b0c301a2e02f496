// The reference's KD-tree (numba_kdtree.py:410-521), built exactly on the
// GPU, and the order in which the reference's depth-first walks meet its
// points -- the tie-breaker of the reference tie mode.
#pragma once
#include "index.cuh"

namespace fhg {

// n points, `levels` levels, nodes = 2^levels - 1 in heap order (children of
// v at 2v+1, 2v+2); node v covers tree positions [s, s + (e - s) / 2) on the
// left and the rest on the right of its range [s, e).
struct RefTree {
    int64_t n = 0;
    int32_t d = 0;
    int32_t levels = 0;
    int64_t nodes = 0;
    int32_t* idx = nullptr;  // [n] tree position -> caller index (idx_array)
    int32_t* pos = nullptr;  // [n] caller index -> tree position
    float* box = nullptr;    // [nodes][2][d] lower then upper corner (node_bounds)
};

struct RefTreeView {
    int64_t n, nodes;
    int32_t d;
    const int32_t* __restrict__ pos;
    const float* __restrict__ box;
};
inline RefTreeView view_of(const RefTree& t) {
    return RefTreeView{t.n, t.nodes, t.d, t.pos, t.box};
}

// numba_kdtree.py:486 n_levels for leaf_size 40.
int ref_tree_levels(int64_t n);
// Builds the tree of the index's points; `ws` owns idx, pos and box.
int ref_tree_build(Workspace& ws, const fhg_index& ix, RefTree* out);
// Copies the tree out in the reference's layout: idx_array [n] and
// node_bounds [2][nodes][d] (either may be null).
int ref_tree_export(const RefTree& t, int32_t* idx_array, float* node_bounds, cudaStream_t s);

// numba_kdtree.py:765 parallel_tree_query(tree, data, k) for every point, as
// the reference computes it: its depth-first walk of this tree, its max-heap
// of k (squared distance, index) entries and its heap sort, so that equal
// distances come out in the reference's order.  With sqrt_order the sort
// runs on the square roots (the query without output_rdist, boruvka.py:567).
// d_s / s_s hold the engine's lists (Morton-order rows of kk = min(k, n)
// squared distances and Morton positions, (distance, index) order) and tie
// (nullable) its flags of a point outside the list at the k-th distance; the
// rows that can differ from the reference's -- equal distances inside, or a
// tie at the k-th -- are recomputed by the reference's query and written
// over, with columns 1.. of the caller-order neighbour matrix nbr_o
// (nullable, nbr_cols columns).  k <= 64, d <= 32.
int ref_knn(const RefTree& t, const fhg_index& ix, int k, bool sqrt_order, const int8_t* tie,
            float* d_s, int32_t* s_s, int32_t* nbr_o, int nbr_cols, cudaStream_t s);

// numba_kdtree.py:549 point_to_node_lower_bound_rdist of node v's box, in
// the reference's float32 operation order.
__device__ __forceinline__ float ref_node_lb(const RefTreeView& t, int64_t v, const float* q) {
    const float* b = t.box + v * 2 * t.d;
    float r = 0.0f;
    for (int j = 0; j < t.d; ++j) {
        const float lo = b[j], hi = b[t.d + j];
        const float dlo = lo > q[j] ? __fsub_rn(lo, q[j]) : 0.0f;
        const float dhi = q[j] > hi ? __fsub_rn(q[j], hi) : 0.0f;
        const float dd = __fadd_rn(dlo, dhi);
        r = __fadd_rn(r, __fmul_rn(dd, dd));
    }
    return r;
}

// True when the reference's depth-first walk for the query point q meets
// tree position pa before tree position pb (boruvka.py:222-285: at every
// internal node the child of smaller box bound first, the left one on
// equal bounds; inside a leaf, tree order).  Both paths go down from the
// root until they part; the node where they part decides.
__device__ __forceinline__ bool ref_before(const RefTreeView& t, const float* q, int64_t pa,
                                           int64_t pb) {
    int64_t v = 0, s = 0, e = t.n;
    while (2 * v + 1 < t.nodes && e - s >= 2) {
        const int64_t mid = s + (e - s) / 2;
        const bool ra = pa >= mid, rb = pb >= mid;
        if (ra != rb) {
            const bool left_first = ref_node_lb(t, 2 * v + 1, q) <= ref_node_lb(t, 2 * v + 2, q);
            return ra ? !left_first : left_first;
        }
        v = 2 * v + 1 + (ra ? 1 : 0);
        if (ra) s = mid;
        else e = mid;
    }
    return pa < pb;
}

}  // namespace fhg
