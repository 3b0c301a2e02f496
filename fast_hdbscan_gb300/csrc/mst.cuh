// Minimum spanning tree of the mutual-reachability graph (Boruvka).
#pragma once
#include "index.cuh"

namespace fhg {

// Device outputs of a Boruvka run, all in caller order / caller indices.
struct MstResult {
    int64_t m = 0;               // edges written (n - 1 for a connected input)
    int32_t rounds = 0;          // Boruvka rounds after the kNN-seeded round
    int32_t* src = nullptr;      // [n-1] caller index inside the choosing component
    int32_t* dst = nullptr;      // [n-1]
    float* w2 = nullptr;         // [n-1] squared mutual-reachability weight
};

// Runs kNN (k = min_samples + 1, or 2 when min_samples <= 1) and Boruvka.
// With sample weights (caller order, nullable) the reference's weighted path:
// k = weighted_k = int(2 * min_samples / mean weight), weighted core
// distances, round 0 on plain distances (boruvka.py:561-573).
// `ws` owns every returned buffer.  Optional outputs (nullable):
//   core_o  [n]       sqrt core distance, caller order
//   nbr_o   [n*(k-1)] neighbours without the point itself, caller order
// The edge list comes in the reference's order (the round-0 edges by caller
// index of the choosing point, then every round's by component); with
// any_order the round-0 edges come in index order instead, for callers that
// sort the edges anyway.
// kNN-graph Kruskal MST (kruskal.py:950): query_k nearest points per point
// (itself included), float64 mutual-reachability weights, the minimum
// spanning forest in Kruskal's acceptance order followed by +inf bridges.
// edges: (n-1) x 3 float64; neighbors (nullable): n x cols (query_k - 1
// with weights, else max(min_samples, 1)); core: n float64.
int kruskal_knn_mst(const fhg_index& index, int min_samples, int query_k, const float* weights,
                    double* edges, int32_t* neighbors, double* core, int64_t* n_components,
                    cudaStream_t s);
// Spanning forest of a core graph (CSR, rows sorted by weight) with the
// reference's Boruvka choices (core_graph.py:198): edges (p, neighbour,
// weight) float64 in the reference's order; *n_edges of them.
// seg_end (nullable): per row, the end of its graph's block of rows, when
// several disjoint graphs share the CSR (each then evolves as alone).
int core_graph_boruvka(int64_t n, const int32_t* indptr, const int32_t* indices,
                       const float* weights, const int32_t* seg_end, double* edges,
                       int64_t* n_edges, cudaStream_t s);

// Label propagation to noise points within clusters (sub_clusters.py:132),
// every cluster in one launch; see fhg_propagate_labels in fhg.h.
int propagate_labels(int64_t nclusters, const int32_t* noise_first, const int32_t* noise_pt,
                     const int32_t* adj_ptr, const int32_t* adj_other, const double* adj_w,
                     int32_t* labels, cudaStream_t s);

// Block CSR of many clusters' core graphs (rows = points, cluster after
// cluster): nb (P x k local ids or -1), lens (P, float64), core (P), the
// cluster block [blk_start, blk_end) of every row, M MST edges (parent row,
// child local id, distance).  Outputs indptr (P + 1), per entry the local and
// the block index of the child, weight and distance (room for P k + M
// entries), seg_end per row; *nnz entries.
int core_graphs_layout(int64_t P, int k, const int32_t* nb, const double* lens, const float* core,
                       const int32_t* blk_start, const int32_t* blk_end, int64_t M,
                       const int32_t* mparent, const int32_t* mchild, const double* mdist,
                       int32_t* indptr, int32_t* idx_local, int32_t* idx_block, float* w,
                       float* dist, int32_t* seg_end, int64_t* nnz, cudaStream_t s);

// The same on kNN lists from the spatial index (index given) or from the
// brute-force high-dimensional kNN of X (n x d, index NULL) -- the latter is
// nndescent.py:179 compute_mst_from_knn_graph with an exact kNN graph.
int kruskal_mst_of_lists(int64_t n, int min_samples, int query_k, const float* weights,
                         const fhg_index* index, const float* X, int d, double* edges,
                         int32_t* neighbors, double* core, int64_t* n_components,
                         cudaStream_t s);

// The minimum spanning forest of n points over m edges given in rank order
// (strictly increasing weight), in Kruskal's acceptance order, then +inf
// bridges between consecutive component representatives (each component's
// smallest point): (n-1) x 3 float64 rows (src, dst, weight).  Edge r's
// endpoints are uv[r], or -- with uv NULL -- point eid[r] / (kq-1) and its
// kNN column eid[r] % (kq-1) + 1 in the rows ix of kq entries.  Weights: w64
// when given, else the float32 keys key32 (their square roots in float64
// unless key_weighted).
int sorted_forest_edges(Workspace& ws, int64_t n, int64_t m, int kq, const int32_t* eid,
                        const int32_t* ix, const int2* uv, const uint32_t* key32,
                        int key_weighted, double* edges, int64_t* n_components,
                        const double* w64 = nullptr);

// Minimum spanning forest of a precomputed sparse graph given as COO entries
// (precomputed.py:479 / :410; see precomputed.cu): edges (n-1) x 3 float64,
// neighbors n x max(1, min_samples) int32 (-1 padded), core n float64.
int precomputed_mst(const int32_t* rows, const int32_t* cols, const double* data, int64_t nnz,
                    int64_t n, int min_samples, double* edges, int32_t* neighbors, double* core,
                    int64_t* n_components, cudaStream_t s);

// The Boruvka tie rule of the calling host thread: FHG_TIES_CANONICAL (a
// total order on indices) or FHG_TIES_REFERENCE (the reference's own choices,
// from its KD-tree's traversal order).  set_tie_rule returns the old rule.
int tie_rule();
int set_tie_rule(int rule);

int boruvka_mst(Workspace& ws, const fhg_index& ix, int min_samples, MstResult* out,
                float* core_o, int32_t* nbr_o, const float* weights = nullptr,
                int weighted_k = 0, bool any_order = false);

}  // namespace fhg
