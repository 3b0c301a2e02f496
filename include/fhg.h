/*
 * fhg.h -- C ABI of the GB300-native HDBSCAN engine (libfhg.so, sm_103a).
 *
 * The reference (fast_hdbscan 0.3.2) is a Python + Numba library; its
 * "plugin API" is the Python signatures of the functions on the fit path.
 * Each entry point below replaces one of those functions (cited as
 * reference-file:line).  A Python binding (ctypes) or any other FFI passes
 * plain device pointers, sizes and a cudaStream_t given as void*.
 *
 * Conventions
 *   - All array arguments named *_dev are device pointers; *_host are host.
 *   - Indices of points are positions in the caller's input (the reference's
 *     numbering), never an internal permutation.
 *   - Every call is stream-ordered on `stream` (NULL = legacy default stream)
 *     and returns an FHG_* status; FHG_OK = 0.  fhg_last_error() returns a
 *     message for the calling thread's last failure.
 *   - A size or count of zero is an empty input, not an error; a negative
 *     one, or a null pointer where data is needed, is FHG_ERR_INVALID,
 *     reported before any CUDA call.
 *   - Scratch memory is taken with cudaMallocAsync on `stream` and released
 *     on the same stream before the call returns.
 *   - Ties are broken by a total order on point indices by default: kNN
 *     lists by (distance, index); a Boruvka component's outgoing edge by
 *     (weight, min endpoint, max endpoint).  On tie-free input this yields the
 *     reference's core distances, kNN lists and MST weight multiset exactly;
 *     fhg_set_tie_rule(FHG_TIES_REFERENCE) makes the Boruvka edge choices the
 *     reference's own as well.
 */
#ifndef FHG_H
#define FHG_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FHG_OK 0
#define FHG_ERR_INVALID 1        /* bad argument (maps to ValueError)            */
#define FHG_ERR_OOM 2            /* device allocation failed                     */
#define FHG_ERR_CUDA 3           /* a CUDA runtime call failed                   */
#define FHG_ERR_NO_CONVERGENCE 4 /* a bounded device loop hit its iteration cap  */
#define FHG_ERR_UNSUPPORTED 5    /* valid but not implemented (NotImplementedError) */

/* Message for the calling thread's most recent failure ("" if none). */
const char* fhg_last_error(void);
/* ABI version of this library (bumped when a signature changes). */
int fhg_abi_version(void);

/* Tracing (no counterpart in the reference, whose benchmark harness times
 * whole calls with perf_counter).  fhg_launch_count: kernels launched by this
 * library since load.  fhg_profile_enable(1): every stage records a pair of
 * CUDA events on its stream, and counters add their values (for instance
 * "boruvka_components": the component count at the start of every Boruvka
 * round).  fhg_profile_report: waits for those events and writes
 * {"stage": [total_ms, count], "counter": [sum, samples], ...} as JSON into
 * buf, then clears them. */
uint64_t fhg_launch_count(void);
int fhg_profile_enable(int on);
int fhg_profile_report(char* buf, int64_t cap);

/* Boruvka tie rule of the calling host thread, for every later call from that
 * thread (returns the previous rule).  Replaces the `reproducible` flag of
 * boruvka.py:557 parallel_boruvka (hdbscan.py:343, :658):
 *   FHG_TIES_CANONICAL (default): among equal mutual-reachability weights, a
 *     total order on point indices -- a component's edge by (weight, min
 *     endpoint, max endpoint).  The result does not depend on any thread
 *     count or index layout.
 *   FHG_TIES_REFERENCE: the reference's own choices, as its loops make them
 *     when run in order: a component's edge comes from its point of lowest
 *     index that attains the component's least weight, and goes to the first
 *     point of that weight met by the depth-first walk of the reference's
 *     KD-tree (built exactly, on the GPU, for this); edges that would close a
 *     cycle are skipped in the reference's component order; kNN rows with
 *     equal distances are listed as the reference's own query and heap list
 *     them.  This reproduces the reference's MST, neighbour matrix, labels
 *     and probabilities exactly, duplicates included.  It adds the tree
 *     build, the re-query of tied kNN rows and one short walk per component
 *     and round. */
#define FHG_TIES_CANONICAL 0
#define FHG_TIES_REFERENCE 1
int fhg_set_tie_rule(int rule);

/* Device scratch comes from one stream-ordered memory pool per device, owned
 * by this library, that keeps freed blocks cached for the next call (no
 * counterpart in the reference, which allocates host memory through numpy).
 * fhg_release_cached_memory returns every cached block that no call is using
 * to the driver. */
int fhg_release_cached_memory(void);

/* Opaque spatial index: points sorted along a Morton curve into buckets of
 * 32 with a complete binary tree of bounding boxes over the buckets. */
typedef struct fhg_index fhg_index;

/* Replaces numba_kdtree.py:478 build_kdtree(data, leaf_size=40).
 * X_dev: n x d float32, row-major, caller order.  1 <= d <= 32. */
int fhg_index_build(const float* X_dev, int64_t n, int32_t d, void* stream, fhg_index** out);
/* numba_kdtree.py:478 build_kdtree(data, leaf_size=40) exactly: the
 * reference's own median-split KD-tree, every introselect partition
 * reproduced (GPU), for the reference tie mode (fhg_set_tie_rule) and for
 * callers that need the reference's arrays.  X_dev: n x d float32 (1 <= d <=
 * 32); levels = fhg_reference_kdtree_levels(n), nodes = 2^levels - 1.
 *   idx_array_dev   n int32 (the reference's idx_array; nullable)
 *   node_bounds_dev 2 x nodes x d float32 (node_bounds: lower corners, then
 *                   upper corners; nullable)
 * idx_start, idx_end and is_leaf follow from n alone (each node's range is
 * halved, the left child taking the smaller half). */
int32_t fhg_reference_kdtree_levels(int64_t n);
int fhg_reference_kdtree(const float* X_dev, int64_t n, int32_t d, int32_t* idx_array_dev,
                         float* node_bounds_dev, void* stream);

/* Releases an index built by fhg_index_build. */
int fhg_index_free(fhg_index* index, void* stream);
/* Number of points and dimensions of an index. */
int fhg_index_shape(const fhg_index* index, int64_t* n, int32_t* d);

/* Replaces numba_kdtree.py:765 parallel_tree_query(tree, tree.data, k,
 * output_rdist=True): for every point its k nearest points (itself included)
 * by squared float32 distance, ascending.  rdist_dev: n x k float32,
 * idx_dev: n x k int32, rows in caller order.  1 <= k <= 2048 (lists longer
 * than 64 are kept in shared memory, a warp per query); entries past the
 * n-th neighbour are (+inf, -1). */
int fhg_index_knn(fhg_index* index, int32_t k, float* rdist_dev, int32_t* idx_dev,
                  void* stream);

/* Replaces boruvka.py:542 parallel_boruvka(tree, n_threads, min_samples,
 * sample_weights, reproducible): the minimum spanning tree of the
 * mutual-reachability graph.  The result does not depend on any thread
 * count; among equal weights it makes the choices of the calling thread's
 * tie rule (fhg_set_tie_rule: a total order on indices, or the reference's
 * own choices -- its `reproducible` flag in this library).
 *   sample_weights_dev NULL, or n float32 weights (caller order): the
 *                 reference's weighted path (boruvka.py:561-573), which queries
 *                 k = weighted_k = int(2 * min_samples / mean weight)
 *                 neighbours and takes sample_weight_core_distance (:527).
 *   edges_dev     (n-1) x 3 float64: src, dst, sqrt(weight), in Boruvka order
 *                 (round by round; within a round by each component's lowest
 *                 point index), src inside the component that chose the edge.
 *   neighbors_dev n x (k-1) int32: kNN without the point itself
 *                 (neighbors[:, 1:]; k = min_samples + 1, at least 2, or
 *                 weighted_k).  min(k, n) <= 2048 (64 in the reference tie
 *                 mode), else FHG_ERR_UNSUPPORTED; the same holds for every
 *                 Boruvka fit entry point.
 *   core_dev      n float32: sqrt of the core value (boruvka.py:647).
 *   n_rounds_host optional: Boruvka rounds after the kNN-seeded round. */
int fhg_index_boruvka(fhg_index* index, int32_t min_samples, const float* sample_weights_dev,
                      int32_t weighted_k, double* edges_dev, int32_t* neighbors_dev,
                      float* core_dev, int32_t* n_rounds_host, void* stream);

/* Replaces kruskal.py:821 kruskal_mst_from_feature_matrix(tree, min_samples,
 * knn_k=<int>, sample_weights) without cannot-link constraints
 * (kruskal.py:950 _kruskal_mst_knn; the algorithm="kruskal" back-end of
 * hdbscan.py:470): the minimum spanning forest of the mutual-reachability
 * edges of every point's kNN list, in Kruskal's acceptance order (float64
 * weight, then edge position: point-major, neighbour order), followed by +inf
 * bridges between consecutive component representatives (the smallest point
 * of each component) when the kNN graph is disconnected.
 *   query_k       kNN query size, the point itself included, as the
 *                 reference computes it: max(knn_k, min_samples) + 1
 *                 (knn_k + 1 when min_samples == 1; with sample weights
 *                 max(knn_k, int(2 * min_samples / float(np.mean(w)))) + 1).
 *                 2 <= query_k <= 2048.
 *   sample_weights_dev NULL, or n float32 weights: the weighted core
 *                 distance (boruvka.py:528) and float32 edge lengths.
 *   edges_dev     (n-1) x 3 float64: src, dst, weight.
 *   neighbors_dev optional, n x cols int32: cols = query_k - 1 with weights,
 *                 else min_samples (1 when min_samples == 1).
 *   core_dev      n float64 core distances.
 *   n_components_host optional: components of the kNN graph. */
int fhg_index_kruskal_knn(fhg_index* index, int32_t min_samples, int32_t query_k,
                          const float* sample_weights_dev, double* edges_dev,
                          int32_t* neighbors_dev, double* core_dev, int64_t* n_components_host,
                          void* stream);

/* Replaces precomputed.py:479 compute_mst_from_precomputed_sparse_kruskal
 * (algorithm 1) and :410 compute_mst_from_precomputed_sparse (algorithm 0),
 * without cannot-link constraints: the metric="precomputed" back-ends of
 * hdbscan.py:427.  Input: a sparse graph as COO entries (the reference's
 * X.tocoo(); finite, non-negative float64 weights; duplicates and the
 * diagonal allowed).  The graph is symmetrised by the least weight per pair
 * without its diagonal, core distances are the min_samples-th smallest
 * weight of each row, and the minimum spanning forest of the float64
 * mutual-reachability weights comes in Kruskal's acceptance order (weight,
 * then position in the symmetrised CSR), followed by +inf bridges between
 * consecutive component representatives (each component's smallest point).
 * Both algorithms return that forest: the reference's Boruvka finds a forest
 * of the same weights whose equal-weight choices and order are its own.
 *   edges_dev      (n-1) x 3 float64 (src, dst, weight)
 *   neighbors_dev  n x max(1, min_samples) int32, -1 where a row is short
 *   core_dev       n float64 (+inf for rows shorter than min_samples)
 *   n_components_host optional: components of the graph. */
int fhg_precomputed_mst(const int32_t* rows_dev, const int32_t* cols_dev, const double* data_dev,
                        int64_t nnz, int64_t n, int32_t min_samples, int32_t algorithm,
                        double* edges_dev, int32_t* neighbors_dev, double* core_dev,
                        int64_t* n_components_host, void* stream);

/* hdbscan.py:497 clusters_from_spanning_tree (unsupervised) in one call:
 * the tree of n points given as n - 1 float64 rows (src, dst, weight) in any
 * order is sorted by (weight, src, dst), turned into its linkage tree
 * (sample_weights_dev: n float32 or NULL, as fhg_mst_to_linkage_tree),
 * condensed with min_cluster_size, simplified with persistence > 0, and its
 * clusters selected (selection_method 0 = eom with max_cluster_size and
 * allow_single_cluster, 1 = leaf; epsilon > 0: cluster_epsilon_search), then
 * every point labelled with its membership strength.  Outputs as
 * fhg_hdbscan_fit: labels (int64), probabilities (float32), the sorted tree
 * (n - 1 x 3 float64, nullable), the linkage tree (n - 1 x 4 float64,
 * nullable), the condensed tree (capacity 2n rows, *ct_rows_host written),
 * the selected clusters.  n >= 2; the endpoint precondition of
 * fhg_mst_to_linkage_tree applies. */
int fhg_clusters_from_mst(const double* mst_dev, int64_t n, int64_t min_cluster_size,
                          int32_t selection_method, double max_cluster_size,
                          int allow_single_cluster, double epsilon, double persistence,
                          const float* sample_weights_dev, int64_t* labels_dev, float* probs_dev,
                          double* sorted_mst_dev, double* linkage_dev, int64_t* ct_parent_dev,
                          int64_t* ct_child_dev, float* ct_lambda_dev, float* ct_size_dev,
                          int64_t* ct_rows_host, int64_t* selected_dev,
                          int64_t* n_selected_host, void* stream);

/* Replaces the np.lexsort((mst[:,1], mst[:,0], mst[:,2])) of hdbscan.py:511:
 * rows of an m x 3 float64 edge list ordered by (weight, src, dst). */
int fhg_sort_mst(const double* mst_dev, int64_t m, double* sorted_dev, void* stream);

/* Replaces cluster_trees.py:65 mst_to_linkage_tree(sorted_mst) and, with
 * sample_weights_dev (m + 1 float32, else NULL), :98
 * mst_to_linkage_tree_w_sample_weights: m x 4 float64 rows
 * [max(root_l, root_r), min(root_l, root_r), weight, size], size = points
 * (or the float32 sum of their weights) under the merge.
 * Precondition (as in the reference): the rows form a spanning tree of the
 * points 0..m, so every endpoint is an integer in [0, m].  Endpoints outside
 * that range are clamped into it (no memory outside the call's buffers is
 * touched) and the resulting tree is meaningless. */
int fhg_mst_to_linkage_tree(const double* sorted_mst_dev, int64_t m,
                            const float* sample_weights_dev, double* linkage_dev, void* stream);

/* Same result as fhg_mst_to_linkage_tree, with no device allocation at all.
 * No counterpart in the reference: this entry point exists for callers that
 * cannot allocate device memory while they run -- a process whose HBM is
 * reserved up front by its own pool allocator, or a latency-critical loop
 * that must never enter the CUDA allocator.  All scratch comes from a fixed
 * device array compiled into libfhg.so (about 6.8 MB for the limit below),
 * which every GPU that loads the library holds until the process exits.
 *   - m must not exceed FHG_NOALLOC_MAX_EDGES; larger inputs are rejected
 *     with FHG_ERR_INVALID (use fhg_mst_to_linkage_tree instead).
 *   - The same endpoint precondition as fhg_mst_to_linkage_tree: every
 *     endpoint in [0, m]; others are clamped into range.
 *   - The first call on each device looks up the array's device address
 *     (cudaGetSymbolAddress, with that device current); make that first call
 *     before any stream capture.  The address is cached per device for the
 *     life of the process: after cudaDeviceReset (or anything else that
 *     tears down and recreates the device's primary context) the cache is
 *     stale, so do not call this entry point again in that process.
 *   - Every call shares the one array: calls that overlap on the GPU (for
 *     instance on two streams) race and corrupt each other's results.  Each
 *     call initialises what it reads, so back-to-back calls are safe. */
#define FHG_NOALLOC_MAX_EDGES 65536
int fhg_mst_to_linkage_tree_noalloc(const double* sorted_mst_dev, int64_t m,
                                    double* linkage_dev, void* stream);

/* Replaces cluster_trees.py:205 condense_tree(hierarchy, min_cluster_size,
 * max_cluster_size, sample_weights) (sample_weights_dev: m + 1 float32, or
 * NULL for unit weights; with weights the hierarchy's size column holds weight
 * sums, as mst_to_linkage_tree_w_sample_weights writes it).  Output buffers
 * hold 2*m rows; *n_rows_host receives the row count.  Rows come in the
 * reference's order. */
int fhg_condense_tree(const double* linkage_dev, int64_t m, int64_t min_cluster_size,
                      double max_cluster_size, const float* sample_weights_dev,
                      int64_t* parent_dev, int64_t* child_dev, float* lambda_dev,
                      float* child_size_dev, int64_t* n_rows_host, void* stream);

/* Replaces cluster_trees.py:724 extract_eom_clusters(condensed_tree,
 * cluster_tree, max_cluster_size, allow_single_cluster).  sel_dev holds up
 * to `rows` ids; *n_sel_host receives the count (reference order). */
int fhg_extract_eom_clusters(const int64_t* parent_dev, const int64_t* child_dev,
                             const float* lambda_dev, const float* child_size_dev,
                             int64_t rows, double max_cluster_size, int allow_single_cluster,
                             int64_t* sel_dev, int64_t* n_sel_host, void* stream);

/* Replaces cluster_trees.py:944 get_cluster_label_vector and :1011
 * get_point_membership_strength_vector (cluster_selection_epsilon as given). */
int fhg_label_points(const int64_t* parent_dev, const int64_t* child_dev,
                     const float* lambda_dev, const float* child_size_dev, int64_t rows,
                     const int64_t* sel_dev, int64_t n_sel, double epsilon, int64_t n_samples,
                     int64_t* labels_dev, float* probs_dev, void* stream);

/* Replaces cluster_trees.py:369 cluster_tree_leaves(cluster_tree, n_points)
 * applied to cluster_tree_from_condensed_tree (:672) of the given rows:
 * leaf clusters in increasing id order.  sel_dev holds up to `rows` ids. */
int fhg_cluster_tree_leaves(const int64_t* parent_dev, const int64_t* child_dev,
                            const float* lambda_dev, const float* child_size_dev, int64_t rows,
                            int64_t* sel_dev, int64_t* n_sel_host, void* stream);

/* Replaces cluster_trees.py:1011 get_point_membership_strength_vector(tree,
 * clusters, labels) for caller-given labels (int64[n_samples]). */
int fhg_membership_strengths(const int64_t* parent_dev, const int64_t* child_dev,
                             const float* lambda_dev, const float* child_size_dev, int64_t rows,
                             const int64_t* sel_dev, int64_t n_sel, const int64_t* labels_dev,
                             int64_t n_samples, float* probs_dev, void* stream);

/* Replaces hdbscan.py:93 to_numpy_rec_array(condensed_tree) (called by
 * HDBSCAN.fit, hdbscan.py:805): rows x 28 bytes at records_dev (4-byte
 * aligned), numpy's packed layout of the dtype [("parent", intp),
 * ("child", intp), ("lambda_val", float64), ("child_size", float32)]. */
int fhg_condensed_record_array(const int64_t* parent_dev, const int64_t* child_dev,
                               const float* lambda_dev, const float* child_size_dev,
                               int64_t rows, void* records_dev, void* stream);

/* Replaces cluster_trees.py:774 simplify_hierarchy(condensed_tree,
 * persistence_threshold).  Like the reference, relabels the rows it keeps in
 * the input arrays in place; the simplified tree (kept rows, in order) goes
 * to out_* (room for `rows` rows), *out_rows_host receives its row count. */
int fhg_simplify_hierarchy(int64_t* parent_dev, int64_t* child_dev, float* lambda_dev,
                           const float* child_size_dev, int64_t rows, double threshold,
                           int64_t* out_parent_dev, int64_t* out_child_dev,
                           float* out_lambda_dev, float* out_child_size_dev,
                           int64_t* out_rows_host, void* stream);

/* Replaces cluster_trees.py:834 cluster_epsilon_search(clusters,
 * cluster_tree, min_epsilon) over the child_size > 1 rows of the given tree.
 * out_dev holds up to n_clusters ids; *n_out_host receives the count. */
int fhg_cluster_epsilon_search(const int64_t* parent_dev, const int64_t* child_dev,
                               const float* lambda_dev, const float* child_size_dev,
                               int64_t rows, const int64_t* clusters_dev, int64_t n_clusters,
                               double min_epsilon, int64_t* out_dev, int64_t* n_out_host,
                               void* stream);

/* Replaces cluster_trees.py:906 get_cluster_labelling_at_cut(linkage_tree,
 * cut, min_cluster_size) (hdbscan.py:824 HDBSCAN.dbscan_clustering):
 * labels_dev receives int64[m + 1] labels, -1 for noise. */
int fhg_labelling_at_cut(const double* linkage_dev, int64_t m, double cut,
                         int64_t min_cluster_size, int64_t* labels_dev, void* stream);

/* Many independent fits (no reference counterpart: the reference runs one
 * fit per call, e.g. sub_clusters.py:75-95 loops over clusters in Python).
 * Instance i is X_dev[i] (n[i] >= 2 points, d[i] <= 8) with min_samples[i],
 * min_cluster_size[i] and the shared selection options; its labels and
 * probabilities go to labels_dev[i] / probs_dev[i] (device pointers; the
 * pointer arrays themselves are host memory), status_host[i] receives its
 * FHG_* status.  n_workers host threads, each with its own stream, run the
 * fused fit on instances taken in order; results equal fhg_hdbscan_fit's.
 * The work follows what is queued on `stream`, which waits for all of it. */
int fhg_hdbscan_fit_batch(int64_t count, const float* const* X_dev, const int64_t* n,
                          const int32_t* d, const int32_t* min_samples,
                          const int64_t* min_cluster_size, int32_t selection_method,
                          double max_cluster_size, int allow_single_cluster,
                          int64_t* const* labels_dev, float* const* probs_dev, int32_t n_workers,
                          int32_t* status_host, void* stream);

/* The whole fit of hdbscan.py:686 HDBSCAN.fit / :199 fast_hdbscan on device
 * data (Euclidean): spatial index, kNN core distances, Boruvka MST and the
 * tree passes (with cluster_selection_persistence and
 * cluster_selection_epsilon as in hdbscan.py:528-559, and sample weights as
 * in fhg_index_boruvka / fhg_mst_to_linkage_tree / fhg_condense_tree), with
 * every intermediate kept in HBM.  The condensed tree returned is the
 * simplified one when persistence > 0; selected_dev receives the final
 * selection.
 *   selection_method: 0 = "eom", 1 = "leaf".
 *   Required outputs: labels_dev (int64[n]), probs_dev (float32[n]).
 *   Optional outputs (NULL to skip): mst_dev ((n-1) x 3 float64, sorted as
 *   in hdbscan.py:511), linkage_dev ((n-1) x 4), ct_* (condensed tree, room
 *   for 2n rows; *ct_rows_host = rows), neighbors_dev (n x (k-1), k as in
 *   fhg_index_boruvka), core_dev (n), selected_dev (room for n ids;
 *   *n_selected_host = count). */
int fhg_hdbscan_fit(const float* X_dev, int64_t n, int32_t d, int32_t min_samples,
                    int64_t min_cluster_size, int32_t selection_method, double max_cluster_size,
                    int allow_single_cluster, double epsilon, double persistence,
                    const float* sample_weights_dev, int32_t weighted_k,
                    int64_t* labels_dev, float* probs_dev, double* mst_dev, double* linkage_dev,
                    int64_t* ct_parent_dev, int64_t* ct_child_dev, float* ct_lambda_dev,
                    float* ct_size_dev, int64_t* ct_rows_host, int32_t* neighbors_dev,
                    float* core_dev, int64_t* selected_dev, int64_t* n_selected_host,
                    void* stream);

/* fhg_hdbscan_fit on the kNN-graph Kruskal MST (hdbscan.py:306 with
 * algorithm="kruskal" and an integer knn_k; the MST as fhg_index_kruskal_knn
 * builds it, then the same tree passes).  query_k as for
 * fhg_index_kruskal_knn; neighbors_dev (optional) takes its columns and
 * core_dev (optional) is float64.  Sample weights (NULL or n float32) enter
 * the core distances, the edge lengths and the tree sizes. */
int fhg_hdbscan_fit_kruskal(const float* X_dev, int64_t n, int32_t d, int32_t min_samples,
                            int32_t knn_k, int32_t query_k, int64_t min_cluster_size,
                            int32_t selection_method, double max_cluster_size,
                            int allow_single_cluster, double epsilon, double persistence,
                            const float* sample_weights_dev, int64_t* labels_dev,
                            float* probs_dev, double* mst_dev, double* linkage_dev,
                            int64_t* ct_parent_dev, int64_t* ct_child_dev,
                            float* ct_lambda_dev, float* ct_size_dev, int64_t* ct_rows_host,
                            int32_t* neighbors_dev, double* core_dev, int64_t* selected_dev,
                            int64_t* n_selected_host, void* stream);

/* The whole fit (hdbscan.py:306) on a precomputed sparse graph
 * (metric="precomputed"): the forest of fhg_precomputed_mst, then the tree
 * passes of fhg_hdbscan_fit.  neighbors_dev (optional, n x max(1,
 * min_samples)) and core_dev (optional, float64) as fhg_precomputed_mst. */
int fhg_hdbscan_fit_precomputed(const int32_t* rows_dev, const int32_t* cols_dev,
                                const double* data_dev, int64_t nnz, int64_t n,
                                int32_t min_samples, int32_t algorithm,
                                int64_t min_cluster_size, int32_t selection_method,
                                double max_cluster_size, int allow_single_cluster,
                                double epsilon, double persistence, int64_t* labels_dev,
                                float* probs_dev, double* mst_dev, double* linkage_dev,
                                int64_t* ct_parent_dev, int64_t* ct_child_dev,
                                float* ct_lambda_dev, float* ct_size_dev, int64_t* ct_rows_host,
                                int32_t* neighbors_dev, double* core_dev, int64_t* selected_dev,
                                int64_t* n_selected_host, void* stream);

/* Candidate kernel of the exact high-dimensional kNN (fhg_highd_knn and the
 * d > 30 fits) for later calls from the calling thread; returns the previous
 * choice.  No counterpart in the reference (its d > 30 route is pynndescent).
 *   FHG_HD_TCGEN05 (default): a Blackwell pipeline -- TMA loads of the
 *     operand tiles into shared memory, tcgen05.mma into tensor-memory
 *     accumulators, candidate selection in the epilogue warps -- for padded
 *     depths of 32 and 64 with k <= 32 (the others fall back);
 *   FHG_HD_MMA_SYNC: the warp-level mma.sync kernel.
 * Both give the same certified kNN. */
#define FHG_HD_TCGEN05 0
#define FHG_HD_MMA_SYNC 1
int fhg_set_highd_kernel(int kernel);

/* Exact kNN of every point of X (n x d float32, 1 <= d <= 96) by brute force:
 * bfloat16 tensor-core candidates (k + 32 per query, from a two-term bf16
 * split of the centred points), re-ranked in exact float32 and certified by
 * a rounding bound; uncertified queries are searched again exactly.  Rows of
 * k (squared distance, index), the point itself included, in (distance,
 * index) order -- fhg_index_knn's output for any d.  k + 32 <= 128.
 * *fallbacks_host (optional) = queries searched again.  Replaces the kNN
 * graph of nndescent.py:41 build_knn_graph (pynndescent, approximate). */
int fhg_highd_knn(const float* X_dev, int64_t n, int32_t d, int32_t k, float* rdist_dev,
                  int32_t* idx_dev, int64_t* fallbacks_host, void* stream);

/* nndescent.py:179 compute_mst_from_knn_graph (the d > 30 route of
 * hdbscan.py:447) on the exact kNN graph of fhg_highd_knn with knn_k
 * neighbours besides the point itself (the caller resolves knn_k: None ->
 * max(3 min_samples, 15), then max(knn_k, min_samples)): float64 core
 * distances (the min_samples-th neighbour; 0 for min_samples 1), neighbours
 * n x min_samples, the Kruskal forest of the mutual-reachability kNN edges
 * with +inf bridges (edges (n-1) x 3 float64).  knn_k <= 63, else
 * FHG_ERR_UNSUPPORTED. */
int fhg_knn_graph_mst(const float* X_dev, int64_t n, int32_t d, int32_t min_samples,
                      int32_t knn_k, double* edges_dev, int32_t* neighbors_dev, double* core_dev,
                      int64_t* n_components_host, void* stream);

/* The whole fit on fhg_knn_graph_mst's forest (hdbscan.py:306 with
 * d > 30 and no sample weights); outputs as fhg_hdbscan_fit_kruskal. */
int fhg_hdbscan_fit_knn_graph(const float* X_dev, int64_t n, int32_t d, int32_t min_samples,
                              int32_t knn_k, int64_t min_cluster_size, int32_t selection_method,
                              double max_cluster_size, int allow_single_cluster, double epsilon,
                              double persistence, int64_t* labels_dev, float* probs_dev,
                              double* mst_dev, double* linkage_dev, int64_t* ct_parent_dev,
                              int64_t* ct_child_dev, float* ct_lambda_dev, float* ct_size_dev,
                              int64_t* ct_rows_host, int32_t* neighbors_dev, double* core_dev,
                              int64_t* selected_dev, int64_t* n_selected_host, void* stream);

/* core_graph.py:198 boruvka_mst: the spanning forest of a cluster's core
 * graph (CSR of n rows, each sorted by float32 weight, ties in insertion
 * order; nnz = indptr[n]) with the reference's choices among equal weights.
 * Several clusters' graphs may share the CSR as disjoint blocks of rows:
 * seg_end_dev (optional, n int32) gives each row the end of its block, and
 * every block evolves as if alone.  Writes *n_edges_host <= n - 1 edges
 * (point, neighbour, weight) float64; each block's edges appear in the
 * reference's order for that block. */
int fhg_core_graph_mst(const int32_t* indptr_dev, const int32_t* indices_dev,
                       const float* weights_dev, const int32_t* seg_end_dev, int64_t n,
                       double* edges_dev, int64_t* n_edges_host, void* stream);

/* sub_clusters.py:132 propagate_labels_per_cluster for many clusters in one
 * launch.  labels_dev: the sub-cluster labels of every cluster's points (any
 * layout; -1 = noise), updated in place.  Cluster c's noise points are
 * noise_pt_dev[noise_first_dev[c] .. noise_first_dev[c+1]) in increasing
 * index order; noise point x's neighbours are adj_other_dev[adj_ptr_dev[x] ..
 * adj_ptr_dev[x+1]) (indices into labels_dev) in the order of the reference's
 * per-point dict, with the inverse weights adj_w_dev (float64).  Each cluster
 * sweeps its noise points in order, giving each the label of largest summed
 * inverse weight among its labelled neighbours (first label wins ties; later
 * points of the same sweep see the new labels), until a sweep labels nothing.
 * Unlike the reference, which loops forever when some noise point cannot be
 * reached, such points stay -1. */
int fhg_propagate_labels(int64_t n_clusters, const int32_t* noise_first_dev,
                         const int32_t* noise_pt_dev, const int32_t* adj_ptr_dev,
                         const int32_t* adj_other_dev, const double* adj_w_dev,
                         int32_t* labels_dev, void* stream);

/* core_graph.py:19 knn_mst_union + :47 flatten_to_csr + :70 sort_by_lens for
 * many clusters at once, as one block CSR of P rows (the clusters' points one
 * cluster after another).  nb_dev: P x k in-cluster neighbour ids (-1: none);
 * lens_dev (float64) and core_dev per row; blk_start/blk_end_dev: the row's
 * cluster block; M MST edges (parent row, child in-cluster id, distance).
 * A row holds its kNN children (each once, in neighbour order) then its MST
 * children not already present (in MST order), stably sorted by weight =
 * float32(max lens); distance = max core for kNN children, else the MST
 * distance.  Outputs: indptr_dev (P + 1), children as in-cluster and as block
 * ids, weights, distances (room for P k + M entries), seg_end_dev (P, the
 * block end, for fhg_core_graph_mst); *nnz_host entries. */
int fhg_core_graphs(int64_t P, int32_t k, const int32_t* nb_dev, const double* lens_dev,
                    const float* core_dev, const int32_t* blk_start_dev,
                    const int32_t* blk_end_dev, int64_t M, const int32_t* mparent_dev,
                    const int32_t* mchild_dev, const double* mdist_dev, int32_t* indptr_dev,
                    int32_t* idx_local_dev, int32_t* idx_block_dev, float* weights_dev,
                    float* distances_dev, int32_t* seg_end_dev, int64_t* nnz_host, void* stream);

/* fhg_hdbscan_fit, with the large outputs also copied to host memory while
 * the fit runs: each non-NULL *_host destination receives its output from a
 * side stream as soon as the fit has finished writing it (neighbours and
 * core distances after the MST, the sorted MST and the linkage tree before
 * the condensed tree is built, the condensed tree's record array before
 * cluster selection), so that the transfers overlap the later stages.  Host
 * destinations should be pinned for the copies to run asynchronously.  On
 * return every copy is ordered before work queued later on `stream`;
 * synchronise the stream before reading the host buffers.
 *   ct_records_dev (room for 2n records of 28 bytes, 4-byte aligned) receives
 *   the condensed tree as the record array HDBSCAN.fit stores (hdbscan.py:93,
 *   fields parent i8, child i8, lambda_val f8, child_size f4, packed), as
 *   fhg_condensed_record_array writes it; it needs the ct_* buffers.
 * Each exported output needs its device buffer (FHG_ERR_INVALID otherwise). */
int fhg_hdbscan_fit_export(const float* X_dev, int64_t n, int32_t d, int32_t min_samples,
                           int64_t min_cluster_size, int32_t selection_method,
                           double max_cluster_size, int allow_single_cluster, double epsilon,
                           double persistence, const float* sample_weights_dev,
                           int32_t weighted_k, int64_t* labels_dev, float* probs_dev,
                           double* mst_dev, double* linkage_dev, int64_t* ct_parent_dev,
                           int64_t* ct_child_dev, float* ct_lambda_dev, float* ct_size_dev,
                           int64_t* ct_rows_host, int32_t* neighbors_dev, float* core_dev,
                           int64_t* selected_dev, int64_t* n_selected_host,
                           int32_t* neighbors_host, float* core_host, double* mst_host,
                           double* linkage_host, void* ct_records_dev, void* ct_records_host,
                           void* stream);

/* ---- Learned kNN search radius (no reference counterpart: a network that
 * proposes each query's search radius for the kNN of core_distances /
 * parallel_tree_query, boruvka.py:561-585; the certified search keeps every
 * kNN output identical to fhg_index_knn's).
 * The model is a float32 block of fhg_radius_param_count() parameters:
 * W1[64][11] b1[64] W2[64][64] b2[64] w3[64] b3 mu[11] sigma[11], the network
 * 11 -> 64 -> 64 -> 1 (ReLU, bfloat16 operands, float32 accumulation) on
 * standardised features, predicting the log core distance. */
int fhg_radius_param_count(void);
/* 11 features per point (caller order, row-major n x 11): the first three
 * coordinates scaled to the bounding box and the log point density of the
 * point's bucket and its 7 ancestor nodes. */
int fhg_radius_features(fhg_index* index, float* feat_dev, void* stream);
/* Training targets: log of every point's k-th neighbour distance (caller
 * order), the point itself counted. */
int fhg_radius_targets(fhg_index* index, int32_t k, float* target_dev, void* stream);
/* Initial parameters: He-normal weights from `seed`, zero biases, b3 = the
 * target mean, mu / sigma the feature means and deviations of the n rows. */
int fhg_radius_init(float* params_dev, const float* feat_dev, const float* target_dev,
                    int64_t n, uint64_t seed, void* stream);
/* Forward pass (tensor-core kernel): log radius of n feature rows. */
int fhg_radius_forward(const float* params_dev, const float* feat_dev, int64_t n,
                       float* log_radius_dev, void* stream);
/* Backward pass over the batch rows_dev[0..batch): grad_dev (the trained
 * parameters, everything before mu) = gradient of the mean squared error,
 * *loss_dev = that error. */
int fhg_radius_backward(const float* params_dev, const float* feat_dev, const float* target_dev,
                        const int32_t* rows_dev, int64_t batch, float* grad_dev, float* loss_dev,
                        void* stream);
/* `steps` Adam steps (learning rate lr) on random batches of `batch` rows;
 * loss_curve_dev (optional, `steps` floats) receives every step's loss. */
int fhg_radius_train(float* params_dev, const float* feat_dev, const float* target_dev,
                     int64_t n, int32_t steps, int32_t batch, float lr, uint64_t seed,
                     float* loss_curve_dev, void* stream);
/* Fits made afterwards by the calling thread search their kNN with this
 * model (radius = exp(prediction) * margin); NULL returns to the plain
 * search.  The parameters must stay alive while in use. */
int fhg_radius_use(const float* params_dev, float margin);
/* Queries the calling thread's last radius search had to search again. */
int fhg_radius_fallbacks(int64_t* count_host, void* stream);
/* fhg_index_knn with the model's radius and the certified fallback: the same
 * outputs; *fallbacks_host (optional) = queries searched again. */
int fhg_index_knn_radius(fhg_index* index, int32_t k, const float* params_dev, float margin,
                         float* rdist_dev, int32_t* idx_dev, int64_t* fallbacks_host,
                         void* stream);
/* Work measure of the kNN of every point: *scans_host = buckets scanned,
 * with the model (params_dev non-NULL) or by the plain search (NULL);
 * *fallbacks_host (optional) = queries searched again. */
int fhg_knn_scan_count(fhg_index* index, int32_t k, const float* params_dev, float margin,
                       int64_t* scans_host, int64_t* fallbacks_host, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FHG_H */
