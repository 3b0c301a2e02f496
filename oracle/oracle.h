/*
 * CPU oracle for the fast_hdbscan fit path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithm (fast_hdbscan 0.3.2,
 * Python + Numba), statement for statement, used by the tests as the checker
 * for the CUDA engine and by the benchmark as the timed CPU baseline.  It is
 * never linked into, or called by, the product library.
 *
 * Two tie-breaking modes:
 *   mode 0 ("reference"): exactly the reference's tie behaviour with its
 *          parallel loops run sequentially (first-found-wins in KD-tree
 *          traversal order, lowest point index wins inside a component).
 *          Pinned bit-for-bit against fixtures produced by the reference.
 *   mode 1 ("canonical"): every tie is broken by a total order on point
 *          indices -- kNN by (distance, index), a point's Boruvka candidate by
 *          (weight, index), a component's edge by (weight, min idx, max idx).
 *          The result does not depend on the spatial index, and is what the
 *          GPU engine reproduces bit for bit.
 *   mode 2 ("reference, parallel"): mode 0's result, computed with the
 *          parallel loops running in parallel and deterministically.  In the
 *          sequential reference a component's edge comes from its
 *          lowest-index point attaining the component minimum w, and that
 *          point's search is never cut short by the shared bound (the bound
 *          only ever holds weights above w when it runs), so its candidate is
 *          the first point at weight w in its KD-tree traversal.  Mode 2
 *          therefore searches every point with a private bound and merges as
 *          mode 0 does; the tests check it against mode 0 run on one thread.
 * On tie-free input all modes give the same core distances and the same MST
 * weight multiset; they can differ only in which of several equal-weight MST
 * edges is kept.
 */
#ifndef FHG_ORACLE_H
#define FHG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_kdtree orc_kdtree;

/* numba_kdtree.py:478 build_kdtree */
orc_kdtree* orc_build_kdtree(const float* X, int64_t n, int64_t d, int64_t leaf_size);
void orc_free_kdtree(orc_kdtree* t);
int64_t orc_kdtree_n_nodes(const orc_kdtree* t);
void orc_kdtree_arrays(const orc_kdtree* t, int64_t* idx_array, int64_t* idx_start,
                       int64_t* idx_end, uint8_t* is_leaf, float* node_bounds);

/* numba_kdtree.py:765 parallel_tree_query(tree, tree.data, k, output_rdist=True) */
void orc_tree_query(const orc_kdtree* t, int64_t k, int mode, int nthreads,
                    float* rdist, int32_t* idx);

/* boruvka.py:542 parallel_boruvka: returns number of edges written to
 * edges[(n-1)*3] (src, dst, sqrt weight), neighbors[n*ms], core[n]. */
/* weights: NULL, or sample weights (caller order) with wk = the reference's
 * weighted kNN k (boruvka.py:561-563) */
int64_t orc_parallel_boruvka(const orc_kdtree* t, int64_t min_samples, int mode,
                             int nthreads, const float* weights, int64_t wk, double* edges,
                             int32_t* neighbors, float* core, int64_t* n_rounds);

/* hdbscan.py:511 lexsort by (weight, src, dst) */
void orc_sort_mst(const double* mst, int64_t m, double* out);
/* cluster_trees.py:65 mst_to_linkage_tree */
void orc_mst_to_linkage_tree(const double* sorted_mst, int64_t m, double* out);
/* cluster_trees.py:98 mst_to_linkage_tree_w_sample_weights */
void orc_mst_to_linkage_tree_w(const double* sorted_mst, int64_t m, const float* w, double* out);
/* cluster_trees.py:205 condense_tree; returns number of rows.  Buffers must
 * hold 2*m rows. */
int64_t orc_condense_tree(const double* linkage, int64_t m, int64_t min_cluster_size,
                          double max_cluster_size, const float* weights, int64_t* parent,
                          int64_t* child,
                          float* lambda_val, float* child_size);
/* cluster_trees.py:774 simplify_hierarchy (in place); returns kept rows */
int64_t orc_simplify_hierarchy(int64_t* parent, int64_t* child, float* lambda_val,
                               float* child_size, int64_t rows, double threshold);
/* cluster_trees.py:724 extract_eom_clusters; returns count written to sel */
int64_t orc_extract_eom_clusters(const int64_t* parent, const int64_t* child,
                                 const float* lambda_val, const float* child_size,
                                 int64_t rows, double max_cluster_size,
                                 int allow_single_cluster, int64_t* sel);
/* cluster_trees.py:369 cluster_tree_leaves */
int64_t orc_cluster_tree_leaves(const int64_t* parent, const int64_t* child,
                                const float* child_size, int64_t rows, int64_t n_points,
                                int64_t* sel);
/* cluster_trees.py:834 cluster_epsilon_search */
int64_t orc_cluster_epsilon_search(const int64_t* parent, const int64_t* child,
                                   const float* lambda_val, const float* child_size,
                                   int64_t rows, const int64_t* clusters, int64_t n_clusters,
                                   double min_epsilon, int64_t* out);
/* cluster_trees.py:944 get_cluster_label_vector; returns 0, or -1 where the
 * reference would raise (a KeyError on an unselected root cluster). */
int orc_get_cluster_label_vector(const int64_t* parent, const int64_t* child,
                                 const float* lambda_val, int64_t rows,
                                 const int64_t* clusters, int64_t n_clusters,
                                 double epsilon, int64_t n_samples, int64_t* labels);
/* cluster_trees.py:1011 get_point_membership_strength_vector */
void orc_get_point_membership_strength_vector(const int64_t* parent, const int64_t* child,
                                              const float* lambda_val,
                                              const float* child_size, int64_t rows,
                                              const int64_t* clusters, int64_t n_clusters,
                                              const int64_t* labels, int64_t n_samples,
                                              float* probs);
/* cluster_trees.py:906 get_cluster_labelling_at_cut */
void orc_get_cluster_labelling_at_cut(const double* linkage, int64_t m, double cut,
                                      int64_t min_cluster_size, int64_t* out);

/* kruskal.py:950 _kruskal_mst_knn without cannot-link constraints, on kNN
 * lists (rdist, idx: n x kq, the point itself first, as orc_tree_query
 * returns them).  weights NULL: core = sqrt(rdist[:, min_samples]) in float64
 * (0 when min_samples <= 1) and edge lengths sqrt(rdist) in float64; weights
 * given: the weighted core (boruvka.py:528) and float32 sqrt lengths, widened.
 * Writes the MST edges (src, dst, weight; +inf bridges join the components of
 * a disconnected kNN graph) and core[n]; returns the edge count (n - 1). */
int64_t orc_kruskal_knn(const float* rdist, const int32_t* idx, int64_t n, int64_t kq,
                        int64_t min_samples, const float* weights, double* edges,
                        double* core);

/* precomputed.py:479 compute_mst_from_precomputed_sparse_kruskal without
 * cannot-link constraints, on a COO graph (rows, cols, float64 data; the
 * reference's X.tocoo()): the min-symmetrised graph without its diagonal,
 * core distances = the min_samples-th smallest weight of a row (rows ordered
 * by weight, ties by position), float64 mutual-reachability weights, Kruskal
 * with +inf bridges.  neighbors: n x max(1, min_samples) (-1 padded).
 * Returns the edge count (n - 1). */
int64_t orc_precomputed_kruskal(const int32_t* rows, const int32_t* cols, const double* data,
                                int64_t nnz, int64_t n, int64_t min_samples, double* edges,
                                int32_t* neighbors, double* core);

#ifdef __cplusplus
}
#endif
#endif
