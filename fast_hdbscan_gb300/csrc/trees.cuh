// Tree passes over the minimum spanning tree: sort, single-linkage tree,
// condensed tree, cluster selection, labels and membership strengths.
#pragma once
#include "fhg_common.cuh"

namespace fhg {

// Single-linkage (Kruskal) tree of a sorted MST.  Node ids: points are
// 0..n-1, the merge made by sorted edge i is node n + i.
struct Linkage {
    int64_t n = 0, m = 0;      // m = n - 1 merges
    int32_t* left = nullptr;   // [m] max(root_l, root_r)  (hierarchy[:, 0])
    int32_t* right = nullptr;  // [m] min(root_l, root_r)  (hierarchy[:, 1])
    double* w = nullptr;       // [m] merge distance       (hierarchy[:, 2])
    int32_t* size = nullptr;   // [2n-1] leaves under every node (points: 1)
    float* wsize = nullptr;    // [2n-1] sample-weight sums, or null (unit weights)
    int32_t* ssrc = nullptr;   // [m] sorted MST src (caller index)
    int32_t* sdst = nullptr;   // [m] sorted MST dst
};

// Sorts MST rows by (weight, src, dst) (hdbscan.py:511) and builds the
// linkage tree (cluster_trees.py:65).  w may be the float64 weight column or,
// when w2 is given instead, the squared float32 weights (sqrt is applied).
int sort_and_link(Workspace& ws, int64_t n, const int32_t* src, const int32_t* dst,
                  const double* w, const float* w2, Linkage* out, bool presorted = false);

// Column views of the reference's float64 arrays.
int split_mst_f64(Workspace& ws, const double* mst, int64_t m, int32_t** src, int32_t** dst,
                  double** w);
int linkage_from_f64(Workspace& ws, const double* lk, int64_t m, Linkage* out);

// Condensed tree rows in the reference's order (cluster_trees.py:205).
// Labels: points 0..n-1, clusters n (root), n+1, ...
struct Condensed {
    int64_t n = 0;
    int64_t rows = 0;
    int64_t n_clusters = 0;      // labels n .. n + n_clusters - 1
    int32_t* parent = nullptr;   // [rows]
    int32_t* child = nullptr;    // [rows]
    float* lambda = nullptr;     // [rows]
    float* csize = nullptr;      // [rows]
};
int condense_tree(Workspace& ws, const Linkage& lk, int64_t min_cluster_size,
                  double max_cluster_size, Condensed* out);
// Internal view of the reference's CondensedTree arrays (int64 labels); the
// number of points is the root label parent[0].
int condensed_from_arrays(Workspace& ws, const int64_t* parent, const int64_t* child,
                          const float* lambda, const float* csize, int64_t rows, Condensed* out);

// The selection-independent part of label_points (row of every point and
// cluster, cluster parents, the root's and every cluster's largest point
// lambda), buffers owned by the Workspace it was computed in.
struct LabelPre {
    bool ready = false;
    int32_t *row_of_point = nullptr, *row_of_cluster = nullptr, *cpar = nullptr;
    float* nsize = nullptr;
    int8_t* in_tree = nullptr;
    unsigned int *root_max = nullptr, *death = nullptr;
};
int label_prework(Workspace& ws, const Condensed& ct, LabelPre* pre);

// Cluster selection.  `sel` receives selected labels in the reference's
// order; *n_sel its count (host).  With `pre`, label_prework runs on the
// stream while the cluster stabilities (a sequential float32 sum per
// cluster) are computed beside it.
int select_eom(Workspace& ws, const Condensed& ct, double max_cluster_size, bool allow_single,
               int32_t* sel, int64_t* n_sel, LabelPre* pre = nullptr);
int select_leaf(Workspace& ws, const Condensed& ct, int32_t* sel, int64_t* n_sel,
                LabelPre* pre = nullptr);

// Labels and membership strengths (cluster_trees.py:944, :1011).  Returns
// FHG_ERR_INVALID where the reference raises a KeyError.  `pre`: the
// label_prework of the same tree, or NULL.
int label_points(Workspace& ws, const Condensed& ct, const int32_t* sel, int64_t n_sel,
                 double epsilon, int64_t* labels, float* probs, const LabelPre* pre = nullptr);
// Membership strengths for given labels (cluster_trees.py:1011).
int membership_strengths(Workspace& ws, const Condensed& ct, const int32_t* sel, int64_t n_sel,
                         const int64_t* labels, float* probs);

// Sample weights (cluster_trees.py:98 mst_to_linkage_tree_w_sample_weights):
// lk.wsize[v] = the weights of the points under v, summed in float64 over a
// preorder numbering and rounded to float32 (the reference sums float32 along
// the merges; the two agree whenever its float32 sums are exact).
int weighted_sizes(Workspace& ws, Linkage& lk, const float* weights);
// Leaf counts (lk.size) of a linkage tree given by its rows only, rebuilt by
// the rank-halving linkage over one representative point per child.
int linkage_leaf_counts(Workspace& ws, Linkage& lk);

// Selection options (cluster_trees.py:774, :834, :906).
// simplify_hierarchy relabels the kept rows of `ct` in place, as the
// reference mutates its argument, and returns the compacted tree in `out`.
int simplify_hierarchy(Workspace& ws, const Condensed& ct, double threshold, Condensed* out);
// The reference's order of the searched selection; out holds up to n_sel.
int epsilon_search(Workspace& ws, const Condensed& ct, const int32_t* sel, int64_t n_sel,
                   double min_epsilon, int32_t* out, int64_t* n_out);
// DBSCAN labels of every point at a cut of the linkage tree.
int labelling_at_cut(Workspace& ws, const Linkage& lk, double cut, int64_t min_cluster_size,
                     int64_t* labels);

// Device-side copies to the reference's dtypes.
int linkage_to_f64(const Linkage& lk, double* out, cudaStream_t s);
int condensed_to_arrays(const Condensed& ct, int64_t* parent, int64_t* child, float* lambda,
                        float* csize, cudaStream_t s);
int sorted_mst_to_f64(const Linkage& lk, double* out, cudaStream_t s);

}  // namespace fhg
