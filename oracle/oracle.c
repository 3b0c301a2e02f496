/*
 * CPU oracle for the fast_hdbscan fit path -- TEST INFRASTRUCTURE ONLY.
 * See oracle.h for the two tie-breaking modes.  Every function cites the
 * reference statement it restates (paths relative to the fast_hdbscan repo).
 *
 * Floating point: compiled with -ffp-contract=off so that every float32
 * multiply and add rounds separately, as the reference's arithmetic does when
 * run statement by statement.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct orc_kdtree {
    int64_t n, d, n_nodes;
    float* data;          /* n*d float32 copy (build_kdtree: data.astype(float32)) */
    int64_t* idx_array;   /* n */
    int64_t* idx_start;   /* n_nodes */
    int64_t* idx_end;     /* n_nodes */
    uint8_t* is_leaf;     /* n_nodes */
    float* node_bounds;   /* [2][n_nodes][d]: [0] lower, [1] upper */
};

#define LO(t, node) ((t)->node_bounds + (int64_t)(node) * (t)->d)
#define HI(t, node) ((t)->node_bounds + ((t)->n_nodes + (int64_t)(node)) * (t)->d)
#define ROW(t, i) ((t)->data + (int64_t)(i) * (t)->d)

/* ------------------------------------------------------------------------- */
/* KD-tree build: numba_kdtree.py:67-521                                      */
/* ------------------------------------------------------------------------- */

/* numba_kdtree.py:164 _compare_indices */
static int cmp_idx(const orc_kdtree* t, int64_t axis, int64_t i1, int64_t i2) {
    float v1 = t->data[i1 * t->d + axis], v2 = t->data[i2 * t->d + axis];
    if (v1 < v2) return -1;
    if (v1 > v2) return 1;
    if (i1 < i2) return -1;
    if (i1 > i2) return 1;
    return 0;
}

/* numba_kdtree.py:200 _insertion_sort_indices */
static void insertion_sort(const orc_kdtree* t, int64_t* idx, int64_t axis, int64_t left,
                           int64_t right) {
    for (int64_t i = left + 1; i < right; ++i) {
        int64_t key = idx[i];
        int64_t j = i - 1;
        while (j >= left && cmp_idx(t, axis, idx[j], key) > 0) {
            idx[j + 1] = idx[j];
            --j;
        }
        idx[j + 1] = key;
    }
}

/* numba_kdtree.py:225 _sift_down_indices */
static void sift_down_idx(const orc_kdtree* t, int64_t* idx, int64_t axis, int64_t offset,
                          int64_t start, int64_t end) {
    int64_t root = start;
    while (root * 2 + 1 < end) {
        int64_t child = root * 2 + 1, swap = root;
        if (cmp_idx(t, axis, idx[offset + swap], idx[offset + child]) < 0) swap = child;
        if (child + 1 < end && cmp_idx(t, axis, idx[offset + swap], idx[offset + child + 1]) < 0)
            swap = child + 1;
        if (swap == root) return;
        int64_t tmp = idx[offset + root];
        idx[offset + root] = idx[offset + swap];
        idx[offset + swap] = tmp;
        root = swap;
    }
}

/* numba_kdtree.py:263 _heapsort_indices */
static void heapsort_idx(const orc_kdtree* t, int64_t* idx, int64_t axis, int64_t left,
                         int64_t right) {
    int64_t size = right - left;
    for (int64_t i = size / 2 - 1; i >= 0; --i) sift_down_idx(t, idx, axis, left, i, size);
    for (int64_t i = size - 1; i > 0; --i) {
        int64_t tmp = idx[left];
        idx[left] = idx[left + i];
        idx[left + i] = tmp;
        sift_down_idx(t, idx, axis, left, 0, i);
    }
}

/* numba_kdtree.py:288 _median_of_three_pivot */
static int64_t median3(const orc_kdtree* t, int64_t* idx, int64_t axis, int64_t left,
                       int64_t right) {
    int64_t mid = (left + right - 1) / 2;
    int64_t il = idx[left], im = idx[mid], ir = idx[right - 1], tmp;
    if (cmp_idx(t, axis, il, im) > 0) {
        tmp = idx[left]; idx[left] = idx[mid]; idx[mid] = tmp;
        tmp = il; il = im; im = tmp;
    }
    if (cmp_idx(t, axis, im, ir) > 0) {
        tmp = idx[mid]; idx[mid] = idx[right - 1]; idx[right - 1] = tmp;
        tmp = im; im = ir; ir = tmp;
        if (cmp_idx(t, axis, il, im) > 0) {
            tmp = idx[left]; idx[left] = idx[mid]; idx[mid] = tmp;
        }
    }
    return mid;
}

/* numba_kdtree.py:325 _partition_indices */
static int64_t partition_idx(const orc_kdtree* t, int64_t* idx, int64_t axis, int64_t left,
                             int64_t right, int64_t pivot_idx) {
    int64_t tmp = idx[pivot_idx];
    idx[pivot_idx] = idx[right - 1];
    idx[right - 1] = tmp;
    int64_t pivot_orig = idx[right - 1];
    int64_t i = left, j = right - 2;
    for (;;) {
        while (i <= j && cmp_idx(t, axis, idx[i], pivot_orig) < 0) ++i;
        while (i <= j && cmp_idx(t, axis, idx[j], pivot_orig) >= 0) --j;
        if (i >= j) break;
        tmp = idx[i]; idx[i] = idx[j]; idx[j] = tmp;
        ++i;
        --j;
    }
    tmp = idx[i]; idx[i] = idx[right - 1]; idx[right - 1] = tmp;
    return i;
}

/* numba_kdtree.py:362 _introselect_impl */
static void introselect_impl(const orc_kdtree* t, int64_t* idx, int64_t axis, int64_t left,
                             int64_t right, int64_t nth, int64_t depth_limit) {
    while (right - left > 16) {
        if (depth_limit == 0) {
            heapsort_idx(t, idx, axis, left, right);
            return;
        }
        --depth_limit;
        int64_t pivot = median3(t, idx, axis, left, right);
        int64_t pos = partition_idx(t, idx, axis, left, right, pivot);
        if (nth < pos) right = pos;
        else if (nth > pos) left = pos + 1;
        else return;
    }
    insertion_sort(t, idx, axis, left, right);
}

/* numba_kdtree.py:398 _introselect */
static void introselect(const orc_kdtree* t, int64_t* idx, int64_t axis, int64_t left,
                        int64_t right, int64_t nth) {
    int64_t size = right - left;
    if (size <= 16) {
        insertion_sort(t, idx, axis, left, right);
        return;
    }
    int64_t max_depth = 2 * (int64_t)log2((double)size);
    introselect_impl(t, idx, axis, left, right, nth, max_depth);
}

/* numba_kdtree.py:79 _init_node (bounds only; radius is never read on the path) */
static void init_node(orc_kdtree* t, int64_t node, int64_t s, int64_t e) {
    float* lo = LO(t, node);
    float* hi = HI(t, node);
    for (int64_t j = 0; j < t->d; ++j) {
        lo[j] = INFINITY;
        hi[j] = -INFINITY;
    }
    for (int64_t i = s; i < e; ++i) {
        const float* r = ROW(t, t->idx_array[i]);
        for (int64_t j = 0; j < t->d; ++j) {
            lo[j] = r[j] < lo[j] ? r[j] : lo[j];
            hi[j] = r[j] > hi[j] ? r[j] : hi[j];
        }
    }
    t->idx_start[node] = s;
    t->idx_end[node] = e;
}

/* numba_kdtree.py:122 _find_node_split_dim */
static int64_t split_dim(const orc_kdtree* t, int64_t s, int64_t e) {
    int64_t result = 0;
    float max_spread = 0.0f;
    for (int64_t j = 0; j < t->d; ++j) {
        float mx = t->data[t->idx_array[s] * t->d + j], mn = mx;
        for (int64_t i = s + 1; i < e; ++i) {
            float v = t->data[t->idx_array[i] * t->d + j];
            mx = v > mx ? v : mx;
            mn = v < mn ? v : mn;
        }
        float spread = mx - mn;
        if (spread > max_spread) {
            max_spread = spread;
            result = j;
        }
    }
    return result;
}

/* numba_kdtree.py:410 _recursive_build_tree */
static void build_rec(orc_kdtree* t, int64_t s, int64_t e, int64_t node) {
    int64_t n_mid = (e - s) / 2;
    init_node(t, node, s, e);
    if (2 * node + 1 >= t->n_nodes) {
        t->is_leaf[node] = 1;
    } else if (e - s < 2) {
        t->is_leaf[node] = 1;
    } else {
        t->is_leaf[node] = 0;
        int64_t axis = split_dim(t, s, e);
        introselect(t, t->idx_array, axis, s, e, s + n_mid);
        build_rec(t, s, s + n_mid, 2 * node + 1);
        build_rec(t, s + n_mid, e, 2 * node + 2);
    }
}

/* numba_kdtree.py:478 build_kdtree */
orc_kdtree* orc_build_kdtree(const float* X, int64_t n, int64_t d, int64_t leaf_size) {
    orc_kdtree* t = (orc_kdtree*)calloc(1, sizeof(orc_kdtree));
    t->n = n;
    t->d = d;
    double ratio = (double)(n - 1) / (double)leaf_size;
    int64_t n_levels = (int64_t)(log2(ratio > 1.0 ? ratio : 1.0) + 1.0);
    t->n_nodes = ((int64_t)1 << n_levels) - 1;
    t->data = (float*)malloc(sizeof(float) * (size_t)(n * d > 0 ? n * d : 1));
    memcpy(t->data, X, sizeof(float) * (size_t)(n * d));
    t->idx_array = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) t->idx_array[i] = i;
    t->idx_start = (int64_t*)calloc((size_t)t->n_nodes, sizeof(int64_t));
    t->idx_end = (int64_t*)calloc((size_t)t->n_nodes, sizeof(int64_t));
    t->is_leaf = (uint8_t*)calloc((size_t)t->n_nodes, 1);
    t->node_bounds = (float*)calloc((size_t)(2 * t->n_nodes * d), sizeof(float));
    build_rec(t, 0, n, 0);
    return t;
}

void orc_free_kdtree(orc_kdtree* t) {
    if (!t) return;
    free(t->data);
    free(t->idx_array);
    free(t->idx_start);
    free(t->idx_end);
    free(t->is_leaf);
    free(t->node_bounds);
    free(t);
}

int64_t orc_kdtree_n_nodes(const orc_kdtree* t) { return t->n_nodes; }

void orc_kdtree_arrays(const orc_kdtree* t, int64_t* idx_array, int64_t* idx_start,
                       int64_t* idx_end, uint8_t* is_leaf, float* node_bounds) {
    memcpy(idx_array, t->idx_array, sizeof(int64_t) * (size_t)t->n);
    memcpy(idx_start, t->idx_start, sizeof(int64_t) * (size_t)t->n_nodes);
    memcpy(idx_end, t->idx_end, sizeof(int64_t) * (size_t)t->n_nodes);
    memcpy(is_leaf, t->is_leaf, (size_t)t->n_nodes);
    memcpy(node_bounds, t->node_bounds, sizeof(float) * (size_t)(2 * t->n_nodes * t->d));
}

/* ------------------------------------------------------------------------- */
/* Distances and kNN: numba_kdtree.py:524-792                                 */
/* ------------------------------------------------------------------------- */

/* numba_kdtree.py:524 rdist: float32 sum of float32 squares, in order */
static inline float rdist(const float* x, const float* y, int64_t d) {
    float r = 0.0f;
    for (int64_t i = 0; i < d; ++i) {
        float diff = x[i] - y[i];
        r += diff * diff;
    }
    return r;
}

/* numba_kdtree.py:549 point_to_node_lower_bound_rdist (called with the
 * node's lower bounds as `upper` and its upper bounds as `lower`) */
static inline float node_lb(const orc_kdtree* t, int64_t node, const float* pt) {
    const float* lo = LO(t, node);
    const float* hi = HI(t, node);
    float r = 0.0f;
    for (int64_t i = 0; i < t->d; ++i) {
        float d_lo = lo[i] > pt[i] ? lo[i] - pt[i] : 0.0f;
        float d_hi = pt[i] > hi[i] ? pt[i] - hi[i] : 0.0f;
        float dd = d_lo + d_hi;
        r += dd * dd;
    }
    return r;
}

/* (distance, index) ordering.  Mode 0 compares distances only, as the
 * reference's heap does; mode 1 breaks ties by index. */
static inline int pair_lt(int mode, float a, int32_t ia, float b, int32_t ib) {
    if (a < b) return 1;
    if (mode && a == b && (uint32_t)ia < (uint32_t)ib) return 1;
    return 0;
}

/* numba_kdtree.py:578 simple_heap_push (max-heap of size k at heap[0]) */
static void heap_push(int mode, float* pri, int32_t* ind, int64_t size, float p, int32_t n) {
    if (!pair_lt(mode, p, n, pri[0], ind[0])) return;
    pri[0] = p;
    ind[0] = n;
    int64_t i = 0, i_swap;
    for (;;) {
        int64_t ic1 = 2 * i + 1, ic2 = ic1 + 1;
        if (ic1 >= size) break;
        else if (ic2 >= size) {
            if (pair_lt(mode, p, n, pri[ic1], ind[ic1])) i_swap = ic1;
            else break;
        } else if (!pair_lt(mode, pri[ic1], ind[ic1], pri[ic2], ind[ic2])) {
            if (pair_lt(mode, p, n, pri[ic1], ind[ic1])) i_swap = ic1;
            else break;
        } else {
            if (pair_lt(mode, p, n, pri[ic2], ind[ic2])) i_swap = ic2;
            else break;
        }
        pri[i] = pri[i_swap];
        ind[i] = ind[i_swap];
        i = i_swap;
    }
    pri[i] = p;
    ind[i] = n;
}

/* numba_kdtree.py:638 siftdown */
static void siftdown(int mode, float* h1, int32_t* h2, int64_t len, int64_t elt) {
    while (elt * 2 + 1 < len) {
        int64_t l = elt * 2 + 1, r = l + 1, swap = elt;
        if (pair_lt(mode, h1[swap], h2[swap], h1[l], h2[l])) swap = l;
        if (r < len && pair_lt(mode, h1[swap], h2[swap], h1[r], h2[r])) swap = r;
        if (swap == elt) break;
        float tf = h1[elt]; h1[elt] = h1[swap]; h1[swap] = tf;
        int32_t ti = h2[elt]; h2[elt] = h2[swap]; h2[swap] = ti;
        elt = swap;
    }
}

/* numba_kdtree.py:667 deheap_sort (one row) */
static void deheap_row(int mode, float* d, int32_t* ix, int64_t k) {
    for (int64_t j = k - 1; j > 0; --j) {
        int32_t ti = ix[0]; ix[0] = ix[j]; ix[j] = ti;
        float tf = d[0]; d[0] = d[j]; d[j] = tf;
        siftdown(mode, d, ix, j, 0);
    }
}

/* numba_kdtree.py:680 tree_query_recursion */
static void query_rec(const orc_kdtree* t, int mode, int64_t node, const float* pt,
                      float* hp, int32_t* hi_, int64_t k, float lb) {
    if (lb > hp[0]) return;
    if (t->is_leaf[node]) {
        for (int64_t i = t->idx_start[node]; i < t->idx_end[node]; ++i) {
            int64_t idx = t->idx_array[i];
            float dd = rdist(pt, ROW(t, idx), t->d);
            if (pair_lt(mode, dd, (int32_t)idx, hp[0], hi_[0]))
                heap_push(mode, hp, hi_, k, dd, (int32_t)idx);
        }
    } else {
        int64_t l = 2 * node + 1, r = l + 1;
        float lbl = node_lb(t, l, pt), lbr = node_lb(t, r, pt);
        if (lbl <= lbr) {
            query_rec(t, mode, l, pt, hp, hi_, k, lbl);
            query_rec(t, mode, r, pt, hp, hi_, k, lbr);
        } else {
            query_rec(t, mode, r, pt, hp, hi_, k, lbr);
            query_rec(t, mode, l, pt, hp, hi_, k, lbl);
        }
    }
}

/* numba_kdtree.py:765 parallel_tree_query(..., output_rdist=True).
 * In mode 1 the initial heap index is INT32_MAX ("none") rather than -1 so
 * that the (distance, index) order places every real candidate before it. */
void orc_tree_query(const orc_kdtree* t, int64_t k, int mode, int nthreads, float* rdist_out,
                    int32_t* idx_out) {
    int64_t n = t->n;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256) if (nthreads != 1)
#endif
    for (int64_t i = 0; i < n; ++i) {
        float* hp = rdist_out + i * k;
        int32_t* hi_ = idx_out + i * k;
        for (int64_t j = 0; j < k; ++j) {
            hp[j] = INFINITY;
            hi_[j] = mode ? INT32_MAX : -1;
        }
        const float* pt = ROW(t, i);
        query_rec(t, mode, 0, pt, hp, hi_, k, node_lb(t, 0, pt));
        deheap_row(mode, hp, hi_, k);
        if (mode)
            for (int64_t j = 0; j < k; ++j)
                if (hi_[j] == INT32_MAX) hi_[j] = -1;
    }
}

/* ------------------------------------------------------------------------- */
/* Disjoint set: disjoint_set.py                                              */
/* ------------------------------------------------------------------------- */

/* disjoint_set.py:21 ds_find.  The reference's tuple assignment
 * `x, parent[x] = parent[x], parent[parent[x]]` rebinds x before the store,
 * so the store is a no-op: the walk does not compress.  Roots are the same
 * either way. */
static inline int32_t ds_find(const int32_t* parent, int32_t x) {
    while (parent[x] != x) x = parent[x];
    return x;
}

/* disjoint_set.py:29 ds_union_by_rank */
static void ds_union_rank(int32_t* parent, int32_t* rank, int32_t x, int32_t y) {
    x = ds_find(parent, x);
    y = ds_find(parent, y);
    if (x == y) return;
    if (rank[x] < rank[y]) {
        int32_t t = x; x = y; y = t;
    }
    parent[y] = x;
    if (rank[x] == rank[y]) rank[x] += 1;
}

/* ------------------------------------------------------------------------- */
/* Boruvka: boruvka.py                                                        */
/* ------------------------------------------------------------------------- */

typedef struct {
    const orc_kdtree* t;
    int mode;
    const float* core;
    const int64_t* pc;      /* point_components */
    const int64_t* nc;      /* node_components */
    const int64_t* orig;    /* identity (indices are the reference's) */
} bq_ctx;

/* The reference's shared per-component bound is a plain racy float; here it
 * is read and written with relaxed atomics on its bit pattern. */
static inline float relaxed_load(const float* p) {
    uint32_t u = __atomic_load_n((const uint32_t*)(const void*)p, __ATOMIC_RELAXED);
    float f;
    memcpy(&f, &u, sizeof f);
    return f;
}
static inline void relaxed_store(float* p, float v) {
    uint32_t u;
    memcpy(&u, &v, sizeof u);
    __atomic_store_n((uint32_t*)(void*)p, u, __ATOMIC_RELAXED);
}

/* boruvka.py:127 component_aware_query_recursion */
static void cq_rec(const bq_ctx* c, int64_t node, const float* pt, float* hp, int32_t* hix,
                   float core_i, int64_t comp, float lb, float* bound) {
    const orc_kdtree* t = c->t;
    float b = relaxed_load(bound);
    if (lb > hp[0]) return;
    if (lb > b || core_i > b) return;
    if (c->nc[node] == comp) return;
    if (t->is_leaf[node]) {
        for (int64_t i = t->idx_start[node]; i < t->idx_end[node]; ++i) {
            int64_t idx = t->idx_array[i];
            if (c->pc[idx] == comp) continue;
            float bb = relaxed_load(bound);
            int ok = c->mode ? (c->core[idx] <= bb) : (c->core[idx] < bb);
            if (!ok) continue;
            float dd = rdist(pt, ROW(t, idx), t->d);
            dd = dd > core_i ? dd : core_i;
            dd = dd > c->core[idx] ? dd : c->core[idx];
            if (pair_lt(c->mode, dd, (int32_t)idx, hp[0], *hix)) {
                hp[0] = dd;
                *hix = (int32_t)idx;
                if (dd < relaxed_load(bound)) relaxed_store(bound, dd);
            }
        }
    } else {
        int64_t l = 2 * node + 1, r = l + 1;
        float lbl = node_lb(t, l, pt), lbr = node_lb(t, r, pt);
        if (lbl <= lbr) {
            cq_rec(c, l, pt, hp, hix, core_i, comp, lbl, bound);
            cq_rec(c, r, pt, hp, hix, core_i, comp, lbr, bound);
        } else {
            cq_rec(c, r, pt, hp, hix, core_i, comp, lbr, bound);
            cq_rec(c, l, pt, hp, hix, core_i, comp, lbl, bound);
        }
    }
}

/* boruvka.py:81 update_component_vectors */
static void update_components(const orc_kdtree* t, const int32_t* parent, int64_t* nc,
                              int64_t* pc, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (nthreads != 1)
#endif
    for (int64_t i = 0; i < t->n; ++i) pc[i] = ds_find(parent, (int32_t)i);
    for (int64_t i = t->n_nodes - 1; i >= 0; --i) {
        if (t->is_leaf[i]) {
            int64_t s = t->idx_start[i], e = t->idx_end[i];
            if (e <= s) continue; /* empty range: reference reads idx_array[s] */
            int64_t cand = pc[t->idx_array[s]];
            int same = 1;
            for (int64_t j = s + 1; j < e; ++j)
                if (pc[t->idx_array[j]] != cand) {
                    same = 0;
                    break;
                }
            if (same) nc[i] = cand;
        } else {
            int64_t l = 2 * i + 1, r = l + 1;
            if (nc[l] == nc[r]) nc[i] = nc[l];
        }
    }
}

/* canonical (weight, min index, max index) order for an undirected edge */
static inline int edge_lt(float w1, int64_t a1, int64_t b1, float w2, int64_t a2, int64_t b2) {
    if (w1 != w2) return w1 < w2;
    int64_t m1 = a1 < b1 ? a1 : b1, M1 = a1 < b1 ? b1 : a1;
    int64_t m2 = a2 < b2 ? a2 : b2, M2 = a2 < b2 ? b2 : a2;
    if (m1 != m2) return m1 < m2;
    return M1 < M2;
}

/* boruvka.py:34 merge_components.  Components are visited in order of first
 * appearance (the dict's insertion order); mode 0 keeps the first strictly
 * smaller candidate, mode 1 the canonical minimum. */
static int64_t merge_components(int mode, int32_t* parent, int32_t* rank, const int32_t* cand_idx,
                                const float* cand_d, const int64_t* pc, int64_t n, double* out,
                                int64_t* slot_of, int64_t* order, int64_t* best_i) {
    int64_t n_comp = 0;
    for (int64_t i = 0; i < n; ++i) slot_of[i] = -1;
    for (int64_t i = 0; i < n; ++i) {
        int64_t fc = pc[i];
        int64_t s = slot_of[fc];
        if (s >= 0 && !isnan(cand_d[i])) {
            int64_t b = best_i[s];
            int better = mode ? edge_lt(cand_d[i], i, cand_idx[i], cand_d[b], b, cand_idx[b])
                              : (cand_d[i] < cand_d[b]);
            if (mode && cand_idx[i] < 0) better = 0;
            if (mode && cand_idx[b] < 0 && cand_idx[i] >= 0) better = 1;
            if (better) best_i[s] = i;
        } else {
            if (s < 0) {
                s = n_comp++;
                slot_of[fc] = s;
                order[s] = fc;
            }
            best_i[s] = i;
        }
    }
    int64_t m = 0;
    for (int64_t s = 0; s < n_comp; ++s) {
        int64_t i = best_i[s];
        int32_t q = cand_idx[i];
        if (q < 0) continue; /* no candidate: the reference would index [-1] */
        int32_t fcmp = ds_find(parent, (int32_t)i), tcmp = ds_find(parent, q);
        if (fcmp != tcmp) {
            out[m * 3 + 0] = (double)i;
            out[m * 3 + 1] = (double)q;
            out[m * 3 + 2] = (double)cand_d[i];
            ++m;
            ds_union_rank(parent, rank, fcmp, tcmp);
        }
    }
    return m;
}

/* boruvka.py:474 initialize_boruvka_from_knn */
static int64_t init_from_knn(const int32_t* knn_idx, const float* knn_d, int64_t k,
                             const float* core, int64_t n, int32_t* parent, int32_t* rank,
                             double* out) {
    int64_t m = 0;
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t j = 1; j < k; ++j) {
            int32_t q = knn_idx[i * k + j];
            if (q < 0) break;
            if (core[i] >= core[q]) {
                float w = core[i] > knn_d[i * k + j] ? core[i] : knn_d[i * k + j];
                int32_t f = ds_find(parent, (int32_t)i), tt = ds_find(parent, q);
                if (f != tt) {
                    out[m * 3 + 0] = (double)i;
                    out[m * 3 + 1] = (double)q;
                    out[m * 3 + 2] = (double)w;
                    ++m;
                    ds_union_rank(parent, rank, f, tt);
                }
                break;
            }
        }
    }
    return m;
}

/* boruvka.py:542 parallel_boruvka.  weights == NULL: the unweighted path;
 * otherwise (boruvka.py:561-573) the kNN query of k = wk neighbours returns
 * plain distances (output_rdist=False: sqrt of the float32 rdist),
 * sample_weight_core_distance (:527) picks the core distance, round 0 works
 * on those plain distances and the Boruvka rounds compare them with squared
 * distances, exactly as the reference does. */
int64_t orc_parallel_boruvka(const orc_kdtree* t, int64_t min_samples, int mode, int nthreads,
                             const float* weights, int64_t wk, double* edges, int32_t* neighbors,
                             float* core_out, int64_t* n_rounds) {
    int64_t n = t->n;
    int64_t k = weights ? wk : (min_samples > 1 ? min_samples + 1 : 2);
    /* mode 2: mode 0's rules with a private search bound per point (see
     * oracle.h); everything else runs as mode 0 */
    const int private_bound = mode == 2;
    if (mode == 2) mode = 0;
    float* kd = (float*)malloc(sizeof(float) * (size_t)(n * k));
    int32_t* ki = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n * k));
    orc_tree_query(t, k, mode, nthreads, kd, ki);
    float* core = (float*)malloc(sizeof(float) * (size_t)n);
    if (weights) {
        for (int64_t i = 0; i < n * k; ++i) kd[i] = sqrtf(kd[i]);
        for (int64_t i = 0; i < n; ++i) {
            double total = 0.0;
            int64_t j = 0;
            while (total < (double)min_samples && j < k) {
                int32_t q = ki[i * k + j];
                total += (double)weights[q >= 0 ? q : n + q];  /* numba wraps index -1 */
                ++j;
            }
            core[i] = kd[i * k + (j > 0 ? j - 1 : k - 1)];
        }
    } else {
        for (int64_t i = 0; i < n; ++i) core[i] = min_samples > 1 ? kd[i * k + k - 1] : 0.0f;
    }

    int32_t* parent = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int32_t* rank = (int32_t*)calloc((size_t)n, sizeof(int32_t));
    for (int64_t i = 0; i < n; ++i) parent[i] = (int32_t)i;
    int64_t* pc = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    int64_t* nc = (int64_t*)malloc(sizeof(int64_t) * (size_t)t->n_nodes);
    for (int64_t i = 0; i < t->n_nodes; ++i) nc[i] = -1;
    double* buf = (double*)malloc(sizeof(double) * 3 * (size_t)n);

    int64_t m = init_from_knn(ki, kd, k, core, n, parent, rank, buf);
    memcpy(edges, buf, sizeof(double) * 3 * (size_t)m);
    update_components(t, parent, nc, pc, nthreads);

    int64_t n_comp = 0;
    for (int64_t i = 0; i < n; ++i) n_comp += (pc[i] == i);

    float* cd = (float*)malloc(sizeof(float) * (size_t)n);
    int32_t* cix = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    float* cnnd = (float*)malloc(sizeof(float) * (size_t)n);
    int64_t* slot_of = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    int64_t* order = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    int64_t* best_i = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    bq_ctx ctx = {t, mode, core, pc, nc, NULL};
    int64_t rounds = 0;
    while (n_comp > 1) {
        for (int64_t i = 0; i < n; ++i) {
            cd[i] = INFINITY;
            cix[i] = mode ? INT32_MAX : -1;
            cnnd[i] = INFINITY;
        }
        /* boruvka.py:290 boruvka_tree_query */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) if (nthreads != 1)
#endif
        for (int64_t i = 0; i < n; ++i) {
            const float* pt = ROW(t, i);
            float own = INFINITY;
            cq_rec(&ctx, 0, pt, &cd[i], &cix[i], core[i], pc[i], node_lb(t, 0, pt),
                   private_bound ? &own : &cnnd[pc[i]]);
        }
        if (mode)
            for (int64_t i = 0; i < n; ++i)
                if (cix[i] == INT32_MAX) cix[i] = -1;
        int64_t added = merge_components(mode, parent, rank, cix, cd, pc, n, buf, slot_of,
                                         order, best_i);
        memcpy(edges + 3 * m, buf, sizeof(double) * 3 * (size_t)added);
        m += added;
        n_comp -= added;
        update_components(t, parent, nc, pc, nthreads);
        ++rounds;
        if (added == 0) break; /* disconnected: only when every candidate is missing */
    }
    for (int64_t e = 0; e < m; ++e) edges[e * 3 + 2] = sqrt(edges[e * 3 + 2]);
    int64_t ms_cols = k - 1;
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = 1; j < k; ++j) neighbors[i * ms_cols + j - 1] = ki[i * k + j];
    for (int64_t i = 0; i < n; ++i) core_out[i] = sqrtf(core[i]);
    if (n_rounds) *n_rounds = rounds;
    free(kd); free(ki); free(core); free(parent); free(rank); free(pc); free(nc); free(buf);
    free(cd); free(cix); free(cnnd); free(slot_of); free(order); free(best_i);
    return m;
}

/* ------------------------------------------------------------------------- */
/* Tree passes: hdbscan.py:511, cluster_trees.py                              */
/* ------------------------------------------------------------------------- */

static const double* g_sort_mst;
static int cmp_mst(const void* a, const void* b) {
    int64_t i = *(const int64_t*)a, j = *(const int64_t*)b;
    const double* x = g_sort_mst + 3 * i;
    const double* y = g_sort_mst + 3 * j;
    if (x[2] != y[2]) return x[2] < y[2] ? -1 : 1;
    if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
    if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
    return i < j ? -1 : (i > j);
}

/* hdbscan.py:511 np.lexsort((mst[:,1], mst[:,0], mst[:,2])) (stable) */
void orc_sort_mst(const double* mst, int64_t m, double* out) {
    int64_t* o = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
    for (int64_t i = 0; i < m; ++i) o[i] = i;
    g_sort_mst = mst;
    qsort(o, (size_t)m, sizeof(int64_t), cmp_mst);
    for (int64_t i = 0; i < m; ++i) memcpy(out + 3 * i, mst + 3 * o[i], 3 * sizeof(double));
    free(o);
}

/* cluster_trees.py:38 linkage_merge_find */
static int64_t lm_find(int64_t* parent, int64_t node) {
    int64_t relabel = node;
    while (parent[node] != -1 && parent[node] != node) node = parent[node];
    parent[node] = node;
    while (parent[relabel] != node) {
        int64_t nx = parent[relabel];
        parent[relabel] = node;
        relabel = nx;
    }
    return node;
}

/* cluster_trees.py:98 mst_to_linkage_tree_w_sample_weights: sizes are float32
 * sums of the weights (create_linkage_merge_data_w_sample_weights, :29). */
void orc_mst_to_linkage_tree_w(const double* smst, int64_t m, const float* w, double* out) {
    int64_t n = m + 1;
    int64_t* parent = (int64_t*)malloc(sizeof(int64_t) * (size_t)(2 * n - 1));
    float* size = (float*)malloc(sizeof(float) * (size_t)(2 * n - 1));
    for (int64_t i = 0; i < 2 * n - 1; ++i) {
        parent[i] = -1;
        size[i] = i < n ? w[i] : 0.0f;
    }
    int64_t next = n;
    for (int64_t e = 0; e < m; ++e) {
        int64_t l = (int64_t)smst[3 * e], r = (int64_t)smst[3 * e + 1];
        int64_t lc = lm_find(parent, l), rc = lm_find(parent, r);
        out[4 * e + 0] = (double)(lc > rc ? lc : rc);
        out[4 * e + 1] = (double)(lc > rc ? rc : lc);
        out[4 * e + 2] = smst[3 * e + 2];
        float sz = size[lc] + size[rc];
        out[4 * e + 3] = (double)sz;
        size[next] = sz;
        parent[lc] = next;
        parent[rc] = next;
        ++next;
    }
    free(parent);
    free(size);
}

/* cluster_trees.py:65 mst_to_linkage_tree */
void orc_mst_to_linkage_tree(const double* smst, int64_t m, double* out) {
    int64_t n = m + 1;
    int64_t* parent = (int64_t*)malloc(sizeof(int64_t) * (size_t)(2 * n - 1));
    int64_t* size = (int64_t*)malloc(sizeof(int64_t) * (size_t)(2 * n - 1));
    for (int64_t i = 0; i < 2 * n - 1; ++i) {
        parent[i] = -1;
        size[i] = i < n ? 1 : 0;
    }
    int64_t next = n;
    for (int64_t e = 0; e < m; ++e) {
        int64_t l = (int64_t)smst[3 * e], r = (int64_t)smst[3 * e + 1];
        int64_t lc = lm_find(parent, l), rc = lm_find(parent, r);
        out[4 * e + 0] = (double)(lc > rc ? lc : rc);
        out[4 * e + 1] = (double)(lc > rc ? rc : lc);
        out[4 * e + 2] = smst[3 * e + 2];
        out[4 * e + 3] = (double)(size[lc] + size[rc]);
        size[next] = size[lc] + size[rc];
        parent[lc] = next;
        parent[rc] = next;
        ++next;
    }
    free(parent);
    free(size);
}

/* cluster_trees.py:130 bfs_from_hierarchy */
static int64_t bfs_hier(const double* h, int64_t root, int64_t num_points, int64_t* out,
                        int64_t* tmp) {
    int64_t cnt = 0, lvl_s = 0, lvl_e;
    out[cnt++] = root;
    (void)tmp;
    while (lvl_s < cnt) {
        lvl_e = cnt;
        for (int64_t q = lvl_s; q < lvl_e; ++q) {
            int64_t nd = out[q];
            if (nd >= num_points) {
                int64_t i = nd - num_points;
                out[cnt++] = (int64_t)h[4 * i + 0];
                out[cnt++] = (int64_t)h[4 * i + 1];
            }
        }
        lvl_s = lvl_e;
    }
    return cnt;
}

/* cluster_trees.py:192 hdbscan_lambda_value, rounded to the float32 store */
static inline float lambda_of(double dist) { return (float)(dist > 0.0 ? 1.0 / dist : INFINITY); }

/* cluster_trees.py:205 condense_tree; w == NULL: unit sample weights */
int64_t orc_condense_tree(const double* h, int64_t m, int64_t mcs, double max_cs, const float* w,
                          int64_t* parents, int64_t* children, float* lambdas, float* sizes) {
    int64_t root = 2 * m, num_points = m + 1, next_label = num_points + 1;
    int64_t* node_list = (int64_t*)malloc(sizeof(int64_t) * (size_t)(root + 1));
    int64_t* sub = (int64_t*)malloc(sizeof(int64_t) * (size_t)(root + 1));
    int64_t n_list = bfs_hier(h, root, num_points, node_list, NULL);
    int64_t* relabel = (int64_t*)calloc((size_t)(root + 1), sizeof(int64_t));
    uint8_t* ignore = (uint8_t*)calloc((size_t)(root + 1), 1);
    relabel[root] = num_points;
    int64_t idx = 0;
    for (int64_t q = 0; q < n_list; ++q) {
        int64_t node = node_list[q];
        if (ignore[node] || node < num_points) continue;
        int64_t parent_node = relabel[node];
        const double* row = h + 4 * (node - num_points);
        int64_t left = (int64_t)row[0], right = (int64_t)row[1];
        float lam = lambda_of(row[2]);
        float lc = left >= num_points ? (float)h[4 * (left - num_points) + 3]
                                      : (w ? w[left] : 1.0f);
        float rc = right >= num_points ? (float)h[4 * (right - num_points) + 3]
                                       : (w ? w[right] : 1.0f);
        int elim_l = 0, elim_r = 0;
        if (left < num_points && rc >= (float)mcs) {
            relabel[right] = parent_node;
            parents[idx] = parent_node;
            children[idx] = left;
            lambdas[idx] = lam;
            sizes[idx] = 1.0f;
            ++idx;
        } else if (lc < (float)mcs && rc >= (float)mcs) {
            relabel[right] = parent_node;
            elim_l = 1;
        } else if (lc >= (float)mcs && rc < (float)mcs) {
            relabel[left] = parent_node;
            elim_r = 1;
        } else if (lc < (float)mcs && rc < (float)mcs) {
            elim_l = elim_r = 1;
        } else if ((double)lc > max_cs && (double)rc > max_cs) {
            relabel[left] = parent_node;
            relabel[right] = parent_node;
        } else {
            relabel[left] = next_label;
            parents[idx] = parent_node;
            children[idx] = next_label;
            lambdas[idx] = lam;
            sizes[idx] = lc;
            ++next_label;
            ++idx;
            relabel[right] = next_label;
            parents[idx] = parent_node;
            children[idx] = next_label;
            lambdas[idx] = lam;
            sizes[idx] = rc;
            ++next_label;
            ++idx;
        }
        /* cluster_trees.py:148 eliminate_branch */
        for (int side = 0; side < 2; ++side) {
            if (!(side == 0 ? elim_l : elim_r)) continue;
            int64_t br = side == 0 ? left : right;
            if (br < num_points) {
                parents[idx] = parent_node;
                children[idx] = br;
                lambdas[idx] = lam;
                sizes[idx] = 1.0f;
                ++idx;
            } else {
                int64_t cnt = bfs_hier(h, br, num_points, sub, NULL);
                for (int64_t s = 0; s < cnt; ++s) {
                    int64_t sn = sub[s];
                    if (sn < num_points) {
                        children[idx] = sn;
                        parents[idx] = parent_node;
                        lambdas[idx] = lam;
                        sizes[idx] = 1.0f;
                        ++idx;
                    } else {
                        ignore[sn] = 1;
                    }
                }
            }
        }
    }
    free(node_list);
    free(sub);
    free(relabel);
    free(ignore);
    return idx;
}

/* cluster_trees.py:656 score_condensed_tree_nodes: float32, in row order.
 * scores are indexed by label - root (root = parent[0]). */
static void score_nodes(const int64_t* parent, const int64_t* child, const float* lam,
                        const float* size, int64_t rows, int64_t root, float* score) {
    score[0] = 0.0f;
    for (int64_t i = 0; i < rows; ++i) {
        if (size[i] > 1.0f) score[child[i] - root] = -lam[i] * size[i];
        score[parent[i] - root] += lam[i] * size[i];
    }
}

static int64_t max_label(const int64_t* parent, const int64_t* child, int64_t rows) {
    int64_t mx = 0;
    for (int64_t i = 0; i < rows; ++i) {
        if (parent[i] > mx) mx = parent[i];
        if (child[i] > mx) mx = child[i];
    }
    return mx;
}

/* cluster_trees.py:724 extract_eom_clusters with eom_recursion (:694) and
 * unselect_below_node (:687), evaluated bottom-up: labels are assigned in BFS
 * order, so every cluster's children have larger labels than it does. */
int64_t orc_extract_eom_clusters(const int64_t* parent, const int64_t* child, const float* lam,
                                 const float* size, int64_t rows, double max_cs,
                                 int allow_single, int64_t* sel) {
    int64_t ct_rows = 0, root = -1;
    for (int64_t i = 0; i < rows; ++i)
        if (size[i] > 1.0f) {
            ++ct_rows;
            if (root < 0 || parent[i] < root) root = parent[i];
        }
    if (ct_rows == 0) return 0;
    int64_t top = max_label(parent, child, rows);
    int64_t L = top - root + 1;
    float* score = (float*)calloc((size_t)L, sizeof(float));
    float* nsize = (float*)calloc((size_t)L, sizeof(float));
    double* ret = (double*)calloc((size_t)L, sizeof(double));
    double* ctot = (double*)calloc((size_t)L, sizeof(double));
    uint8_t* chose = (uint8_t*)calloc((size_t)L, 1);
    uint8_t* blocked = (uint8_t*)calloc((size_t)L, 1);
    uint8_t* in_ct = (uint8_t*)calloc((size_t)L, 1);
    int64_t* cpar = (int64_t*)malloc(sizeof(int64_t) * (size_t)L);
    /* children of each cluster in row order (CSR) */
    int64_t* cnt = (int64_t*)calloc((size_t)L + 1, sizeof(int64_t));
    int64_t* lst = (int64_t*)malloc(sizeof(int64_t) * (size_t)(ct_rows > 0 ? ct_rows : 1));
    score_nodes(parent, child, lam, size, rows, parent[0], score);
    for (int64_t i = 0; i < L; ++i) cpar[i] = -1;
    for (int64_t i = 0; i < rows; ++i)
        if (size[i] > 1.0f) {
            nsize[child[i] - root] = size[i];
            in_ct[child[i] - root] = 1;
            cpar[child[i] - root] = parent[i] - root;
            cnt[parent[i] - root + 1]++;
        }
    nsize[0] = (float)(root - 1);
    in_ct[0] = 1;
    for (int64_t i = 0; i < L; ++i) cnt[i + 1] += cnt[i];
    {
        int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)L);
        for (int64_t i = 0; i < L; ++i) fill[i] = cnt[i];
        for (int64_t i = 0; i < rows; ++i)
            if (size[i] > 1.0f) lst[fill[parent[i] - root]++] = child[i] - root;
        free(fill);
    }
    /* scope: the recursion starts at the root (allow_single) or its children */
    for (int64_t v = L - 1; v >= 0; --v) {
        if (!in_ct[v]) continue;
        if (v == 0 && !allow_single) continue;
        double cur = (double)score[v] > 0.0 ? (double)score[v] : 0.0;
        double tot = 0.0;
        for (int64_t e = cnt[v]; e < cnt[v + 1]; ++e) tot += ret[lst[e]];
        ctot[v] = tot;
        if (tot > cur || (double)nsize[v] > max_cs) {
            ret[v] = tot;
        } else {
            chose[v] = 1;
            ret[v] = cur;
        }
    }
    for (int64_t v = 1; v < L; ++v) {
        if (!in_ct[v]) continue;
        int64_t p = cpar[v];
        blocked[v] = blocked[p] || (chose[p] && (p != 0 || allow_single));
    }
    int64_t ns = 0;
    /* output in the dict's insertion order: root, then cluster rows */
    if (allow_single && chose[0]) sel[ns++] = root;
    for (int64_t i = 0; i < rows; ++i)
        if (size[i] > 1.0f) {
            int64_t v = child[i] - root;
            if (chose[v] && !blocked[v]) sel[ns++] = child[i];
        }
    free(score); free(nsize); free(ret); free(ctot); free(chose); free(blocked); free(in_ct);
    free(cpar); free(cnt); free(lst);
    return ns;
}

/* cluster_trees.py:369 cluster_tree_leaves */
int64_t orc_cluster_tree_leaves(const int64_t* parent, const int64_t* child, const float* size,
                                int64_t rows, int64_t n_points, int64_t* sel) {
    int64_t mx = -1;
    for (int64_t i = 0; i < rows; ++i)
        if (size[i] > 1.0f && child[i] > mx) mx = child[i];
    if (mx < 0) return 0;
    int64_t L = mx + 1 - n_points;
    uint8_t* leaf = (uint8_t*)malloc((size_t)L);
    memset(leaf, 1, (size_t)L);
    for (int64_t i = 0; i < rows; ++i)
        if (size[i] > 1.0f) leaf[parent[i] - n_points] = 0;
    int64_t ns = 0;
    for (int64_t v = 0; v < L; ++v)
        if (leaf[v]) sel[ns++] = v + n_points;
    free(leaf);
    return ns;
}

/* cluster tree rows (child_size > 1) gathered in row order */
typedef struct {
    int64_t n;
    int64_t *parent, *child;
    float* lam;
} ctree;

static ctree make_ctree(const int64_t* parent, const int64_t* child, const float* lam,
                        const float* size, int64_t rows) {
    ctree c;
    c.n = 0;
    c.parent = (int64_t*)malloc(sizeof(int64_t) * (size_t)(rows + 1));
    c.child = (int64_t*)malloc(sizeof(int64_t) * (size_t)(rows + 1));
    c.lam = (float*)malloc(sizeof(float) * (size_t)(rows + 1));
    for (int64_t i = 0; i < rows; ++i)
        if (size[i] > 1.0f) {
            c.parent[c.n] = parent[i];
            c.child[c.n] = child[i];
            c.lam[c.n] = lam[i];
            ++c.n;
        }
    return c;
}
static void free_ctree(ctree* c) {
    free(c->parent);
    free(c->child);
    free(c->lam);
}

/* cluster_trees.py:866 traverse_upwards */
static int64_t traverse_upwards(const ctree* c, double min_eps, int64_t root, int64_t seg) {
    for (;;) {
        int64_t par = -1;
        for (int64_t i = 0; i < c->n; ++i)
            if (c->child[i] == seg) {
                par = c->parent[i];
                break;
            }
        if (par == root) return root;
        float pl = 0.0f;
        for (int64_t i = 0; i < c->n; ++i)
            if (c->child[i] == par) {
                pl = c->lam[i];
                break;
            }
        double pe = pl > 0.0f ? 1.0 / (double)pl : INFINITY;
        if (pe >= min_eps) return par;
        seg = par;
    }
}

/* cluster_trees.py:881 segments_in_branch: the closure of {seg} under
 * x -> {children[i], children[i+1]}, i = np.searchsorted(parents, x), over the
 * cluster tree sorted by parent.  The lookup does not check parents[i] == x:
 * for a leaf x it takes the first two children of the next larger parent, as
 * the reference does.  Marks the closure in `processed`. */
static void segments_in_branch(const int64_t* sp, const int64_t* sc, int64_t len, int64_t seg,
                               uint8_t* processed, int64_t mx) {
    int64_t* stack = (int64_t*)malloc(sizeof(int64_t) * (size_t)(2 * (mx + 2)));
    int64_t top = 0;
    stack[top++] = seg;
    while (top) {
        int64_t x = stack[--top];
        if (x < 0 || x > mx || processed[x]) continue;
        processed[x] = 1;
        int64_t lo = 0, hi = len;
        while (lo < hi) {
            int64_t mid = (lo + hi) / 2;
            if (sp[mid] < x) lo = mid + 1;
            else hi = mid;
        }
        if (lo >= len) continue;
        stack[top++] = sc[lo];
        if (lo + 1 < len) stack[top++] = sc[lo + 1];
    }
    free(stack);
}

/* cluster_trees.py:834 cluster_epsilon_search */
int64_t orc_cluster_epsilon_search(const int64_t* parent, const int64_t* child, const float* lam,
                                   const float* size, int64_t rows, const int64_t* clusters,
                                   int64_t n_clusters, double min_eps, int64_t* out) {
    ctree c = make_ctree(parent, child, lam, size, rows);
    int64_t root = INT64_MAX, mx = 0;
    for (int64_t i = 0; i < c.n; ++i) {
        if (c.parent[i] < root) root = c.parent[i];
        if (c.child[i] > mx) mx = c.child[i];
    }
    uint8_t* processed = (uint8_t*)calloc((size_t)(mx + 2), 1);
    /* np.argsort(cluster_tree.parent): a stable order (siblings share a parent,
     * so the pair of children taken for a parent is the same either way) */
    int64_t* sp = (int64_t*)malloc(sizeof(int64_t) * (size_t)(c.n + 1));
    int64_t* sc = (int64_t*)malloc(sizeof(int64_t) * (size_t)(c.n + 1));
    for (int64_t i = 0; i < c.n; ++i) {
        sp[i] = c.parent[i];
        sc[i] = c.child[i];
    }
    for (int64_t i = 1; i < c.n; ++i) { /* insertion sort, stable */
        int64_t kp = sp[i], kc = sc[i], j = i - 1;
        while (j >= 0 && sp[j] > kp) {
            sp[j + 1] = sp[j];
            sc[j + 1] = sc[j];
            --j;
        }
        sp[j + 1] = kp;
        sc[j + 1] = kc;
    }
    int64_t ns = 0;
    for (int64_t q = 0; q < n_clusters; ++q) {
        int64_t cl = clusters[q];
        /* np.searchsorted(cluster_tree.child, cluster): children are ascending */
        int64_t idx = 0;
        while (idx < c.n && c.child[idx] < cl) ++idx;
        float lm = c.lam[idx < c.n ? idx : c.n - 1];
        double death = lm > 0.0f ? 1.0 / (double)lm : INFINITY;
        if (death < min_eps) {
            if (!processed[cl]) {
                int64_t par = traverse_upwards(&c, min_eps, root, cl);
                out[ns++] = par;
                segments_in_branch(sp, sc, c.n, par, processed, mx);
            }
        } else {
            out[ns++] = cl;
        }
    }
    free(processed);
    free(sp);
    free(sc);
    free_ctree(&c);
    return ns;
}

/* cluster_trees.py:774 simplify_hierarchy (mutates in place, returns rows kept,
 * compacted to the front in order) */
int64_t orc_simplify_hierarchy(int64_t* parent, int64_t* child, float* lam, float* size,
                               int64_t rows, double thr) {
    ctree c = make_ctree(parent, child, lam, size, rows);
    if (c.n == 0) {
        free_ctree(&c);
        return rows;
    }
    int64_t n_points = parent[0];
    int64_t n_nodes = c.child[c.n - 1] + 1;
    int64_t L = n_nodes - n_points;
    uint8_t* leaf = (uint8_t*)malloc((size_t)L);
    memset(leaf, 1, (size_t)L);
    for (int64_t i = 0; i < c.n; ++i) leaf[c.parent[i] - n_points] = 0;
    float* max_births = (float*)malloc(sizeof(float) * (size_t)L);
    for (int64_t i = 0; i < L; ++i) max_births[i] = 0.0f; /* np.empty: every slot is written below */
    for (int64_t i = 0; i < rows; ++i) max_births[parent[i] - n_points] = lam[i];
    int64_t* parent_map = (int64_t*)malloc(sizeof(int64_t) * (size_t)L);
    for (int64_t i = 0; i < L; ++i) parent_map[i] = n_points + i;
    uint8_t* has_lm = (uint8_t*)calloc((size_t)L, 1);
    float* lmap = (float*)calloc((size_t)L, sizeof(float));
    for (int64_t idx = c.n - 1; idx > 0; idx -= 2) {
        int64_t par = c.parent[idx];
        int64_t ch0 = c.child[idx - 1], ch1 = c.child[idx];
        float death = c.lam[idx];
        int64_t n0 = ch0 - n_points, n1 = ch1 - n_points;
        float b0 = max_births[n0], b1 = max_births[n1];
        float bmax = b0 > b1 ? b0 : b1, bmin = b0 < b1 ? b0 : b1;
        float cur = max_births[par - n_points];
        max_births[par - n_points] = cur > bmax ? cur : bmax;
        if ((double)(bmin - death) >= thr) continue;
        int64_t sib = (b0 <= b1) ? 1 : 0;
        int64_t sib_node = sib ? n1 : n0;
        int64_t other = sib ? ch0 : ch1;
        if (leaf[sib_node]) {
            leaf[par - n_points] = 1;
        } else {
            has_lm[other - n_points] = 1;
            lmap[other - n_points] = death;
        }
        parent_map[n0] = par;
        parent_map[n1] = par;
    }
    uint8_t* skipped = (uint8_t*)calloc((size_t)L, 1);
    for (int64_t i = 0; i < L; ++i) parent_map[i] = parent_map[parent_map[i] - n_points];
    /* prefix count of skipped nodes */
    int64_t* pre = (int64_t*)calloc((size_t)L + 1, sizeof(int64_t));
    for (int64_t i = 0; i < L; ++i) {
        int64_t p = parent_map[i];
        skipped[i] = p != (i + n_points);
        /* n_skipped[: p - n_points].sum(): only entries < i can be set yet
         * when p - n_points <= i, as the reference's sequential loop sees */
        int64_t s = 0;
        for (int64_t j = 0; j < p - n_points; ++j) s += skipped[j];
        parent_map[i] = p - s;
    }
    free(pre);
    int64_t out = 0;
    for (int64_t i = 0; i < rows; ++i) {
        int64_t ch = child[i];
        int64_t key = ch - n_points > 0 ? ch - n_points : 0;
        if (skipped[key]) continue;
        int64_t p = parent[i];
        float lv = lam[i];
        if (has_lm[p - n_points]) lv = lmap[p - n_points];
        int64_t np_ = parent_map[p - n_points];
        int64_t nch = ch >= n_points ? parent_map[ch - n_points] : ch;
        parent[out] = np_;
        child[out] = nch;
        lam[out] = lv;
        size[out] = size[i];
        ++out;
    }
    free(leaf); free(max_births); free(parent_map); free(has_lm); free(lmap); free(skipped);
    free_ctree(&c);
    return out;
}

static int cmp_i64(const void* a, const void* b) {
    int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return x < y ? -1 : (x > y);
}

/* cluster_trees.py:944 get_cluster_label_vector */
int orc_get_cluster_label_vector(const int64_t* parent, const int64_t* child, const float* lam,
                                 int64_t rows, const int64_t* clusters, int64_t n_clusters,
                                 double eps, int64_t n_samples, int64_t* labels) {
    for (int64_t i = 0; i < n_samples; ++i) labels[i] = -1;
    if (rows == 0 || n_clusters == 0) return 0;
    int64_t root = INT64_MAX, mx = 0;
    for (int64_t i = 0; i < rows; ++i) {
        if (parent[i] < root) root = parent[i];
        if (parent[i] > mx) mx = parent[i];
        if (child[i] > mx) mx = child[i];
    }
    int64_t nds = mx + 1;
    uint8_t* is_sel = (uint8_t*)calloc((size_t)nds + 1, 1);
    int64_t* label_of = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nds + 1));
    for (int64_t i = 0; i <= nds; ++i) label_of[i] = -1;
    int64_t n_distinct = 0;
    for (int64_t q = 0; q < n_clusters; ++q)
        if (clusters[q] >= 0 && clusters[q] < nds && !is_sel[clusters[q]]) {
            is_sel[clusters[q]] = 1;
            ++n_distinct;
        }
    /* {c: n for n, c in enumerate(np.sort(clusters))}: the last position of
     * each id in the sorted list */
    {
        int64_t* srt = (int64_t*)malloc(sizeof(int64_t) * (size_t)n_clusters);
        memcpy(srt, clusters, sizeof(int64_t) * (size_t)n_clusters);
        qsort(srt, (size_t)n_clusters, sizeof(int64_t), cmp_i64);
        for (int64_t q = 0; q < n_clusters; ++q)
            if (srt[q] >= 0 && srt[q] < nds) label_of[srt[q]] = q;
        free(srt);
    }
    int32_t* dp = (int32_t*)malloc(sizeof(int32_t) * (size_t)nds);
    int32_t* dr = (int32_t*)calloc((size_t)nds, sizeof(int32_t));
    for (int64_t i = 0; i < nds; ++i) dp[i] = (int32_t)i;
    for (int64_t i = 0; i < rows; ++i) {
        int64_t ch = child[i], p = parent[i];
        if (!is_sel[ch]) {
            if (ch < n_samples && lam[i] == 0.0f) continue;
            ds_union_rank(dp, dr, (int32_t)p, (int32_t)ch);
        }
    }
    int rc = 0;
    for (int64_t nn = 0; nn < root; ++nn) {
        int64_t cl = ds_find(dp, (int32_t)nn);
        if (cl < root) {
            labels[nn] = -1;
        } else if (cl == root) {
            if (n_distinct == 1) {
                float max_l = -INFINITY;
                for (int64_t i = 0; i < rows; ++i)
                    if (parent[i] == cl && lam[i] > max_l) max_l = lam[i];
                float cur = NAN;
                for (int64_t i = 0; i < rows; ++i)
                    if (child[i] == nn) {
                        cur = lam[i];
                        break;
                    }
                int take;
                if (eps > 0.0) take = (double)cur >= 1.0 / eps;
                else take = cur >= max_l;
                if (take) {
                    if (label_of[cl] < 0) rc = -1;
                    labels[nn] = label_of[cl];
                } else {
                    labels[nn] = -1;
                }
            } else {
                labels[nn] = -1;
            }
        } else {
            if (label_of[cl] < 0) rc = -1;
            labels[nn] = label_of[cl];
        }
    }
    free(is_sel); free(label_of); free(dp); free(dr);
    return rc;
}

/* cluster_trees.py:1011 get_point_membership_strength_vector with
 * max_lambdas (:999); the ratio is formed in float64 and stored as float32 */
void orc_get_point_membership_strength_vector(const int64_t* parent, const int64_t* child,
                                              const float* lam, const float* size, int64_t rows,
                                              const int64_t* clusters, int64_t n_clusters,
                                              const int64_t* labels, int64_t n_samples,
                                              float* probs) {
    for (int64_t i = 0; i < n_samples; ++i) probs[i] = 0.0f;
    if (rows == 0) return;
    int64_t root = INT64_MAX, mx = 0;
    for (int64_t i = 0; i < rows; ++i) {
        if (parent[i] < root) root = parent[i];
        if (parent[i] > mx) mx = parent[i];
        if (child[i] > mx) mx = child[i];
    }
    for (int64_t q = 0; q < n_clusters; ++q)
        if (clusters[q] > mx) mx = clusters[q];
    double* deaths = (double*)calloc((size_t)mx + 1, sizeof(double));
    uint8_t* is_sel = (uint8_t*)calloc((size_t)mx + 1, 1);
    for (int64_t q = 0; q < n_clusters; ++q) is_sel[clusters[q]] = 1;
    for (int64_t i = 0; i < rows; ++i)
        if (is_sel[parent[i]] && size[i] == 1.0f)
            if ((double)lam[i] > deaths[parent[i]]) deaths[parent[i]] = (double)lam[i];
    /* {n: c for n, c in enumerate(np.sort(clusters))}: label -> cluster id */
    int64_t* by_label = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n_clusters + 1));
    memcpy(by_label, clusters, sizeof(int64_t) * (size_t)n_clusters);
    qsort(by_label, (size_t)n_clusters, sizeof(int64_t), cmp_i64);
    for (int64_t i = 0; i < rows; ++i) {
        int64_t pt = child[i];
        if (pt >= root || labels[pt] < 0) continue;
        int64_t cl = by_label[labels[pt]];
        double ml = deaths[cl];
        if (ml == 0.0 || !isfinite(lam[i])) {
            probs[pt] = 1.0f;
        } else {
            double lv = (double)lam[i] < ml ? (double)lam[i] : ml;
            probs[pt] = (float)(lv / ml);
        }
    }
    free(deaths); free(is_sel); free(by_label);
}

/* cluster_trees.py:906 get_cluster_labelling_at_cut */
void orc_get_cluster_labelling_at_cut(const double* lk, int64_t m, double cut, int64_t mcs,
                                      int64_t* out) {
    int64_t root = 2 * m, num_points = m + 1;
    int32_t* dp = (int32_t*)malloc(sizeof(int32_t) * (size_t)(root + 1));
    int32_t* dr = (int32_t*)calloc((size_t)(root + 1), sizeof(int32_t));
    for (int64_t i = 0; i <= root; ++i) dp[i] = (int32_t)i;
    int64_t cluster = num_points;
    for (int64_t i = 0; i < m; ++i) {
        if (lk[4 * i + 2] < cut) {
            ds_union_rank(dp, dr, (int32_t)lk[4 * i + 0], (int32_t)cluster);
            ds_union_rank(dp, dr, (int32_t)lk[4 * i + 1], (int32_t)cluster);
        }
        ++cluster;
    }
    int64_t* csize = (int64_t*)calloc((size_t)(cluster + 1), sizeof(int64_t));
    for (int64_t p = 0; p < num_points; ++p) {
        int64_t c = ds_find(dp, (int32_t)p);
        csize[c]++;
        out[p] = c;
    }
    /* labels in increasing cluster id order (np.unique) */
    int64_t* map = (int64_t*)malloc(sizeof(int64_t) * (size_t)(cluster + 1));
    uint8_t* seen = (uint8_t*)calloc((size_t)(cluster + 1), 1);
    for (int64_t p = 0; p < num_points; ++p) seen[out[p]] = 1;
    int64_t lab = 0;
    for (int64_t c = 0; c <= cluster; ++c) {
        if (!seen[c]) continue;
        if (csize[c] < mcs) map[c] = -1;
        else map[c] = lab++;
    }
    for (int64_t p = 0; p < num_points; ++p) out[p] = map[out[p]];
    free(dp); free(dr); free(csize); free(map); free(seen);
}

/* ------------------------------------------------------------------------- */
/* kNN-graph Kruskal MST: kruskal.py:950-1034 (_kruskal_mst_knn without       */
/* cannot-link constraints), kruskal.py:456 _build_mrd_edges_knn, :32         */
/* _kruskal_core, :723 _finish_mst + precomputed.py:308 bridge_forest_with_inf */
/* ------------------------------------------------------------------------- */

static const double* g_kr_w;
/* kruskal.py:1028 np.argsort(weights, kind="stable"): by weight, then position */
static int cmp_kr(const void* a, const void* b) {
    const int64_t i = *(const int64_t*)a, j = *(const int64_t*)b;
    const double wi = g_kr_w[i], wj = g_kr_w[j];
    if (wi < wj) return -1;
    if (wi > wj) return 1;
    return (i > j) - (i < j);
}

int64_t orc_kruskal_knn(const float* rdist, const int32_t* idx, int64_t n, int64_t kq,
                        int64_t min_samples, const float* weights, double* edges,
                        double* core) {
    const int64_t kk = kq - 1; /* neighbours per point without the point itself */
    double* dist = (double*)malloc(sizeof(double) * (size_t)(n * (kk > 0 ? kk : 1)));
    /* kruskal.py:981-1015: core distances and edge lengths */
    for (int64_t i = 0; i < n; ++i) {
        if (weights) {
            /* boruvka.py:528 sample_weight_core_distance on the plain (float32
             * sqrt) distances, self first; index -1 reads the last weight */
            double total = 0.0;
            int64_t j = 0;
            while (total < (double)min_samples && j < kq) {
                const int32_t q = idx[i * kq + j];
                total += (double)weights[q >= 0 ? q : n - 1];
                ++j;
            }
            core[i] = (double)sqrtf(rdist[i * kq + (j - 1)]);
        } else if (min_samples > 1) {
            core[i] = sqrt((double)rdist[i * kq + min_samples]);
        } else {
            core[i] = 0.0;
        }
        for (int64_t j = 1; j < kq; ++j)
            dist[i * kk + j - 1] = weights ? (double)sqrtf(rdist[i * kq + j])
                                           : sqrt((double)rdist[i * kq + j]);
    }
    /* kruskal.py:456 _build_mrd_edges_knn, then :1022 drop self-loops and
     * infinite weights, keeping the edge order */
    const int64_t total = n * kk;
    double* w = (double*)malloc(sizeof(double) * (size_t)(total > 0 ? total : 1));
    int32_t* row = (int32_t*)malloc(sizeof(int32_t) * (size_t)(total > 0 ? total : 1));
    int32_t* col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(total > 0 ? total : 1));
    int64_t m = 0;
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t jp = 0; jp < kk; ++jp) {
            const int32_t j = idx[i * kq + jp + 1];
            double mrd = INFINITY;
            int32_t c = (int32_t)i;
            if (j >= 0) {
                mrd = core[i];
                if (core[j] > mrd) mrd = core[j];
                if (dist[i * kk + jp] > mrd) mrd = dist[i * kk + jp];
                c = j;
            }
            if (c != (int32_t)i && isfinite(mrd)) {
                w[m] = mrd;
                row[m] = (int32_t)i;
                col[m] = c;
                ++m;
            }
        }
    }
    int64_t* order = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
    for (int64_t e = 0; e < m; ++e) order[e] = e;
    g_kr_w = w;
    qsort(order, (size_t)m, sizeof(int64_t), cmp_kr);
    /* kruskal.py:32 _kruskal_core: union by rank with full path compression */
    int32_t* pred = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int32_t* rank = (int32_t*)calloc((size_t)n, sizeof(int32_t));
    for (int64_t i = 0; i < n; ++i) pred[i] = (int32_t)i;
    int64_t n_mst = 0;
    for (int64_t t = 0; t < m && n_mst < n - 1; ++t) {
        const int64_t e = order[t];
        int32_t u = row[e], v = col[e], ru = u, rv = v;
        while (pred[ru] != ru) ru = pred[ru];
        for (int32_t c = u; c != ru;) { const int32_t nx = pred[c]; pred[c] = ru; c = nx; }
        while (pred[rv] != rv) rv = pred[rv];
        for (int32_t c = v; c != rv;) { const int32_t nx = pred[c]; pred[c] = rv; c = nx; }
        if (ru != rv) {
            edges[3 * n_mst + 0] = (double)u;
            edges[3 * n_mst + 1] = (double)v;
            edges[3 * n_mst + 2] = w[e];
            ++n_mst;
            if (rank[ru] > rank[rv]) pred[rv] = ru;
            else if (rank[ru] < rank[rv]) pred[ru] = rv;
            else { pred[rv] = ru; rank[ru] += 1; }
        }
    }
    /* kruskal.py:723 _finish_mst: one representative per component -- its
     * smallest point -- in ascending order, joined by +inf bridges */
    int32_t* rep = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) rep[i] = INT32_MAX;
    for (int64_t i = 0; i < n; ++i) {
        int32_t r = (int32_t)i;
        while (pred[r] != r) r = pred[r];
        if ((int32_t)i < rep[r]) rep[r] = (int32_t)i;
    }
    int64_t prev = -1;
    for (int64_t i = 0; i < n; ++i) { /* representatives are points: visit them in order */
        int32_t r = (int32_t)i;
        while (pred[r] != r) r = pred[r];
        if (rep[r] != (int32_t)i) continue;
        if (prev >= 0) {
            edges[3 * n_mst + 0] = (double)prev;
            edges[3 * n_mst + 1] = (double)i;
            edges[3 * n_mst + 2] = INFINITY;
            ++n_mst;
        }
        prev = i;
    }
    free(rep); free(rank); free(pred); free(order); free(col); free(row); free(w); free(dist);
    return n_mst;
}

/* ------------------------------------------------------------------------- */
/* Precomputed sparse graphs: precomputed.py:479                               */
/* compute_mst_from_precomputed_sparse_kruskal (no cannot-link constraints):   */
/* :70 _symmetrize_min_csr, :148 _core_distances_csr, kruskal.py:755           */
/* kruskal_mst_from_csr (:421 _compute_mrd_csr_flat), :723 _finish_mst.        */
/* ------------------------------------------------------------------------- */

typedef struct { int32_t u, v; double d; int64_t pos; } pc_ent;
static int cmp_pc_uv(const void* a, const void* b) { /* lexsort((v, u)), stable */
    const pc_ent *x = (const pc_ent*)a, *y = (const pc_ent*)b;
    if (x->u != y->u) return x->u < y->u ? -1 : 1;
    if (x->v != y->v) return x->v < y->v ? -1 : 1;
    return (x->pos > y->pos) - (x->pos < y->pos);
}
static int cmp_pc_row(const void* a, const void* b) { /* argsort(rows, kind="stable") */
    const pc_ent *x = (const pc_ent*)a, *y = (const pc_ent*)b;
    if (x->u != y->u) return x->u < y->u ? -1 : 1;
    return (x->pos > y->pos) - (x->pos < y->pos);
}
static const double* g_pc_d;
static int cmp_pc_val(const void* a, const void* b) { /* by value, then position */
    const int64_t i = *(const int64_t*)a, j = *(const int64_t*)b;
    if (g_pc_d[i] != g_pc_d[j]) return g_pc_d[i] < g_pc_d[j] ? -1 : 1;
    return (i > j) - (i < j);
}

int64_t orc_precomputed_kruskal(const int32_t* rows, const int32_t* cols, const double* data,
                                int64_t nnz, int64_t n, int64_t min_samples, double* edges,
                                int32_t* neighbors, double* core) {
    /* _symmetrize_min_csr: min weight per undirected pair, no diagonal */
    pc_ent* e = (pc_ent*)malloc(sizeof(pc_ent) * (size_t)(nnz > 0 ? nnz : 1));
    int64_t m0 = 0;
    for (int64_t t = 0; t < nnz; ++t) {
        if (rows[t] == cols[t]) continue;
        e[m0].u = rows[t] < cols[t] ? rows[t] : cols[t];
        e[m0].v = rows[t] < cols[t] ? cols[t] : rows[t];
        e[m0].d = data[t];
        e[m0].pos = m0;
        ++m0;
    }
    qsort(e, (size_t)m0, sizeof(pc_ent), cmp_pc_uv);
    int64_t m = 0;
    for (int64_t t = 0; t < m0; ++t) {
        if (m > 0 && e[m - 1].u == e[t].u && e[m - 1].v == e[t].v) {
            if (e[t].d < e[m - 1].d) e[m - 1].d = e[t].d; /* np.minimum.reduceat */
        } else {
            e[m++] = e[t];
        }
    }
    const int64_t M = 2 * m;
    pc_ent* sym = (pc_ent*)malloc(sizeof(pc_ent) * (size_t)(M > 0 ? M : 1));
    for (int64_t t = 0; t < m; ++t) {
        sym[t].u = e[t].u; sym[t].v = e[t].v; sym[t].d = e[t].d; sym[t].pos = t;
        sym[m + t].u = e[t].v; sym[m + t].v = e[t].u; sym[m + t].d = e[t].d; sym[m + t].pos = m + t;
    }
    qsort(sym, (size_t)M, sizeof(pc_ent), cmp_pc_row);
    int64_t* indptr = (int64_t*)calloc((size_t)(n + 1), sizeof(int64_t));
    for (int64_t t = 0; t < M; ++t) indptr[sym[t].u + 1] += 1;
    for (int64_t i = 0; i < n; ++i) indptr[i + 1] += indptr[i];
    double* sd = (double*)malloc(sizeof(double) * (size_t)(M > 0 ? M : 1));
    int32_t* sc = (int32_t*)malloc(sizeof(int32_t) * (size_t)(M > 0 ? M : 1));
    for (int64_t t = 0; t < M; ++t) { sd[t] = sym[t].d; sc[t] = sym[t].v; }
    /* _core_distances_csr: rows ordered by weight (ties by position) */
    const int64_t k = min_samples > 1 ? min_samples : 1;
    int64_t* order = (int64_t*)malloc(sizeof(int64_t) * (size_t)(M > 0 ? M : 1));
    g_pc_d = sd;
    for (int64_t i = 0; i < n; ++i) {
        const int64_t s0 = indptr[i], deg = indptr[i + 1] - s0;
        for (int64_t j = 0; j < k; ++j) neighbors[i * k + j] = -1;
        core[i] = 0.0;
        if (deg == 0) {
            if (min_samples > 1) core[i] = INFINITY;
            continue;
        }
        for (int64_t j = 0; j < deg; ++j) order[j] = s0 + j;
        qsort(order, (size_t)deg, sizeof(int64_t), cmp_pc_val);
        const int64_t fill = k < deg ? k : deg;
        for (int64_t j = 0; j < fill; ++j) neighbors[i * k + j] = sc[order[j]];
        if (min_samples > 1) core[i] = deg >= min_samples ? sd[order[min_samples - 1]] : INFINITY;
    }
    /* kruskal.py:421 _compute_mrd_csr_flat, stable argsort, :32 _kruskal_core */
    double* w = (double*)malloc(sizeof(double) * (size_t)(M > 0 ? M : 1));
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t p = indptr[i]; p < indptr[i + 1]; ++p) {
            double mrd = core[i];
            if (core[sc[p]] > mrd) mrd = core[sc[p]];
            if (sd[p] > mrd) mrd = sd[p];
            w[p] = mrd;
        }
    }
    for (int64_t p = 0; p < M; ++p) order[p] = p;
    g_pc_d = w;
    qsort(order, (size_t)M, sizeof(int64_t), cmp_pc_val);
    int32_t* pred = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int32_t* rank = (int32_t*)calloc((size_t)(n > 0 ? n : 1), sizeof(int32_t));
    for (int64_t i = 0; i < n; ++i) pred[i] = (int32_t)i;
    int64_t n_mst = 0;
    for (int64_t t = 0; t < M && n_mst < n - 1; ++t) {
        const int64_t p = order[t];
        const int32_t u = sym[p].u, v = sc[p];
        if (u == v) continue;
        int32_t ru = u, rv = v;
        while (pred[ru] != ru) ru = pred[ru];
        for (int32_t c = u; c != ru;) { const int32_t nx = pred[c]; pred[c] = ru; c = nx; }
        while (pred[rv] != rv) rv = pred[rv];
        for (int32_t c = v; c != rv;) { const int32_t nx = pred[c]; pred[c] = rv; c = nx; }
        if (ru != rv) {
            edges[3 * n_mst + 0] = (double)u;
            edges[3 * n_mst + 1] = (double)v;
            edges[3 * n_mst + 2] = w[p];
            ++n_mst;
            if (rank[ru] > rank[rv]) pred[rv] = ru;
            else if (rank[ru] < rank[rv]) pred[ru] = rv;
            else { pred[rv] = ru; rank[ru] += 1; }
        }
    }
    /* _finish_mst: +inf bridges between the smallest points of the components */
    int32_t* rep = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) rep[i] = INT32_MAX;
    for (int64_t i = 0; i < n; ++i) {
        int32_t r = (int32_t)i;
        while (pred[r] != r) r = pred[r];
        if ((int32_t)i < rep[r]) rep[r] = (int32_t)i;
    }
    int64_t prev = -1;
    for (int64_t i = 0; i < n; ++i) {
        int32_t r = (int32_t)i;
        while (pred[r] != r) r = pred[r];
        if (rep[r] != (int32_t)i) continue;
        if (prev >= 0) {
            edges[3 * n_mst + 0] = (double)prev;
            edges[3 * n_mst + 1] = (double)i;
            edges[3 * n_mst + 2] = INFINITY;
            ++n_mst;
        }
        prev = i;
    }
    free(rep); free(rank); free(pred); free(w); free(order); free(sc); free(sd); free(indptr);
    free(sym); free(e);
    return n_mst;
}
