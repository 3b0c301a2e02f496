// extern "C" entry points of libfhg.so (declared in include/fhg.h).
#include <atomic>
#include <cstdarg>
#include <map>
#include <mutex>

#include "index.cuh"
#include "highd.cuh"
#include "mst.cuh"
#include "radius.cuh"
#include "reftree.cuh"
#include "trees.cuh"

#include <initializer_list>

namespace fhg {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
}
const char* last_error() { return g_last_error.c_str(); }

// Sizes and counts: zero is an empty input, a negative value a caller error.
int check_counts(const char* fn, std::initializer_list<int64_t> cs) {
    for (int64_t c : cs)
        if (c < 0) {
            set_error("%s: negative size or count (%lld)", fn, (long long)c);
            return FHG_ERR_INVALID;
        }
    return FHG_OK;
}

int finalize_edges(const MstResult& r, double* edges, cudaStream_t s);

// ---------------------------------------------------------------- tracing
static std::atomic<uint64_t> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

namespace {
struct StageRec {
    std::string name;
    cudaEvent_t a, b;
};
std::atomic<bool> g_prof_on{false};
std::mutex g_prof_mu;
std::vector<StageRec> g_prof;
std::map<std::string, std::pair<double, int64_t>> g_counts;  // name -> (sum, samples)
}  // namespace

void profile_count(const char* name, double value) {
    if (!g_prof_on.load(std::memory_order_relaxed)) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    auto& e = g_counts[name];
    e.first += value;
    e.second += 1;
}

Stage::Stage(cudaStream_t s, const char* name) : s_(s), name_(name) {
    if (!g_prof_on.load(std::memory_order_relaxed)) return;
    if (cudaEventCreate(&a_) != cudaSuccess) {
        a_ = nullptr;
        return;
    }
    cudaEventRecord(a_, s_);
}

Stage::~Stage() {
    if (!a_) return;
    cudaEvent_t b;
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a_);
        return;
    }
    cudaEventRecord(b, s_);
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof.push_back(StageRec{name_, a_, b});
}

constexpr int kMaxDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pools[kMaxDevices] = {};

int device_pool(cudaMemPool_t* out) {
    int dev = -1;
    FHG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("device %d out of range", dev);
        return FHG_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pools[dev]) {
        cudaMemPoolProps props;
        memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        FHG_CUDA(cudaMemPoolCreate(&pool, &props));
        uint64_t keep = UINT64_MAX;
        FHG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
        g_pools[dev] = pool;
    }
    *out = g_pools[dev];
    return FHG_OK;
}

}  // namespace fhg

using namespace fhg;

#define FHG_API extern "C" __attribute__((visibility("default")))

static inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

FHG_API const char* fhg_last_error(void) { return last_error(); }
FHG_API int fhg_abi_version(void) { return 2; }

FHG_API uint64_t fhg_launch_count(void) { return g_launches.load(); }

FHG_API int fhg_release_cached_memory(void) {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (int d = 0; d < kMaxDevices; ++d)
        if (g_pools[d]) FHG_CUDA(cudaMemPoolTrimTo(g_pools[d], 0));
    return FHG_OK;
}

FHG_API int fhg_set_tie_rule(int rule) {
    if (rule != FHG_TIES_CANONICAL && rule != FHG_TIES_REFERENCE) {
        set_error("fhg_set_tie_rule: unknown rule %d", rule);
        return -1;
    }
    return set_tie_rule(rule);
}

FHG_API int fhg_set_highd_kernel(int kernel) {
    if (kernel != FHG_HD_TCGEN05 && kernel != FHG_HD_MMA_SYNC) {
        set_error("fhg_set_highd_kernel: unknown kernel %d", kernel);
        return -1;
    }
    return highd_use_legacy(kernel == FHG_HD_MMA_SYNC ? 1 : 0);
}

FHG_API int fhg_profile_enable(int on) {
    g_prof_on.store(on != 0);
    return FHG_OK;
}

FHG_API int fhg_profile_report(char* buf, int64_t cap) {
    std::vector<StageRec> recs;
    std::map<std::string, std::pair<double, int64_t>> agg;
    {
        std::lock_guard<std::mutex> lk(g_prof_mu);
        recs.swap(g_prof);
        agg.swap(g_counts);
    }
    int rc = FHG_OK;
    for (auto& r : recs) {
        float ms = 0.0f;
        if (cudaEventSynchronize(r.b) != cudaSuccess ||
            cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) {
            set_error("profile: event timing failed");
            rc = FHG_ERR_CUDA;
        }
        auto& e = agg[r.name];
        e.first += ms;
        e.second += 1;
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    std::string out = "{";
    bool first = true;
    for (auto& kv : agg) {
        char item[256];
        snprintf(item, sizeof item, "%s\"%s\": [%.6f, %lld]", first ? "" : ", ", kv.first.c_str(),
                 kv.second.first, (long long)kv.second.second);
        out += item;
        first = false;
    }
    out += "}";
    if (buf && cap > 0) {
        size_t n = out.size() < (size_t)(cap - 1) ? out.size() : (size_t)(cap - 1);
        memcpy(buf, out.data(), n);
        buf[n] = 0;
    }
    return rc;
}

FHG_API int fhg_index_build(const float* X_dev, int64_t n, int32_t d, void* stream,
                            fhg_index** out) {
    if (!out || !X_dev) {
        set_error("fhg_index_build: null pointer");
        return FHG_ERR_INVALID;
    }
    return index_build(X_dev, n, d, as_stream(stream), out);
}

FHG_API int32_t fhg_reference_kdtree_levels(int64_t n) { return ref_tree_levels(n); }

FHG_API int fhg_reference_kdtree(const float* X_dev, int64_t n, int32_t d, int32_t* idx_array_dev,
                                 float* node_bounds_dev, void* stream) {
    if (!X_dev || (!idx_array_dev && !node_bounds_dev)) {
        set_error("fhg_reference_kdtree: null pointer");
        return FHG_ERR_INVALID;
    }
    cudaStream_t s = as_stream(stream);
    fhg_index* ix = nullptr;
    FHG_TRY(index_build(X_dev, n, d, s, &ix));
    int rc;
    {
        Workspace ws(s);
        RefTree t;
        rc = ref_tree_build(ws, *ix, &t);
        if (rc == FHG_OK) rc = ref_tree_export(t, idx_array_dev, node_bounds_dev, s);
    }
    const int rc2 = index_free(ix, s);
    return rc != FHG_OK ? rc : rc2;
}

FHG_API int fhg_index_free(fhg_index* index, void* stream) {
    return index_free(index, as_stream(stream));
}

FHG_API int fhg_index_shape(const fhg_index* index, int64_t* n, int32_t* d) {
    if (!index) {
        set_error("fhg_index_shape: null index");
        return FHG_ERR_INVALID;
    }
    if (n) *n = index->n;
    if (d) *d = index->d;
    return FHG_OK;
}

FHG_API int fhg_index_knn(fhg_index* index, int32_t k, float* rdist_dev, int32_t* idx_dev,
                          void* stream) {
    if (!index || !rdist_dev || !idx_dev) {
        set_error("fhg_index_knn: null pointer");
        return FHG_ERR_INVALID;
    }
    return index_knn(*index, k, nullptr, nullptr, rdist_dev, idx_dev, as_stream(stream));
}

// ------------------------------------------------------ learned radius
FHG_API int fhg_radius_param_count(void) { return kRadiusParams; }

FHG_API int fhg_radius_features(fhg_index* index, float* feat_dev, void* stream) {
    if (!index || !feat_dev) {
        set_error("fhg_radius_features: null pointer");
        return FHG_ERR_INVALID;
    }
    return radius_features(*index, index->orig, feat_dev, as_stream(stream));
}

FHG_API int fhg_radius_targets(fhg_index* index, int32_t k, float* target_dev, void* stream) {
    if (!index || !target_dev) {
        set_error("fhg_radius_targets: null pointer");
        return FHG_ERR_INVALID;
    }
    if (k < 1 || k > 64) {
        set_error("fhg_radius_targets: k must be in [1, 64] (got %d)", k);
        return FHG_ERR_INVALID;
    }
    return radius_targets(*index, k, target_dev, as_stream(stream));
}

FHG_API int fhg_radius_init(float* params_dev, const float* feat_dev, const float* target_dev,
                            int64_t n, uint64_t seed, void* stream) {
    if (!params_dev || !feat_dev || !target_dev) {
        set_error("fhg_radius_init: null pointer");
        return FHG_ERR_INVALID;
    }
    return radius_init(params_dev, feat_dev, target_dev, n, seed, as_stream(stream));
}

FHG_API int fhg_radius_forward(const float* params_dev, const float* feat_dev, int64_t n,
                               float* log_radius_dev, void* stream) {
    if (!params_dev || !feat_dev || !log_radius_dev) {
        set_error("fhg_radius_forward: null pointer");
        return FHG_ERR_INVALID;
    }
    return radius_predict(params_dev, feat_dev, n, 1.0f, log_radius_dev, nullptr,
                          as_stream(stream));
}

FHG_API int fhg_radius_backward(const float* params_dev, const float* feat_dev,
                                const float* target_dev, const int32_t* rows_dev, int64_t batch,
                                float* grad_dev, float* loss_dev, void* stream) {
    if (!params_dev || !feat_dev || !target_dev || !rows_dev || !grad_dev || !loss_dev) {
        set_error("fhg_radius_backward: null pointer");
        return FHG_ERR_INVALID;
    }
    return radius_grad(params_dev, feat_dev, target_dev, rows_dev, batch, grad_dev, loss_dev,
                       as_stream(stream));
}

FHG_API int fhg_radius_train(float* params_dev, const float* feat_dev, const float* target_dev,
                             int64_t n, int32_t steps, int32_t batch, float lr, uint64_t seed,
                             float* loss_curve_dev, void* stream) {
    if (!params_dev || !feat_dev || !target_dev) {
        set_error("fhg_radius_train: null pointer");
        return FHG_ERR_INVALID;
    }
    return radius_train(params_dev, feat_dev, target_dev, n, steps, batch, lr, seed,
                        loss_curve_dev, as_stream(stream));
}

FHG_API int fhg_radius_use(const float* params_dev, float margin) {
    if (params_dev && !(margin > 0.0f)) {
        set_error("fhg_radius_use: margin must be positive");
        return FHG_ERR_INVALID;
    }
    radius_set_use(params_dev, margin);
    return FHG_OK;
}

FHG_API int fhg_radius_fallbacks(int64_t* count_host, void* stream) {
    if (!count_host) {
        set_error("fhg_radius_fallbacks: null pointer");
        return FHG_ERR_INVALID;
    }
    return radius_last_fallbacks(count_host, as_stream(stream));
}

FHG_API int fhg_index_knn_radius(fhg_index* index, int32_t k, const float* params_dev,
                                 float margin, float* rdist_dev, int32_t* idx_dev,
                                 int64_t* fallbacks_host, void* stream) {
    if (!index || !params_dev || !rdist_dev || !idx_dev) {
        set_error("fhg_index_knn_radius: null pointer");
        return FHG_ERR_INVALID;
    }
    if (!(margin > 0.0f)) {
        set_error("fhg_index_knn_radius: margin must be positive");
        return FHG_ERR_INVALID;
    }
    cudaStream_t s = as_stream(stream);
    RadiusUse use;
    use.params = params_dev;
    use.margin = margin;
    FHG_TRY(knn_with_radius(*index, k, use, nullptr, nullptr, rdist_dev, idx_dev, s));
    if (fallbacks_host) return radius_last_fallbacks(fallbacks_host, s);
    return FHG_OK;
}

FHG_API int fhg_knn_scan_count(fhg_index* index, int32_t k, const float* params_dev, float margin,
                               int64_t* scans_host, int64_t* fallbacks_host, void* stream) {
    if (!index || !scans_host) {
        set_error("fhg_knn_scan_count: null pointer");
        return FHG_ERR_INVALID;
    }
    if (k < 1 || k > 64) {
        set_error("knn: k must be in [1, 64] (got %d)", k);
        return FHG_ERR_INVALID;
    }
    return knn_scan_count(*index, k, params_dev, margin, scans_host, fallbacks_host,
                          as_stream(stream));
}

FHG_API int fhg_highd_knn(const float* X_dev, int64_t n, int32_t d, int32_t k, float* rdist_dev,
                          int32_t* idx_dev, int64_t* fallbacks_host, void* stream) {
    if (n > 0 && (!X_dev || !rdist_dev || !idx_dev)) {
        set_error("fhg_highd_knn: null pointer");
        return FHG_ERR_INVALID;
    }
    return highd_knn(X_dev, n, d, k, rdist_dev, idx_dev, fallbacks_host, as_stream(stream));
}

FHG_API int fhg_knn_graph_mst(const float* X_dev, int64_t n, int32_t d, int32_t min_samples,
                              int32_t knn_k, double* edges_dev, int32_t* neighbors_dev,
                              double* core_dev, int64_t* n_components_host, void* stream) {
    if (n > 0 && (!X_dev || !edges_dev || !core_dev || !n_components_host)) {
        set_error("fhg_knn_graph_mst: null pointer");
        return FHG_ERR_INVALID;
    }
    if (min_samples < 1 || knn_k < min_samples) {
        set_error("fhg_knn_graph_mst: needs 1 <= min_samples <= knn_k (got %d, %d)", min_samples,
                  knn_k);
        return FHG_ERR_INVALID;
    }
    return kruskal_mst_of_lists(n, min_samples, knn_k + 1, nullptr, nullptr, X_dev, d, edges_dev,
                                neighbors_dev, core_dev, n_components_host, as_stream(stream));
}

FHG_API int fhg_core_graph_mst(const int32_t* indptr_dev, const int32_t* indices_dev,
                               const float* weights_dev, const int32_t* seg_end_dev, int64_t n,
                               double* edges_dev, int64_t* n_edges_host, void* stream) {
    FHG_TRY(check_counts("fhg_core_graph_mst", {n}));
    if (!n_edges_host || (n > 1 && (!indptr_dev || !indices_dev || !weights_dev || !edges_dev))) {
        set_error("fhg_core_graph_mst: null pointer");
        return FHG_ERR_INVALID;
    }
    return core_graph_boruvka(n, indptr_dev, indices_dev, weights_dev, seg_end_dev, edges_dev,
                              n_edges_host, as_stream(stream));
}

FHG_API int fhg_propagate_labels(int64_t n_clusters, const int32_t* noise_first_dev,
                                 const int32_t* noise_pt_dev, const int32_t* adj_ptr_dev,
                                 const int32_t* adj_other_dev, const double* adj_w_dev,
                                 int32_t* labels_dev, void* stream) {
    if (n_clusters < 0) {
        set_error("fhg_propagate_labels: negative cluster count");
        return FHG_ERR_INVALID;
    }
    if (n_clusters > 0 && (!noise_first_dev || !noise_pt_dev || !adj_ptr_dev || !adj_other_dev ||
                           !adj_w_dev || !labels_dev)) {
        set_error("fhg_propagate_labels: null pointer");
        return FHG_ERR_INVALID;
    }
    return propagate_labels(n_clusters, noise_first_dev, noise_pt_dev, adj_ptr_dev, adj_other_dev,
                            adj_w_dev, labels_dev, as_stream(stream));
}

FHG_API int fhg_core_graphs(int64_t P, int32_t k, const int32_t* nb_dev, const double* lens_dev,
                            const float* core_dev, const int32_t* blk_start_dev,
                            const int32_t* blk_end_dev, int64_t M, const int32_t* mparent_dev,
                            const int32_t* mchild_dev, const double* mdist_dev,
                            int32_t* indptr_dev, int32_t* idx_local_dev, int32_t* idx_block_dev,
                            float* weights_dev, float* distances_dev, int32_t* seg_end_dev,
                            int64_t* nnz_host, void* stream) {
    if (!nnz_host || (P > 0 && (!nb_dev || !lens_dev || !core_dev || !blk_start_dev ||
                                !blk_end_dev || !indptr_dev || !idx_local_dev || !idx_block_dev ||
                                !weights_dev || !distances_dev || !seg_end_dev)) ||
        (M > 0 && (!mparent_dev || !mchild_dev || !mdist_dev))) {
        set_error("fhg_core_graphs: null pointer");
        return FHG_ERR_INVALID;
    }
    if (k < 0 || M < 0) {
        set_error("fhg_core_graphs: negative size");
        return FHG_ERR_INVALID;
    }
    return core_graphs_layout(P, k, nb_dev, lens_dev, core_dev, blk_start_dev, blk_end_dev, M,
                              mparent_dev, mchild_dev, mdist_dev, indptr_dev, idx_local_dev,
                              idx_block_dev, weights_dev, distances_dev, seg_end_dev, nnz_host,
                              as_stream(stream));
}

FHG_API int fhg_index_boruvka(fhg_index* index, int32_t min_samples,
                              const float* sample_weights_dev, int32_t weighted_k,
                              double* edges_dev, int32_t* neighbors_dev, float* core_dev,
                              int32_t* n_rounds_host, void* stream) {
    if (!index || !edges_dev || !neighbors_dev || !core_dev) {
        set_error("fhg_index_boruvka: null pointer");
        return FHG_ERR_INVALID;
    }
    if (min_samples < 1) {
        set_error("min_samples must be a positive integer");
        return FHG_ERR_INVALID;
    }
    cudaStream_t s = as_stream(stream);
    Workspace ws(s);
    MstResult r;
    FHG_TRY(boruvka_mst(ws, *index, min_samples, &r, core_dev, neighbors_dev, sample_weights_dev,
                        weighted_k));
    FHG_TRY(finalize_edges(r, edges_dev, s));
    if (n_rounds_host) *n_rounds_host = r.rounds;
    if (r.m != index->n - 1 && index->n > 1) {
        set_error("boruvka: spanning forest has %lld edges for %lld points", (long long)r.m,
                  (long long)index->n);
        return FHG_ERR_NO_CONVERGENCE;
    }
    return FHG_OK;
}

FHG_API int fhg_index_kruskal_knn(fhg_index* index, int32_t min_samples, int32_t query_k,
                                  const float* sample_weights_dev, double* edges_dev,
                                  int32_t* neighbors_dev, double* core_dev,
                                  int64_t* n_components_host, void* stream) {
    if (!index || !edges_dev || !core_dev) {
        set_error("fhg_index_kruskal_knn: null pointer");
        return FHG_ERR_INVALID;
    }
    if (min_samples < 1) {
        set_error("min_samples must be a positive integer");
        return FHG_ERR_INVALID;
    }
    int64_t nc = 0;
    FHG_TRY(kruskal_knn_mst(*index, min_samples, query_k, sample_weights_dev, edges_dev,
                            neighbors_dev, core_dev, &nc, as_stream(stream)));
    if (n_components_host) *n_components_host = nc;
    return FHG_OK;
}

FHG_API int fhg_precomputed_mst(const int32_t* rows_dev, const int32_t* cols_dev,
                                const double* data_dev, int64_t nnz, int64_t n,
                                int32_t min_samples, int32_t algorithm, double* edges_dev,
                                int32_t* neighbors_dev, double* core_dev,
                                int64_t* n_components_host, void* stream) {
    if (n < 0 || nnz < 0 || (nnz > 0 && (!rows_dev || !cols_dev || !data_dev)) ||
        (n > 0 && (!neighbors_dev || !core_dev)) || (n > 1 && !edges_dev)) {
        set_error("fhg_precomputed_mst: invalid sizes or null pointer");
        return FHG_ERR_INVALID;
    }
    if (algorithm != 0 && algorithm != 1) {
        set_error("fhg_precomputed_mst: algorithm must be 0 (boruvka) or 1 (kruskal)");
        return FHG_ERR_INVALID;
    }
    if (n > 0x7fffffffLL) {
        set_error("fhg_precomputed_mst: %lld points exceed int32 indices", (long long)n);
        return FHG_ERR_UNSUPPORTED;
    }
    int64_t nc = 0;
    FHG_TRY(precomputed_mst(rows_dev, cols_dev, data_dev, nnz, n,
                            min_samples > 0 ? min_samples : 1, edges_dev, neighbors_dev,
                            core_dev, &nc, as_stream(stream)));
    if (n_components_host) *n_components_host = nc;
    return FHG_OK;
}

// ------------------------------------------------------------- tree passes
namespace fhg {
namespace capi {

__global__ void widen_sel_kernel(int64_t k, const int32_t* __restrict__ a, int64_t* __restrict__ b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < k) b[i] = a[i];
}
__global__ void narrow_sel_kernel(int64_t k, const int64_t* __restrict__ a, int32_t* __restrict__ b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < k) b[i] = (int32_t)a[i];
}
__global__ void fill_labels_kernel(int64_t n, int64_t* __restrict__ labels, float* __restrict__ probs) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        labels[i] = -1;
        probs[i] = 0.0f;
    }
}

int check_ptrs(const char* fn, std::initializer_list<const void*> ps) {
    for (const void* p : ps)
        if (!p) {
            set_error("%s: null pointer argument", fn);
            return FHG_ERR_INVALID;
        }
    return FHG_OK;
}

}  // namespace capi
}  // namespace fhg
using namespace fhg::capi;

FHG_API int fhg_sort_mst(const double* mst_dev, int64_t m, double* sorted_dev, void* stream) {
    FHG_TRY(check_counts("fhg_sort_mst", {m}));
    if (m == 0) return FHG_OK;
    FHG_TRY(check_ptrs("fhg_sort_mst", {mst_dev, sorted_dev}));
    cudaStream_t s = as_stream(stream);
    Workspace ws(s);
    int32_t *src, *dst;
    double* w;
    FHG_TRY(split_mst_f64(ws, mst_dev, m, &src, &dst, &w));
    Linkage lk;
    FHG_TRY(sort_and_link(ws, m + 1, src, dst, w, nullptr, &lk));
    return sorted_mst_to_f64(lk, sorted_dev, s);
}

FHG_API int fhg_mst_to_linkage_tree(const double* sorted_mst_dev, int64_t m,
                                    const float* sample_weights_dev, double* linkage_dev,
                                    void* stream) {
    FHG_TRY(check_counts("fhg_mst_to_linkage_tree", {m}));
    if (m == 0) return FHG_OK;
    FHG_TRY(check_ptrs("fhg_mst_to_linkage_tree", {sorted_mst_dev, linkage_dev}));
    cudaStream_t s = as_stream(stream);
    Workspace ws(s);
    int32_t *src, *dst;
    double* w;
    FHG_TRY(split_mst_f64(ws, sorted_mst_dev, m, &src, &dst, &w));
    Linkage lk;
    FHG_TRY(sort_and_link(ws, m + 1, src, dst, w, nullptr, &lk, /*presorted=*/true));
    if (sample_weights_dev) FHG_TRY(weighted_sizes(ws, lk, sample_weights_dev));
    return linkage_to_f64(lk, linkage_dev, s);
}

FHG_API int fhg_condense_tree(const double* linkage_dev, int64_t m, int64_t min_cluster_size,
                              double max_cluster_size, const float* sample_weights_dev,
                              int64_t* parent_dev, int64_t* child_dev, float* lambda_dev,
                              float* child_size_dev, int64_t* n_rows_host, void* stream) {
    FHG_TRY(check_ptrs("fhg_condense_tree", {n_rows_host}));
    *n_rows_host = 0;
    FHG_TRY(check_counts("fhg_condense_tree", {m}));
    if (m == 0) return FHG_OK;
    FHG_TRY(check_ptrs("fhg_condense_tree",
                       {linkage_dev, parent_dev, child_dev, lambda_dev, child_size_dev}));
    if (min_cluster_size <= 0) {
        set_error("min_cluster_size must be a positive integer");
        return FHG_ERR_INVALID;
    }
    cudaStream_t s = as_stream(stream);
    Workspace ws(s);
    Linkage lk;
    FHG_TRY(linkage_from_f64(ws, linkage_dev, m, &lk));
    if (sample_weights_dev) {
        // the size column holds weight sums: leaf counts come from the rows
        FHG_TRY(linkage_leaf_counts(ws, lk));
        FHG_TRY(weighted_sizes(ws, lk, sample_weights_dev));
    }
    Condensed ct;
    FHG_TRY(condense_tree(ws, lk, min_cluster_size, max_cluster_size, &ct));
    FHG_TRY(condensed_to_arrays(ct, parent_dev, child_dev, lambda_dev, child_size_dev, s));
    *n_rows_host = ct.rows;
    return FHG_OK;
}

FHG_API int fhg_extract_eom_clusters(const int64_t* parent_dev, const int64_t* child_dev,
                                     const float* lambda_dev, const float* child_size_dev,
                                     int64_t rows, double max_cluster_size,
                                     int allow_single_cluster, int64_t* sel_dev,
                                     int64_t* n_sel_host, void* stream) {
    FHG_TRY(check_ptrs("fhg_extract_eom_clusters", {n_sel_host}));
    *n_sel_host = 0;
    FHG_TRY(check_counts("fhg_extract_eom_clusters", {rows}));
    if (rows == 0) return FHG_OK;
    FHG_TRY(check_ptrs("fhg_extract_eom_clusters",
                       {parent_dev, child_dev, lambda_dev, child_size_dev, sel_dev}));
    cudaStream_t s = as_stream(stream);
    Workspace ws(s);
    Condensed ct;
    FHG_TRY(condensed_from_arrays(ws, parent_dev, child_dev, lambda_dev, child_size_dev, rows, &ct));
    int32_t* sel;
    FHG_TRY(ws.alloc(&sel, (size_t)ct.n_clusters));
    int64_t k = 0;
    FHG_TRY(select_eom(ws, ct, max_cluster_size, allow_single_cluster != 0, sel, &k));
    if (k > 0) {
        ::fhg::note_launch();
        widen_sel_kernel<<<grid_for(k, 256), 256, 0, s>>>(k, sel, sel_dev);
        FHG_CUDA(cudaGetLastError());
    }
    *n_sel_host = k;
    return FHG_OK;
}

FHG_API int fhg_label_points(const int64_t* parent_dev, const int64_t* child_dev,
                             const float* lambda_dev, const float* child_size_dev, int64_t rows,
                             const int64_t* sel_dev, int64_t n_sel, double epsilon,
                             int64_t n_samples, int64_t* labels_dev, float* probs_dev,
                             void* stream) {
    FHG_TRY(check_counts("fhg_label_points", {rows, n_sel, n_samples}));
    if (n_samples == 0) return FHG_OK;
    FHG_TRY(check_ptrs("fhg_label_points", {labels_dev, probs_dev}));
    cudaStream_t s = as_stream(stream);
    if (rows == 0 || n_sel == 0) {
        ::fhg::note_launch();
        fill_labels_kernel<<<grid_for(n_samples, 256), 256, 0, s>>>(n_samples, labels_dev, probs_dev);
        FHG_CUDA(cudaGetLastError());
        return FHG_OK;
    }
    FHG_TRY(check_ptrs("fhg_label_points", {parent_dev, child_dev, lambda_dev, child_size_dev,
                                            sel_dev}));
    Workspace ws(s);
    Condensed ct;
    FHG_TRY(condensed_from_arrays(ws, parent_dev, child_dev, lambda_dev, child_size_dev, rows, &ct));
    if (ct.n != n_samples) {
        set_error("fhg_label_points: n_samples (%lld) must equal the root label (%lld)",
                  (long long)n_samples, (long long)ct.n);
        return FHG_ERR_INVALID;
    }
    int32_t* sel;
    FHG_TRY(ws.alloc(&sel, (size_t)n_sel));
    ::fhg::note_launch();
    narrow_sel_kernel<<<grid_for(n_sel, 256), 256, 0, s>>>(n_sel, sel_dev, sel);
    FHG_CUDA(cudaGetLastError());
    return label_points(ws, ct, sel, n_sel, epsilon, labels_dev, probs_dev);
}

FHG_API int fhg_cluster_tree_leaves(const int64_t* parent_dev, const int64_t* child_dev,
                                    const float* lambda_dev, const float* child_size_dev,
                                    int64_t rows, int64_t* sel_dev, int64_t* n_sel_host,
                                    void* stream) {
    FHG_TRY(check_ptrs("fhg_cluster_tree_leaves", {n_sel_host}));
    *n_sel_host = 0;
    FHG_TRY(check_counts("fhg_cluster_tree_leaves", {rows}));
    if (rows == 0) return FHG_OK;
    FHG_TRY(check_ptrs("fhg_cluster_tree_leaves",
                       {parent_dev, child_dev, lambda_dev, child_size_dev, sel_dev}));
    cudaStream_t s = as_stream(stream);
    Workspace ws(s);
    Condensed ct;
    FHG_TRY(condensed_from_arrays(ws, parent_dev, child_dev, lambda_dev, child_size_dev, rows, &ct));
    int32_t* sel;
    FHG_TRY(ws.alloc(&sel, (size_t)ct.n_clusters));
    int64_t k = 0;
    FHG_TRY(select_leaf(ws, ct, sel, &k));
    if (k > 0) {
        ::fhg::note_launch();
        widen_sel_kernel<<<grid_for(k, 256), 256, 0, s>>>(k, sel, sel_dev);
        FHG_CUDA(cudaGetLastError());
    }
    *n_sel_host = k;
    return FHG_OK;
}

FHG_API int fhg_membership_strengths(const int64_t* parent_dev, const int64_t* child_dev,
                                     const float* lambda_dev, const float* child_size_dev,
                                     int64_t rows, const int64_t* sel_dev, int64_t n_sel,
                                     const int64_t* labels_dev, int64_t n_samples,
                                     float* probs_dev, void* stream) {
    FHG_TRY(check_counts("fhg_membership_strengths", {rows, n_sel, n_samples}));
    if (n_samples == 0) return FHG_OK;
    FHG_TRY(check_ptrs("fhg_membership_strengths", {labels_dev, probs_dev}));
    cudaStream_t s = as_stream(stream);
    FHG_CUDA(cudaMemsetAsync(probs_dev, 0, sizeof(float) * n_samples, s));
    if (rows == 0 || n_sel == 0) return FHG_OK;
    FHG_TRY(check_ptrs("fhg_membership_strengths",
                       {parent_dev, child_dev, lambda_dev, child_size_dev, sel_dev}));
    Workspace ws(s);
    Condensed ct;
    FHG_TRY(condensed_from_arrays(ws, parent_dev, child_dev, lambda_dev, child_size_dev, rows, &ct));
    if (ct.n > n_samples) {
        set_error("fhg_membership_strengths: labels hold %lld points, the tree %lld",
                  (long long)n_samples, (long long)ct.n);
        return FHG_ERR_INVALID;
    }
    int32_t* sel;
    FHG_TRY(ws.alloc(&sel, (size_t)n_sel));
    ::fhg::note_launch();
    narrow_sel_kernel<<<grid_for(n_sel, 256), 256, 0, s>>>(n_sel, sel_dev, sel);
    FHG_CUDA(cudaGetLastError());
    return membership_strengths(ws, ct, sel, n_sel, labels_dev, probs_dev);
}

// ------------------------------------------------------ record array layout
namespace fhg {
namespace capi {
// One 28-byte record per row: int64 parent, int64 child, float64 lambda,
// float32 size -- numpy's packed layout of the dtype to_numpy_rec_array
// builds.  Rows start at 4-byte boundaries, so each is written as 7 words.
__global__ void condensed_records_kernel(int64_t rows, const int64_t* __restrict__ parent,
                                         const int64_t* __restrict__ child,
                                         const float* __restrict__ lambda,
                                         const float* __restrict__ size,
                                         uint32_t* __restrict__ out) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const uint64_t p = (uint64_t)parent[r], c = (uint64_t)child[r];
    const uint64_t l = (uint64_t)__double_as_longlong((double)lambda[r]);
    uint32_t* o = out + 7 * r;
    o[0] = (uint32_t)p;
    o[1] = (uint32_t)(p >> 32);
    o[2] = (uint32_t)c;
    o[3] = (uint32_t)(c >> 32);
    o[4] = (uint32_t)l;
    o[5] = (uint32_t)(l >> 32);
    o[6] = __float_as_uint(size[r]);
}
}  // namespace capi
}  // namespace fhg

FHG_API int fhg_condensed_record_array(const int64_t* parent_dev, const int64_t* child_dev,
                                       const float* lambda_dev, const float* child_size_dev,
                                       int64_t rows, void* records_dev, void* stream) {
    FHG_TRY(check_counts("fhg_condensed_record_array", {rows}));
    if (rows == 0) return FHG_OK;
    FHG_TRY(check_ptrs("fhg_condensed_record_array",
                       {parent_dev, child_dev, lambda_dev, child_size_dev, records_dev}));
    if (reinterpret_cast<uintptr_t>(records_dev) % 4 != 0) {
        set_error("fhg_condensed_record_array: records_dev must be 4-byte aligned");
        return FHG_ERR_INVALID;
    }
    cudaStream_t s = as_stream(stream);
    ::fhg::note_launch();
    fhg::capi::condensed_records_kernel<<<grid_for(rows, 256), 256, 0, s>>>(
        rows, parent_dev, child_dev, lambda_dev, child_size_dev,
        static_cast<uint32_t*>(records_dev));
    FHG_CUDA(cudaGetLastError());
    return FHG_OK;
}

// --------------------------------------------------------- selection options
FHG_API int fhg_simplify_hierarchy(int64_t* parent_dev, int64_t* child_dev, float* lambda_dev,
                                   const float* child_size_dev, int64_t rows, double threshold,
                                   int64_t* out_parent_dev, int64_t* out_child_dev,
                                   float* out_lambda_dev, float* out_child_size_dev,
                                   int64_t* out_rows_host, void* stream) {
    FHG_TRY(check_ptrs("fhg_simplify_hierarchy", {out_rows_host}));
    *out_rows_host = 0;
    FHG_TRY(check_counts("fhg_simplify_hierarchy", {rows}));
    if (rows == 0) return FHG_OK;
    FHG_TRY(check_ptrs("fhg_simplify_hierarchy",
                       {parent_dev, child_dev, lambda_dev, child_size_dev, out_parent_dev,
                        out_child_dev, out_lambda_dev, out_child_size_dev}));
    cudaStream_t s = as_stream(stream);
    Workspace ws(s);
    Condensed ct, out;
    FHG_TRY(condensed_from_arrays(ws, parent_dev, child_dev, lambda_dev, child_size_dev, rows, &ct));
    FHG_TRY(simplify_hierarchy(ws, ct, threshold, &out));
    // the input arrays, relabelled in place where rows are kept
    FHG_TRY(condensed_to_arrays(ct, parent_dev, child_dev, lambda_dev,
                                const_cast<float*>(child_size_dev), s));
    FHG_TRY(condensed_to_arrays(out, out_parent_dev, out_child_dev, out_lambda_dev,
                                out_child_size_dev, s));
    *out_rows_host = out.rows;
    return FHG_OK;
}

FHG_API int fhg_cluster_epsilon_search(const int64_t* parent_dev, const int64_t* child_dev,
                                       const float* lambda_dev, const float* child_size_dev,
                                       int64_t rows, const int64_t* clusters_dev,
                                       int64_t n_clusters, double min_epsilon, int64_t* out_dev,
                                       int64_t* n_out_host, void* stream) {
    FHG_TRY(check_ptrs("fhg_cluster_epsilon_search", {n_out_host}));
    *n_out_host = 0;
    FHG_TRY(check_counts("fhg_cluster_epsilon_search", {rows, n_clusters}));
    if (n_clusters == 0) return FHG_OK;
    FHG_TRY(check_ptrs("fhg_cluster_epsilon_search",
                       {parent_dev, child_dev, lambda_dev, child_size_dev, clusters_dev, out_dev}));
    if (rows == 0) {
        set_error("fhg_cluster_epsilon_search: empty cluster tree");
        return FHG_ERR_INVALID;
    }
    cudaStream_t s = as_stream(stream);
    Workspace ws(s);
    Condensed ct;
    FHG_TRY(condensed_from_arrays(ws, parent_dev, child_dev, lambda_dev, child_size_dev, rows, &ct));
    int32_t *sel, *out;
    FHG_TRY(ws.alloc(&sel, (size_t)n_clusters));
    FHG_TRY(ws.alloc(&out, (size_t)n_clusters));
    ::fhg::note_launch();
    narrow_sel_kernel<<<grid_for(n_clusters, 256), 256, 0, s>>>(n_clusters, clusters_dev, sel);
    FHG_CUDA(cudaGetLastError());
    int64_t k = 0;
    FHG_TRY(epsilon_search(ws, ct, sel, n_clusters, min_epsilon, out, &k));
    if (k > 0) {
        ::fhg::note_launch();
        widen_sel_kernel<<<grid_for(k, 256), 256, 0, s>>>(k, out, out_dev);
        FHG_CUDA(cudaGetLastError());
    }
    *n_out_host = k;
    return FHG_OK;
}

FHG_API int fhg_labelling_at_cut(const double* linkage_dev, int64_t m, double cut,
                                 int64_t min_cluster_size, int64_t* labels_dev, void* stream) {
    if (m < 0) {
        set_error("fhg_labelling_at_cut: negative row count");
        return FHG_ERR_INVALID;
    }
    FHG_TRY(check_ptrs("fhg_labelling_at_cut", {labels_dev}));
    if (m > 0) FHG_TRY(check_ptrs("fhg_labelling_at_cut", {linkage_dev}));
    cudaStream_t s = as_stream(stream);
    Workspace ws(s);
    Linkage lk;
    FHG_TRY(linkage_from_f64(ws, linkage_dev, m, &lk));
    return labelling_at_cut(ws, lk, cut, min_cluster_size, labels_dev);
}

// ---------------------------------------------------------------- fused fit
namespace {

// A precomputed sparse graph as the fit's input (metric="precomputed").
struct GraphInput {
    const int32_t* rows = nullptr;
    const int32_t* cols = nullptr;
    const double* data = nullptr;
    int64_t nnz = 0;
};

// Host destinations of the large fit outputs, each copied on a side stream as
// soon as the fit has finished writing it, so that the transfers overlap the
// later stages.  NULL members are not copied.
struct FitExport {
    int32_t* neighbors_host = nullptr;
    float* core_host = nullptr;
    double* mst_host = nullptr;
    double* linkage_host = nullptr;
    void* records_dev = nullptr;
    void* records_host = nullptr;
    int64_t* records_rows_host = nullptr;
};

// Device-to-host copies ordered after the work queued so far on the fit's
// stream, issued on a side stream; the fit's stream waits for all of them
// when the export ends (also on an error return).
class SideCopies {
public:
    explicit SideCopies(cudaStream_t main) : main_(main) {}
    SideCopies(const SideCopies&) = delete;
    SideCopies& operator=(const SideCopies&) = delete;
    ~SideCopies() {
        if (!side_) return;
        cudaEventRecord(ev_, side_);
        cudaStreamWaitEvent(main_, ev_, 0);
        cudaEventDestroy(ev_);
        cudaStreamDestroy(side_);  // released once its copies have completed
    }
    int copy(void* dst, const void* src, size_t bytes) {
        if (!dst || bytes == 0) return FHG_OK;
        if (!side_) {
            FHG_CUDA(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
            if (cudaEventCreateWithFlags(&ev_, cudaEventDisableTiming) != cudaSuccess) {
                cudaStreamDestroy(side_);
                side_ = nullptr;
                set_error("fit export: cudaEventCreateWithFlags failed");
                return FHG_ERR_CUDA;
            }
        }
        FHG_CUDA(cudaEventRecord(ev_, main_));
        FHG_CUDA(cudaStreamWaitEvent(side_, ev_, 0));
        FHG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, side_));
        return FHG_OK;
    }

private:
    cudaStream_t main_;
    cudaStream_t side_ = nullptr;
    cudaEvent_t ev_ = nullptr;
};

int fit_impl(const float* X_dev, int64_t n, int32_t d, int32_t min_samples,
             int64_t min_cluster_size, int32_t selection_method, double max_cluster_size,
             int allow_single_cluster, double epsilon, double persistence,
             const float* sample_weights_dev, int32_t weighted_k, int64_t* labels_dev,
             float* probs_dev, double* mst_dev, double* linkage_dev, int64_t* ct_parent_dev,
             int64_t* ct_child_dev, float* ct_lambda_dev, float* ct_size_dev,
             int64_t* ct_rows_host, int32_t* neighbors_dev, float* core_dev,
             int64_t* selected_dev, int64_t* n_selected_host, void* stream,
             const FitExport& ex, int32_t knn_k = 0, int32_t query_k = 0,
             double* core64_dev = nullptr, const GraphInput* graph = nullptr,
             bool brute_knn = false, const double* mst_in = nullptr) {
    FHG_TRY(check_ptrs("fhg_hdbscan_fit", {labels_dev, probs_dev}));
    if (!graph && !mst_in) FHG_TRY(check_ptrs("fhg_hdbscan_fit", {X_dev}));
    if (min_samples < 1 || min_cluster_size < 1) {
        set_error("Min samples and min cluster size must be positive integers!");
        return FHG_ERR_INVALID;
    }
    if (selection_method != 0 && selection_method != 1) {
        set_error("Invalid cluster_selection_method %d", selection_method);
        return FHG_ERR_INVALID;
    }
    if (n < 2) {
        set_error("fhg_hdbscan_fit needs at least two points");
        return FHG_ERR_INVALID;
    }
    cudaStream_t s = as_stream(stream);
    SideCopies side(s);  // declared before the workspace: joins after its frees are queued
    Workspace ws(s);
    fhg_index* ix = nullptr;
    if (!graph && !brute_knn && !mst_in) FHG_TRY(index_build(X_dev, n, d, s, &ix));
    struct IndexGuard {
        fhg_index* p;
        cudaStream_t s;
        ~IndexGuard() { index_free(p, s); }
    } guard{ix, s};
    Linkage lk;
    if (mst_in) {  // a given spanning tree (hdbscan.py:497 clusters_from_spanning_tree)
        int32_t *src, *dst;
        double* w;
        FHG_TRY(split_mst_f64(ws, mst_in, n - 1, &src, &dst, &w));
        FHG_TRY(sort_and_link(ws, n, src, dst, w, nullptr, &lk, false));
    } else if (graph) {  // a precomputed sparse graph (precomputed.py:410 / :479)
        double *kedges, *core64 = core64_dev;
        int32_t* nb = neighbors_dev;
        FHG_TRY(ws.alloc(&kedges, (size_t)(3 * (n - 1))));
        if (!core64) FHG_TRY(ws.alloc(&core64, (size_t)n));
        if (!nb) FHG_TRY(ws.alloc(&nb, (size_t)(n * (min_samples > 1 ? min_samples : 1))));
        int64_t nc = 0;
        FHG_TRY(precomputed_mst(graph->rows, graph->cols, graph->data, graph->nnz, n,
                                min_samples, kedges, nb, core64, &nc, s));
        int32_t *src, *dst;
        double* w;
        FHG_TRY(split_mst_f64(ws, kedges, n - 1, &src, &dst, &w));
        FHG_TRY(sort_and_link(ws, n, src, dst, w, nullptr, &lk, false));
    } else if (knn_k > 0) {  // the kNN-graph Kruskal back-end (kruskal.py:950)
        double *kedges, *core64 = core64_dev;
        FHG_TRY(ws.alloc(&kedges, (size_t)(3 * (n - 1))));
        if (!core64) FHG_TRY(ws.alloc(&core64, (size_t)n));
        int64_t nc = 0;
        if (brute_knn)  // the high-dimensional kNN graph (nndescent.py:179)
            FHG_TRY(kruskal_mst_of_lists(n, min_samples, query_k, nullptr, nullptr, X_dev, d,
                                         kedges, neighbors_dev, core64, &nc, s));
        else
            FHG_TRY(kruskal_knn_mst(*ix, min_samples, query_k, sample_weights_dev, kedges,
                                    neighbors_dev, core64, &nc, s));
        int32_t *src, *dst;
        double* w;
        FHG_TRY(split_mst_f64(ws, kedges, n - 1, &src, &dst, &w));
        FHG_TRY(sort_and_link(ws, n, src, dst, w, nullptr, &lk, false));
    } else {
        MstResult mst;
        FHG_TRY(boruvka_mst(ws, *ix, min_samples, &mst, core_dev, neighbors_dev,
                            sample_weights_dev, weighted_k, /*any_order=*/true));  // sorted below
        if (neighbors_dev) {
            // the row width boruvka_mst writes: k - 1 for its k-neighbour query
            const int64_t kq =
                sample_weights_dev ? weighted_k : (min_samples > 1 ? min_samples + 1 : 2);
            const int64_t kcols = kq > 1 ? kq - 1 : 0;
            FHG_TRY(side.copy(ex.neighbors_host, neighbors_dev, sizeof(int32_t) * n * kcols));
        }
        if (core_dev) FHG_TRY(side.copy(ex.core_host, core_dev, sizeof(float) * n));
        if (mst.m != n - 1) {
            set_error("boruvka: spanning forest has %lld edges for %lld points", (long long)mst.m,
                      (long long)n);
            return FHG_ERR_NO_CONVERGENCE;
        }
        FHG_TRY(sort_and_link(ws, n, mst.src, mst.dst, nullptr, mst.w2, &lk));
    }
    if (sample_weights_dev) FHG_TRY(weighted_sizes(ws, lk, sample_weights_dev));
    {
        Stage stage(s, "outputs");
        if (mst_dev) FHG_TRY(sorted_mst_to_f64(lk, mst_dev, s));
        if (linkage_dev) FHG_TRY(linkage_to_f64(lk, linkage_dev, s));
    }
    if (mst_dev) FHG_TRY(side.copy(ex.mst_host, mst_dev, sizeof(double) * 3 * (n - 1)));
    if (linkage_dev) FHG_TRY(side.copy(ex.linkage_host, linkage_dev, sizeof(double) * 4 * (n - 1)));
    Condensed ct;
    // hdbscan.py:521: the fit path condenses without max_cluster_size; only
    // the EOM selection reads it.
    FHG_TRY(condense_tree(ws, lk, min_cluster_size, INFINITY, &ct));
    if (persistence > 0.0 && ct.rows > 0) {  // hdbscan.py:528
        Condensed simple;
        FHG_TRY(simplify_hierarchy(ws, ct, persistence, &simple));
        ct = simple;
    }
    if (ct_rows_host) *ct_rows_host = ct.rows;
    if (ct_parent_dev && ct_child_dev && ct_lambda_dev && ct_size_dev) {
        FHG_TRY(condensed_to_arrays(ct, ct_parent_dev, ct_child_dev, ct_lambda_dev, ct_size_dev, s));
        if (ex.records_dev) {
            if (ex.records_rows_host) *ex.records_rows_host = ct.rows;
            if (ct.rows > 0) {
                ::fhg::note_launch();
                fhg::capi::condensed_records_kernel<<<grid_for(ct.rows, 256), 256, 0, s>>>(
                    ct.rows, ct_parent_dev, ct_child_dev, ct_lambda_dev, ct_size_dev,
                    static_cast<uint32_t*>(ex.records_dev));
                FHG_CUDA(cudaGetLastError());
                FHG_TRY(side.copy(ex.records_host, ex.records_dev, (size_t)ct.rows * 28));
            }
        }
    }
    int32_t* sel;
    FHG_TRY(ws.alloc(&sel, (size_t)(ct.n_clusters > 0 ? ct.n_clusters : 1)));
    int64_t k = 0;
    LabelPre lpre;  // labelling work that overlaps the stabilities
    if (selection_method == 0)
        FHG_TRY(select_eom(ws, ct, max_cluster_size, allow_single_cluster != 0, sel, &k, &lpre));
    else
        FHG_TRY(select_leaf(ws, ct, sel, &k, &lpre));
    if (k > 1 && epsilon > 0.0) {  // hdbscan.py:555
        int32_t* searched;
        FHG_TRY(ws.alloc(&searched, (size_t)k));
        int64_t k2 = 0;
        FHG_TRY(epsilon_search(ws, ct, sel, k, epsilon, searched, &k2));
        sel = searched;
        k = k2;
    }
    if (n_selected_host) *n_selected_host = k;
    if (selected_dev && k > 0) {
        ::fhg::note_launch();
        widen_sel_kernel<<<grid_for(k, 256), 256, 0, s>>>(k, sel, selected_dev);
        FHG_CUDA(cudaGetLastError());
    }
    if (k == 0 || ct.rows == 0) {
        ::fhg::note_launch();
        fill_labels_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, labels_dev, probs_dev);
        FHG_CUDA(cudaGetLastError());
        return FHG_OK;
    }
    return label_points(ws, ct, sel, k, epsilon, labels_dev, probs_dev, &lpre);
}

}  // namespace

FHG_API int fhg_hdbscan_fit(const float* X_dev, int64_t n, int32_t d, int32_t min_samples,
                            int64_t min_cluster_size, int32_t selection_method,
                            double max_cluster_size, int allow_single_cluster, double epsilon,
                            double persistence, const float* sample_weights_dev,
                            int32_t weighted_k, int64_t* labels_dev, float* probs_dev,
                            double* mst_dev, double* linkage_dev, int64_t* ct_parent_dev,
                            int64_t* ct_child_dev, float* ct_lambda_dev, float* ct_size_dev,
                            int64_t* ct_rows_host, int32_t* neighbors_dev, float* core_dev,
                            int64_t* selected_dev, int64_t* n_selected_host, void* stream) {
    return fit_impl(X_dev, n, d, min_samples, min_cluster_size, selection_method,
                    max_cluster_size, allow_single_cluster, epsilon, persistence,
                    sample_weights_dev, weighted_k, labels_dev, probs_dev, mst_dev, linkage_dev,
                    ct_parent_dev, ct_child_dev, ct_lambda_dev, ct_size_dev, ct_rows_host,
                    neighbors_dev, core_dev, selected_dev, n_selected_host, stream, FitExport());
}

FHG_API int fhg_hdbscan_fit_kruskal(
    const float* X_dev, int64_t n, int32_t d, int32_t min_samples, int32_t knn_k,
    int32_t query_k, int64_t min_cluster_size, int32_t selection_method, double max_cluster_size,
    int allow_single_cluster, double epsilon, double persistence, const float* sample_weights_dev,
    int64_t* labels_dev, float* probs_dev, double* mst_dev, double* linkage_dev,
    int64_t* ct_parent_dev, int64_t* ct_child_dev, float* ct_lambda_dev, float* ct_size_dev,
    int64_t* ct_rows_host, int32_t* neighbors_dev, double* core_dev, int64_t* selected_dev,
    int64_t* n_selected_host, void* stream) {
    if (knn_k < 1) {
        set_error("fhg_hdbscan_fit_kruskal: knn_k must be a positive integer (got %d)", knn_k);
        return FHG_ERR_INVALID;
    }
    return fit_impl(X_dev, n, d, min_samples, min_cluster_size, selection_method,
                    max_cluster_size, allow_single_cluster, epsilon, persistence,
                    sample_weights_dev, 0, labels_dev, probs_dev, mst_dev, linkage_dev,
                    ct_parent_dev, ct_child_dev, ct_lambda_dev, ct_size_dev, ct_rows_host,
                    neighbors_dev, nullptr, selected_dev, n_selected_host, stream, FitExport(),
                    knn_k, query_k, core_dev);
}

FHG_API int fhg_hdbscan_fit_knn_graph(
    const float* X_dev, int64_t n, int32_t d, int32_t min_samples, int32_t knn_k,
    int64_t min_cluster_size, int32_t selection_method, double max_cluster_size,
    int allow_single_cluster, double epsilon, double persistence, int64_t* labels_dev,
    float* probs_dev, double* mst_dev, double* linkage_dev, int64_t* ct_parent_dev,
    int64_t* ct_child_dev, float* ct_lambda_dev, float* ct_size_dev, int64_t* ct_rows_host,
    int32_t* neighbors_dev, double* core_dev, int64_t* selected_dev, int64_t* n_selected_host,
    void* stream) {
    if (knn_k < 1 || knn_k < min_samples) {
        set_error("fhg_hdbscan_fit_knn_graph: knn_k must be at least max(1, min_samples) "
                  "(got %d)", knn_k);
        return FHG_ERR_INVALID;
    }
    return fit_impl(X_dev, n, d, min_samples, min_cluster_size, selection_method,
                    max_cluster_size, allow_single_cluster, epsilon, persistence, nullptr, 0,
                    labels_dev, probs_dev, mst_dev, linkage_dev, ct_parent_dev, ct_child_dev,
                    ct_lambda_dev, ct_size_dev, ct_rows_host, neighbors_dev, nullptr,
                    selected_dev, n_selected_host, stream, FitExport(), knn_k, knn_k + 1,
                    core_dev, nullptr, /*brute_knn=*/true);
}

FHG_API int fhg_hdbscan_fit_precomputed(
    const int32_t* rows_dev, const int32_t* cols_dev, const double* data_dev, int64_t nnz,
    int64_t n, int32_t min_samples, int32_t algorithm, int64_t min_cluster_size,
    int32_t selection_method, double max_cluster_size, int allow_single_cluster, double epsilon,
    double persistence, int64_t* labels_dev, float* probs_dev, double* mst_dev,
    double* linkage_dev, int64_t* ct_parent_dev, int64_t* ct_child_dev, float* ct_lambda_dev,
    float* ct_size_dev, int64_t* ct_rows_host, int32_t* neighbors_dev, double* core_dev,
    int64_t* selected_dev, int64_t* n_selected_host, void* stream) {
    if (nnz < 0 || (nnz > 0 && (!rows_dev || !cols_dev || !data_dev))) {
        set_error("fhg_hdbscan_fit_precomputed: invalid graph entries");
        return FHG_ERR_INVALID;
    }
    if (algorithm != 0 && algorithm != 1) {
        set_error("fhg_hdbscan_fit_precomputed: algorithm must be 0 (boruvka) or 1 (kruskal)");
        return FHG_ERR_INVALID;
    }
    GraphInput g;
    g.rows = rows_dev;
    g.cols = cols_dev;
    g.data = data_dev;
    g.nnz = nnz;
    return fit_impl(nullptr, n, 0, min_samples, min_cluster_size, selection_method,
                    max_cluster_size, allow_single_cluster, epsilon, persistence, nullptr, 0,
                    labels_dev, probs_dev, mst_dev, linkage_dev, ct_parent_dev, ct_child_dev,
                    ct_lambda_dev, ct_size_dev, ct_rows_host, neighbors_dev, nullptr,
                    selected_dev, n_selected_host, stream, FitExport(), 0, 0, core_dev, &g);
}

FHG_API int fhg_clusters_from_mst(const double* mst_dev, int64_t n, int64_t min_cluster_size,
                                  int32_t selection_method, double max_cluster_size,
                                  int allow_single_cluster, double epsilon, double persistence,
                                  const float* sample_weights_dev, int64_t* labels_dev,
                                  float* probs_dev, double* sorted_mst_dev, double* linkage_dev,
                                  int64_t* ct_parent_dev, int64_t* ct_child_dev,
                                  float* ct_lambda_dev, float* ct_size_dev, int64_t* ct_rows_host,
                                  int64_t* selected_dev, int64_t* n_selected_host, void* stream) {
    if (!mst_dev) {
        set_error("fhg_clusters_from_mst: mst_dev is NULL");
        return FHG_ERR_INVALID;
    }
    return fit_impl(nullptr, n, 0, 1, min_cluster_size, selection_method, max_cluster_size,
                    allow_single_cluster, epsilon, persistence, sample_weights_dev, 0, labels_dev,
                    probs_dev, sorted_mst_dev, linkage_dev, ct_parent_dev, ct_child_dev,
                    ct_lambda_dev, ct_size_dev, ct_rows_host, nullptr, nullptr, selected_dev,
                    n_selected_host, stream, FitExport(), 0, 0, nullptr, nullptr, false, mst_dev);
}

FHG_API int fhg_hdbscan_fit_export(
    const float* X_dev, int64_t n, int32_t d, int32_t min_samples, int64_t min_cluster_size,
    int32_t selection_method, double max_cluster_size, int allow_single_cluster, double epsilon,
    double persistence, const float* sample_weights_dev, int32_t weighted_k, int64_t* labels_dev,
    float* probs_dev, double* mst_dev, double* linkage_dev, int64_t* ct_parent_dev,
    int64_t* ct_child_dev, float* ct_lambda_dev, float* ct_size_dev, int64_t* ct_rows_host,
    int32_t* neighbors_dev, float* core_dev, int64_t* selected_dev, int64_t* n_selected_host,
    int32_t* neighbors_host, float* core_host, double* mst_host, double* linkage_host,
    void* ct_records_dev, void* ct_records_host, void* stream) {
    if (ct_records_dev && reinterpret_cast<uintptr_t>(ct_records_dev) % 4 != 0) {
        set_error("fhg_hdbscan_fit_export: ct_records_dev must be 4-byte aligned");
        return FHG_ERR_INVALID;
    }
    if ((neighbors_host && !neighbors_dev) || (core_host && !core_dev) ||
        (mst_host && !mst_dev) || (linkage_host && !linkage_dev) ||
        (ct_records_host && !ct_records_dev) ||
        (ct_records_dev && !(ct_parent_dev && ct_child_dev && ct_lambda_dev && ct_size_dev))) {
        set_error("fhg_hdbscan_fit_export: every exported output needs its device buffer");
        return FHG_ERR_INVALID;
    }
    FitExport ex;
    ex.neighbors_host = neighbors_host;
    ex.core_host = core_host;
    ex.mst_host = mst_host;
    ex.linkage_host = linkage_host;
    ex.records_dev = ct_records_dev;
    ex.records_host = ct_records_host;
    ex.records_rows_host = ct_rows_host;
    return fit_impl(X_dev, n, d, min_samples, min_cluster_size, selection_method,
                    max_cluster_size, allow_single_cluster, epsilon, persistence,
                    sample_weights_dev, weighted_k, labels_dev, probs_dev, mst_dev, linkage_dev,
                    ct_parent_dev, ct_child_dev, ct_lambda_dev, ct_size_dev, ct_rows_host,
                    neighbors_dev, core_dev, selected_dev, n_selected_host, stream, ex);
}
