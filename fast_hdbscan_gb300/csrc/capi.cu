// extern "C" entry points of libfhg.so (declared in include/fhg.h).
#include <cstdarg>

#include "index.cuh"
#include "mst.cuh"

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

int finalize_edges(const MstResult& r, double* edges, cudaStream_t s);

}  // namespace fhg

using namespace fhg;

#define FHG_API extern "C" __attribute__((visibility("default")))

static inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

FHG_API const char* fhg_last_error(void) { return last_error(); }
FHG_API int fhg_abi_version(void) { return 1; }

FHG_API int fhg_index_build(const float* X_dev, int64_t n, int32_t d, void* stream,
                            fhg_index** out) {
    if (!out || !X_dev) {
        set_error("fhg_index_build: null pointer");
        return FHG_ERR_INVALID;
    }
    return index_build(X_dev, n, d, as_stream(stream), out);
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

FHG_API int fhg_index_boruvka(fhg_index* index, int32_t min_samples, double* edges_dev,
                              int32_t* neighbors_dev, float* core_dev, int32_t* n_rounds_host,
                              void* stream) {
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
    FHG_TRY(boruvka_mst(ws, *index, min_samples, &r, core_dev, neighbors_dev));
    FHG_TRY(finalize_edges(r, edges_dev, s));
    if (n_rounds_host) *n_rounds_host = r.rounds;
    if (r.m != index->n - 1 && index->n > 1) {
        set_error("boruvka: spanning forest has %lld edges for %lld points", (long long)r.m,
                  (long long)index->n);
        return FHG_ERR_NO_CONVERGENCE;
    }
    return FHG_OK;
}
