// Shared helpers for the GB300 HDBSCAN engine (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fhg.h"

namespace fhg {

// Last error message of the calling host thread (read by fhg_last_error()).
void set_error(const char* fmt, ...);
const char* last_error();

// Counts every kernel launch made by the library (read by fhg_launch_count).
void note_launch();

// Per-stage timer: when profiling is on (fhg_profile_enable), records a pair
// of CUDA events on the stage's stream; fhg_profile_report sums them by name.
class Stage {
  public:
    Stage(cudaStream_t s, const char* name);
    ~Stage();
    Stage(const Stage&) = delete;
    Stage& operator=(const Stage&) = delete;

  private:
    cudaStream_t s_;
    const char* name_;
    cudaEvent_t a_ = nullptr;
};

// With profiling on, adds `value` to the named counter; fhg_profile_report
// lists it beside the stages as [sum, samples].
void profile_count(const char* name, double value);

// A status carried through the host driver code.  Device kernels never trap:
// bounded loops report through a device status word instead.
struct Status {
    int code = FHG_OK;
    bool ok() const { return code == FHG_OK; }
};

#define FHG_CUDA(expr)                                                                  \
    do {                                                                                \
        cudaError_t _e = (expr);                                                        \
        if (_e != cudaSuccess) {                                                        \
            ::fhg::set_error("%s failed at %s:%d: %s", #expr, __FILE__, __LINE__,      \
                             cudaGetErrorString(_e));                                   \
            return (_e == cudaErrorMemoryAllocation) ? FHG_ERR_OOM : FHG_ERR_CUDA;      \
        }                                                                               \
    } while (0)

#define FHG_TRY(expr)                      \
    do {                                   \
        int _s = (expr);                   \
        if (_s != FHG_OK) return _s;       \
    } while (0)

// The library's stream-ordered memory pool on the current device.  Freed
// blocks stay cached in the pool (release threshold: unlimited), so that the
// synchronisations inside a fit never hand memory back to the driver and the
// next allocation never has to map it again; fhg_release_cached_memory()
// returns the cached blocks.
int device_pool(cudaMemPool_t* out);

// Stream-ordered scratch allocation.  Every buffer of a call is released on
// the same stream when the Workspace goes out of scope.
class Workspace {
  public:
    explicit Workspace(cudaStream_t s) : stream_(s) {}
    ~Workspace() { release(); }
    Workspace(const Workspace&) = delete;
    Workspace& operator=(const Workspace&) = delete;

    template <class T>
    int alloc(T** out, size_t count) {
        void* p = nullptr;
        size_t bytes = count * sizeof(T);
        if (bytes == 0) bytes = 16;
        if (!pool_) {
            int rc = device_pool(&pool_);
            if (rc != FHG_OK) return rc;
        }
        cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, pool_, stream_);
        if (e != cudaSuccess) {
            set_error("cudaMallocFromPoolAsync(%zu bytes) failed: %s", bytes,
                      cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? FHG_ERR_OOM : FHG_ERR_CUDA;
        }
        bufs_.push_back(p);
        *out = static_cast<T*>(p);
        return FHG_OK;
    }
    void release() {
        for (size_t i = bufs_.size(); i-- > 0;) cudaFreeAsync(bufs_[i], stream_);
        bufs_.clear();
    }
    cudaStream_t stream() const { return stream_; }

  private:
    cudaStream_t stream_;
    cudaMemPool_t pool_ = nullptr;
    std::vector<void*> bufs_;
};

inline unsigned grid_for(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 0x7fffffff) g = 0x7fffffff;
    return (unsigned)g;
}

// Monotone float <-> uint32 for non-negative floats (including +inf).
__host__ __device__ inline uint32_t fbits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
__host__ __device__ inline float bitsf(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

constexpr int kLeaf = 32;     // points per spatial bucket (one warp)
constexpr unsigned kFull = 0xffffffffu;

}  // namespace fhg
