// Learned kNN search radius (radius.cu).
#pragma once
#include "index.cuh"

namespace fhg {

constexpr int kRadiusParams = 64 * 11 + 64 + 64 * 64 + 64 + 64 + 1 + 11 + 11;

// The model a thread's fits use for their kNN step (params on the device).
struct RadiusUse {
    const float* params = nullptr;
    float margin = 1.0f;
};
const RadiusUse* radius_in_use();  // nullptr: plain kNN
void radius_set_use(const float* params, float margin);

int radius_features(const fhg_index& ix, const int32_t* orig, float* feat, cudaStream_t s);
int radius_predict(const float* prm, const float* feat, int64_t n, float margin, float* out_y,
                   float* cap2, cudaStream_t s);
int radius_init(float* prm, const float* feat, const float* tgt, int64_t n, uint64_t seed,
                cudaStream_t s);
int radius_targets(const fhg_index& ix, int k, float* tgt, cudaStream_t s);
int radius_grad(const float* prm, const float* feat, const float* tgt, const int32_t* rows,
                int64_t B, float* grad, float* loss, cudaStream_t s);
int radius_train(float* prm, const float* feat, const float* tgt, int64_t n, int32_t steps,
                 int32_t B, float lr, uint64_t seed, float* loss_curve, cudaStream_t s);
int knn_with_radius(const fhg_index& ix, int k, const RadiusUse& use, float* d_s, int32_t* i_s,
                    float* d_o, int32_t* i_o, cudaStream_t s, int8_t* tie_s = nullptr,
                    int io_stride = 0, int io_skip = 0, unsigned long long* scans = nullptr);
int knn_scan_count(const fhg_index& ix, int k, const float* params, float margin, int64_t* scans,
                   int64_t* fallbacks, cudaStream_t s);
int radius_last_fallbacks(int64_t* out, cudaStream_t s);

}  // namespace fhg
