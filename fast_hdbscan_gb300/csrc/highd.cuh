// Exact brute-force kNN for high-dimensional points (highd.cu).
#pragma once
#include "fhg_common.cuh"

namespace fhg {

constexpr int kHighdMaxDim = 96;

// kNN of every point of X (n x d float32, row-major, caller order), itself
// included: rows of k (squared float32 distance, index) in (distance, index)
// order, as index_knn writes them.  k + 32 <= 128.  *fallbacks (nullable) =
// queries whose tensor-core candidates could not be certified and were
// searched again exactly.
int highd_knn(const float* X, int64_t n, int d, int k, float* rd_o, int32_t* ix_o,
              int64_t* fallbacks, cudaStream_t s);
// Candidate kernel of the calling thread's later calls: 0 the tcgen05
// pipeline (where its buffers fit), 1 the mma.sync kernel.  Returns the old.
int highd_use_legacy(int on);

}  // namespace fhg
