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
// `ws` owns every returned buffer.  Optional outputs (nullable):
//   core_o  [n]       sqrt core distance, caller order
//   nbr_o   [n*(k-1)] neighbours without the point itself, caller order
//   knn_d_o/knn_i_o [n*k] full kNN rows, caller order
int boruvka_mst(Workspace& ws, const fhg_index& ix, int min_samples, MstResult* out,
                float* core_o, int32_t* nbr_o);

}  // namespace fhg
