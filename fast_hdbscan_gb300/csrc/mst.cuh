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
// With sample weights (caller order, nullable) the reference's weighted path:
// k = weighted_k = int(2 * min_samples / mean weight), weighted core
// distances, round 0 on plain distances (boruvka.py:561-573).
// `ws` owns every returned buffer.  Optional outputs (nullable):
//   core_o  [n]       sqrt core distance, caller order
//   nbr_o   [n*(k-1)] neighbours without the point itself, caller order
// The edge list comes in the reference's order (the round-0 edges by caller
// index of the choosing point, then every round's by component); with
// any_order the round-0 edges come in index order instead, for callers that
// sort the edges anyway.
int boruvka_mst(Workspace& ws, const fhg_index& ix, int min_samples, MstResult* out,
                float* core_o, int32_t* nbr_o, const float* weights = nullptr,
                int weighted_k = 0, bool any_order = false);

}  // namespace fhg
