// Device-wide primitives: exclusive scan and LSD radix sort of (key, int32)
// pairs.  Both are stream-ordered and take scratch from a Workspace.
#pragma once
#include "fhg_common.cuh"

namespace fhg {

// out[i] = sum(in[0..i)); `total` (device, nullable) receives sum(in).
// in == out is allowed.
int scan_exclusive_u32(Workspace& ws, const uint32_t* in, uint32_t* out, int64_t n,
                       uint32_t* total);
int scan_exclusive_i64(Workspace& ws, const int64_t* in, int64_t* out, int64_t n, int64_t* total);
// Fixed tile order, so the rounding is the same on every run.
int scan_exclusive_f64(Workspace& ws, const double* in, double* out, int64_t n, double* total);

// Stable sort of (keys, vals) by key bits [begin_bit, end_bit), 8 bits per pass.
int radix_sort_u64(Workspace& ws, uint64_t* keys, int32_t* vals, int64_t n, int begin_bit,
                   int end_bit);
int radix_sort_u32(Workspace& ws, uint32_t* keys, int32_t* vals, int64_t n, int begin_bit,
                   int end_bit);

// Small helpers.
int fill_iota_i32(int32_t* p, int64_t n, cudaStream_t s);

inline int bits_for(int64_t v) {  // number of bits to represent values in [0, v]
    int b = 0;
    while (b < 63 && ((int64_t)1 << b) <= v) ++b;
    return b < 1 ? 1 : b;
}

}  // namespace fhg
