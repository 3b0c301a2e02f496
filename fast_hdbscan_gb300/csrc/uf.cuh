// Lock-free union-find on an int32 parent array (hook the larger root under
// the smaller one with atomicCAS; finds halve paths).  Invariant: parent[x]
// <= x, so every root is the smallest id of its set.
#pragma once
#include "fhg_common.cuh"

namespace fhg {

__device__ __forceinline__ int32_t uf_find(int32_t* par, int32_t x) {
    int32_t cur = par[x];
    if (cur != x) {
        int32_t prev = x, next;
        while (cur > (next = par[cur])) {
            par[prev] = next;
            prev = cur;
            cur = next;
        }
    }
    return cur;
}

__device__ __forceinline__ void uf_union(int32_t* par, int32_t a, int32_t b) {
    int32_t ra = uf_find(par, a), rb = uf_find(par, b);
    while (ra != rb) {
        if (ra < rb) {
            int32_t t = ra; ra = rb; rb = t;
        }
        int32_t old = atomicCAS(&par[ra], ra, rb);
        if (old == ra) return;
        ra = uf_find(par, old);
        rb = uf_find(par, rb);
    }
}

}  // namespace fhg
