// mg_ops.cuh -- the operator surface: per-algorithm device hooks.
//
// This is the GB300 form of the reference's code/user_function.h:211-447
// (initialize / get_partial_result / accumulate / accumulate_nonAtomics /
// update_condition / fused_update_condition, selected there by -DBFS, -DSSSP,
// -DBC, -DCC, -DPR_T, -DPR_D).  Here each algorithm is a struct of static
// __device__ hooks with the same names and meanings, and the engines are
// templates over that struct, so an algorithm is still selected "as it is"
// but at template-instantiation time instead of by macro.  The hooks see
// vertex values only, never the layout.
//
// The signatures are reduced to what each hook uses:
//   initialize(v)                       value of an untouched vertex
//   get_partial_result(src_val, w)      value a source offers along an edge
//   accumulate(loc, data, iter)         fold an offer into *loc (atomic form)
//   accumulate_nonAtomics(acc, data, iter)  same, into a private accumulator
//   update_condition(old, acc, iter)    does a folded value improve the vertex?
//   fused_update_condition(loc, data, iter)  fold + test in one step on the
//                                       destination (push form); true =
//                                       enqueue the destination
#pragma once

#include <cstdint>

namespace mgops {

constexpr int32_t UNSET = 0x64646464;

// BFS levels: user_function.h:217-218, 241-242, 270-274, 338-345, 392-399
struct Bfs {
    __device__ static __forceinline__ int32_t initialize() { return UNSET; }
    __device__ static __forceinline__ int32_t get_partial_result(int32_t src_level, int32_t) { return src_level + 1; }
    __device__ static __forceinline__ void accumulate_nonAtomics(int32_t &acc, int32_t data, int32_t iter)
    {
        if (data <= iter && data < acc) acc = data;
    }
    __device__ static __forceinline__ bool update_condition(int32_t old, int32_t acc, int32_t) { return acc < old; }
    // push form: claim an unvisited destination (the visited bitmap makes the
    // claim exact; the reference's plain store may enqueue duplicates)
    __device__ static __forceinline__ bool fused_update_condition(int32_t *loc, int32_t data, int32_t)
    {
        return atomicCAS(loc, UNSET, data) == UNSET;
    }
};

// SSSP distances: user_function.h:220-221, 244-246, 276-278, 305-309, 346-360, 400-408
struct Sssp {
    __device__ static __forceinline__ int32_t initialize() { return UNSET; }
    __device__ static __forceinline__ int32_t get_partial_result(int32_t src_dist, int32_t w) { return src_dist + w; }
    __device__ static __forceinline__ void accumulate(int32_t *loc, int32_t data, int32_t) { atomicMin(loc, data); }
    __device__ static __forceinline__ void accumulate_nonAtomics(int32_t &acc, int32_t data, int32_t)
    {
        if (data < acc) acc = data;
    }
    __device__ static __forceinline__ bool update_condition(int32_t old, int32_t acc, int32_t) { return acc < old; }
    // atomicMin on the distance, then the destination's bit in the next
    // frontier bitmap so it is enqueued once per iteration (the reference
    // stamps vfc with atomicMax for the same purpose)
    __device__ static __forceinline__ bool fused_update_condition(int32_t *loc, int32_t data, uint32_t *next_bm,
                                                                  int32_t v)
    {
        if (data < *loc) {
            int32_t old = atomicMin(loc, data);
            if (data < old) {
                uint32_t bit = 1u << (v & 31);
                return (atomicOr(&next_bm[v >> 5], bit) & bit) == 0;
            }
        }
        return false;
    }
};

// BC forward (levels + path counts): user_function.h:223-226, 247-251, 279-287, 310-317, 362-373, 409-417
// Path counts are FP64 here (the reference uses int32).
struct BcForward {
    __device__ static __forceinline__ int32_t initialize() { return UNSET; }
    __device__ static __forceinline__ int32_t get_partial_result(int32_t src_level, int32_t) { return src_level + 1; }
    __device__ static __forceinline__ void accumulate(double *sigma_loc, double sigma_src) { atomicAdd(sigma_loc, sigma_src); }
    __device__ static __forceinline__ void accumulate_nonAtomics(double &acc, double sigma_src) { acc += sigma_src; }
    // claim at level `iter` when unvisited; a destination already at `iter`
    // still collects the path count; true = newly discovered
    __device__ static __forceinline__ bool fused_update_condition(int32_t *level_loc, int32_t iter, bool &on_level)
    {
        int32_t lv = *level_loc;
        bool claimed = false;
        if (lv == UNSET) {
            int32_t old = atomicCAS(level_loc, UNSET, iter);
            claimed = (old == UNSET);
            lv = claimed ? iter : old;
        }
        on_level = (lv == iter);
        return claimed;
    }
};

// CC hooking: user_function.h:374-380, 418-436 -- the reference alternates
// min/max hooking by iteration parity and relabels afterwards; here hooking
// always links the larger root under the smaller one, so every root is the
// minimum vertex id of its tree and the labels come out canonical.
struct Cc {
    __device__ static __forceinline__ int32_t initialize(int32_t v) { return v; }
    __device__ static __forceinline__ bool update_condition(int32_t a, int32_t b) { return a != b; }
};

// PageRank (processi.cu:577-670): reference constants common.h:58-61
struct PrRef {
    static constexpr float D = 0.85f;
    static constexpr float TOL = 0.01f;
    __device__ static __forceinline__ float initialize() { return 0.0f; }
    __device__ static __forceinline__ float get_partial_result(float rank, int32_t outdeg)
    {
        return outdeg > 0 ? rank / (float)outdeg : 0.0f;
    }
    __device__ static __forceinline__ void accumulate_nonAtomics(float &acc, float data) { acc += data; }
    __device__ static __forceinline__ float apply(float sum) { return (1.0f - D) + sum * D; }
};

}  // namespace mgops
