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
// Hooks (int32 labels; the reference's V1T):
//   initialize()                        label of an untouched vertex
//   source_value()                      label of a traversal source
//   get_partial_result(src, w)          offer a source makes along an edge
//                                       (w: the edge's integer weight)
//   accumulate(loc, data, iter)         fold an offer into *loc (atomic form)
//   accumulate_nonAtomics(acc, data, iter)  same, into a private accumulator
//   update_condition(old, acc, iter)    does a folded value improve the vertex?
//   fused_update_condition(loc, data, iter)  fold + test in one atomic step on
//                                       the destination (push form); true =
//                                       the destination improved (enqueue it)
//
// The frontier engine (mg_frontier_engine.cuh) reads these capability flags
// of an operator:
//   kLevelSync     labels are BFS levels: a vertex is final when first
//                  reached (visited bitmap, archived level lists); otherwise
//                  labels are relaxed until no offer improves them
//   kFirstParent   level-synchronous pull stops at the first frontier
//                  in-neighbour (BFS)
//   kWeighted      offers read the edge weight
//   kPathCounts    Brandes path counts travel with the levels (BC forward)
//   kMinPlusBound  min-plus with non-negative weights: a pull level skips
//                  rows at or below (least frontier label + least weight)
// and kTag, the prefix of its profiler slot names.
// A relaxed (non level-synchronous) operator must be monotone: an offer of
// an unreached vertex (initialize()) or of a vertex relaxed earlier never
// spoils a label, so dense pull levels may fold every in-neighbour's offer.
#pragma once

#include <cstdint>

namespace mgops {

constexpr int32_t UNSET = 0x64646464;

// BFS levels: user_function.h:217-218, 241-242, 270-274, 338-345, 392-399
struct Bfs {
    static constexpr const char *kTag = "bfs";  // profiler slot prefix
    static constexpr bool kLevelSync = true, kFirstParent = true, kWeighted = false, kPathCounts = false,
                          kMinPlusBound = false;
    __device__ static __forceinline__ int32_t initialize() { return UNSET; }
    __device__ static __forceinline__ int32_t source_value() { return 0; }
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
    static constexpr const char *kTag = "sssp";  // profiler slot prefix
    static constexpr bool kLevelSync = false, kFirstParent = false, kWeighted = true, kPathCounts = false,
                          kMinPlusBound = true;
    __device__ static __forceinline__ int32_t initialize() { return UNSET; }
    __device__ static __forceinline__ int32_t source_value() { return 0; }
    __device__ static __forceinline__ int32_t get_partial_result(int32_t src_dist, int32_t w) { return src_dist + w; }
    __device__ static __forceinline__ void accumulate(int32_t *loc, int32_t data, int32_t) { atomicMin(loc, data); }
    __device__ static __forceinline__ void accumulate_nonAtomics(int32_t &acc, int32_t data, int32_t)
    {
        if (data < acc) acc = data;
    }
    __device__ static __forceinline__ bool update_condition(int32_t old, int32_t acc, int32_t) { return acc < old; }
    // atomicMin on the distance; true when it lowered it (the engine then
    // sets the destination's bit in the next frontier bitmap, so it is
    // enqueued once per iteration -- the reference stamps vfc with atomicMax
    // for the same purpose)
    __device__ static __forceinline__ bool fused_update_condition(int32_t *loc, int32_t data, int32_t)
    {
        return data < *loc && data < atomicMin(loc, data);
    }
};

// Shortest-path counts.  The reference keeps them in int32, which wraps
// after a few dozen levels of a lattice; FP64 alone overflows (past 1.8e308)
// after about a thousand: the number of shortest paths to a point d steps
// away grows like 2^d.  A PathCount is an FP64 mantissa m (0, or in
// [1, 2^512)) with a scale k: sigma = m * 2^(512 k), exact to FP64 precision
// at any depth.  Engines run in one of two modes:
//   plain     k stays 0 and sums are plain FP64 adds (FP64 atomics in push
//             sweeps); the backward sweep keeps (1 + delta) / sigma in FP32,
//             so a count seen at or above PC_PLAIN_MAX = 2^90 (a summed row,
//             an added contribution, or a frontier vertex's count read as a
//             push payload) raises an overflow flag and the run is repeated
//             in extended mode.  Counts one level past the last check stay
//             below 2^90 * 2^31, so 1 / sigma stays a normal FP32 number;
//   extended  every sum renormalises (m >= 2^512: m *= 2^-512, k += 1) and
//             push sweeps add with a 16-byte compare-and-swap.
struct __align__(16) PathCount {
    double m;
    int32_t k;
    int32_t pad;
};
constexpr double PC_TOP = 0x1p512;   // m < PC_TOP
constexpr double PC_DOWN = 0x1p-512;
constexpr double PC_PLAIN_MAX = 0x1p90;  // plain-mode ceiling (see above)

__device__ __forceinline__ PathCount pc_zero() { return PathCount{0.0, 0, 0}; }
__device__ __forceinline__ PathCount pc_one() { return PathCount{1.0, 0, 0}; }

// a + b; in plain mode k is 0 on both sides and no renormalisation happens
__device__ __forceinline__ PathCount pc_add(PathCount a, PathCount b, bool ext)
{
    if (!ext) return PathCount{a.m + b.m, 0, 0};
    if (b.m == 0.0) return a;
    if (a.m == 0.0) return b;
    if (a.k < b.k) {
        const PathCount t = a;
        a = b;
        b = t;
    }
    const int32_t d = a.k - b.k;  // b is below a's ulp when d >= 2
    double m = a.m + (d == 0 ? b.m : (d == 1 ? b.m * PC_DOWN : 0.0));
    int32_t k = a.k;
    if (m >= PC_TOP) {
        m *= PC_DOWN;
        k += 1;
    }
    return PathCount{m, k, 0};
}

// 2^(512 dk) for the exponent differences of neighbouring levels
__device__ __forceinline__ double pc_scale(int32_t dk)
{
    return dk == 0 ? 1.0 : dk == -1 ? PC_DOWN : dk == 1 ? PC_TOP : dk < 0 ? 0.0 : __longlong_as_double(0x7ff0000000000000ll);
}

// FP64 value of a count (infinity past the FP64 range)
__device__ __forceinline__ double pc_to_double(PathCount a)
{
    return a.k == 0 ? a.m : (a.k == 1 ? a.m * PC_TOP : (a.m == 0.0 ? 0.0 : __longlong_as_double(0x7ff0000000000000ll)));
}

// 16-byte load through L2 (counts written by other blocks in the same launch)
__device__ __forceinline__ PathCount pc_load_cg(const PathCount *p)
{
    const longlong2 r = __ldcg(reinterpret_cast<const longlong2 *>(p));
    PathCount c;
    c.m = __longlong_as_double(r.x);
    c.k = (int32_t)(r.y & 0xffffffffll);
    c.pad = 0;
    return c;
}

__device__ __forceinline__ PathCount shfl_xor_val(PathCount v, int o)
{
    v.m = __shfl_xor_sync(0xffffffffu, v.m, o);
    v.k = __shfl_xor_sync(0xffffffffu, v.k, o);
    return v;
}

__device__ __forceinline__ PathCount shfl_val(PathCount v, int src)
{
    v.m = __shfl_sync(0xffffffffu, v.m, src);
    v.k = __shfl_sync(0xffffffffu, v.k, src);
    return v;
}

// *loc += x.  Plain mode: one FP64 atomic add (no result awaited); *ovf is
// set when x itself reaches PC_PLAIN_MAX.  Extended mode: compare-and-swap of
// the 16-byte count;
// every failed attempt means another thread's add went in, so the loop
// ends after at most as many rounds as the vertex has in-edges.
__device__ __forceinline__ void pc_atomic_add(PathCount *loc, PathCount x, bool ext, int32_t *ovf)
{
    if (!ext) {
        atomicAdd(&loc->m, x.m);
        if (x.m >= PC_PLAIN_MAX) *ovf = 1;
        return;
    }
    unsigned __int128 *a = reinterpret_cast<unsigned __int128 *>(loc);
    const longlong2 r = __ldcg(reinterpret_cast<const longlong2 *>(loc));
    unsigned __int128 old = ((unsigned __int128)(unsigned long long)r.y << 64) | (unsigned long long)r.x;
    while (true) {
        PathCount o;
        o.m = __longlong_as_double((long long)(unsigned long long)old);
        o.k = (int32_t)(unsigned)(unsigned long long)(old >> 64);
        o.pad = 0;
        const PathCount n = pc_add(o, x, true);
        const unsigned __int128 nv = ((unsigned __int128)(unsigned)n.k << 64) |
                                     (unsigned long long)__double_as_longlong(n.m);
        const unsigned __int128 prev = atomicCAS(a, old, nv);
        if (prev == old) return;
        old = prev;
    }
}

// BC forward (levels + path counts): user_function.h:223-226, 247-251, 279-287, 310-317, 362-373, 409-417
// Path counts are PathCounts here (the reference uses int32).
struct BcForward {
    static constexpr const char *kTag = "bc";  // profiler slot prefix
    static constexpr bool kLevelSync = true, kFirstParent = false, kWeighted = false, kPathCounts = true,
                          kMinPlusBound = false;
    __device__ static __forceinline__ int32_t initialize() { return UNSET; }
    __device__ static __forceinline__ int32_t source_value() { return 0; }
    __device__ static __forceinline__ int32_t get_partial_result(int32_t src_level, int32_t) { return src_level + 1; }
    __device__ static __forceinline__ void accumulate(PathCount *sigma_loc, PathCount sigma_src, bool ext, int32_t *ovf)
    {
        pc_atomic_add(sigma_loc, sigma_src, ext, ovf);
    }
    __device__ static __forceinline__ void accumulate_nonAtomics(PathCount &acc, PathCount sigma_src, bool ext)
    {
        acc = pc_add(acc, sigma_src, ext);
    }
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
