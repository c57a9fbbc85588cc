// A test-only operator on the frontier engine: widest path (largest
// bottleneck capacity) from a source over the graph's integer weights.
// label[v] = max over paths s ~> v of the least edge weight on the path;
// 0 = unreachable; the source itself gets INT32_MAX.  It is a relaxed,
// weighted max-min operator -- neither a level-synchronous traversal nor
// min-plus -- defined only here and compiled against libmg's public
// operator surface (mg_ops.cuh, mg_plugin.cuh).
#include "mg_plugin.cuh"

#include <climits>

struct WidestPath {
    static constexpr const char *kTag = "widest";
    static constexpr bool kLevelSync = false, kFirstParent = false, kWeighted = true, kPathCounts = false,
                          kMinPlusBound = false;
    __device__ static __forceinline__ int32_t initialize() { return 0; }
    __device__ static __forceinline__ int32_t source_value() { return INT_MAX; }
    __device__ static __forceinline__ int32_t get_partial_result(int32_t src_width, int32_t w)
    {
        return min(src_width, w);
    }
    __device__ static __forceinline__ void accumulate_nonAtomics(int32_t &acc, int32_t data, int32_t)
    {
        if (data > acc) acc = data;
    }
    __device__ static __forceinline__ bool update_condition(int32_t old, int32_t acc, int32_t) { return acc > old; }
    __device__ static __forceinline__ bool fused_update_condition(int32_t *loc, int32_t data, int32_t)
    {
        return data > *loc && data > atomicMax(loc, data);
    }
};

MG_FRONTIER_OPERATOR(mg_widest_path, WidestPath)
