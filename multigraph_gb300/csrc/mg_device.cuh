// mg_device.cuh -- device-side internals shared by the engine translation units.
#pragma once

#include "mg_internal.h"

#include <cuda_runtime.h>

#include "mg_bins.cuh"

#include <functional>
#include <string>
#include <vector>

#define MG_CUDA(call)                                                                                 \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return mgi::fail(MG_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                             __LINE__);                                                               \
    } while (0)

#define MG_TRY(expr)                  \
    do {                              \
        mg_status s_ = (expr);        \
        if (s_ != MG_OK) return s_;   \
    } while (0)

// "unreached" label value (common.h:37-39 of the reference)
constexpr int32_t MG_UNSET = 0x64646464;

namespace mgi {

// ---------------------------------------------------------------------------
// device buffers (allocation goes through the failure-injection counter)
// ---------------------------------------------------------------------------
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    template <class T> T *as() const { return reinterpret_cast<T *>(p); }
};
mg_status dev_alloc(DevBuf &b, size_t bytes);          // no-op when already >= bytes
void dev_free(DevBuf &b);

// ---------------------------------------------------------------------------
// per-kernel profiling with cudaEvents (host-loop runs only)
// ---------------------------------------------------------------------------
struct Profiler {
    bool on = false;
    cudaStream_t stream = nullptr;
    struct Slot { std::string name; int launches = 0; double ms = 0; };
    std::vector<Slot> slots;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pool;
    struct Pending { int slot; size_t ev; };
    std::vector<Pending> pending;
    size_t used = 0;
    void reset(cudaStream_t s, bool enable);
    int slot(const char *name);
    // bracket one launch: begin() before, end() after
    void begin(int slot_id);
    void end();
    mg_status collect(mg_run_info *info);  // after the stream is synchronised
    ~Profiler();
private:
    int open_slot = -1;
};

// ---------------------------------------------------------------------------
// iteration loops: CUDA graph with a device-side WHILE node, or a host loop
// ---------------------------------------------------------------------------
// `body(stream, handle, use_cond)` enqueues one iteration; its last kernel
// must set the loop condition with cudaGraphSetConditional when use_cond is
// set, and always write the continue flag to *more_dev.
using BodyFn = std::function<mg_status(cudaStream_t, cudaGraphConditionalHandle, int)>;

// Key of a captured loop: the raw bytes of every by-value argument its
// kernels take (whole argument structs, zero-filled before they are set so
// that padding compares equal, plus launch shapes and scalars).  A cached
// loop is replayed only when the key matches byte for byte.
struct LoopKey {
    std::string bytes;
    template <class T> LoopKey &add(const T &v)
    {
        bytes.append(reinterpret_cast<const char *>(&v), sizeof(T));
        return *this;
    }
};

struct LoopGraph {
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    std::string key;
    void destroy();
};

mg_status run_loop(int exec_mode, bool profile, cudaStream_t stream, LoopGraph &lg, const LoopKey &key,
                   const BodyFn &body, const int32_t *more_dev, int32_t *more_host, int max_host_iters);

}  // namespace mgi

// shared-memory segmented pull for PageRank sweeps (mg_hub.cu): in-edges
// grouped by 224 KB source segments as 16-bit ids, gathered from shared
// memory; partial sums per (row, segment) pair; ids past the last segment
// stay in an int32 tail (offsets toff) gathered through L2
namespace mgi {
struct HubSplit {
    bool valid = false;      // built for the current pull columns
    bool use = false;        // the split is in use (enough covered edges)
    uint64_t gen = 0;        // build number (process-wide): captured sweeps key on it
    int32_t H = 0, nseg = 0; // vertices per segment; segments
    int32_t ngroups = 0;     // warp groups of equal-length pieces
    int64_t npieces = 0, covered = 0;  // pieces (P entries); edges in the segments
    int64_t ntail = 0;       // edges past the last segment
    int32_t grid = 0;        // CTAs of the sweep (one per SM)
    int32_t nfw = 0, fin_warp = 0;     // row finish: rows of more than fin_warp pieces a warp each (listed in fin)
    DevBuf hdat;             // uint16 local ids: per group [lambda][GROUP], groups segment-major
    DevBuf goff;             // int32 [ngroups+1]: each group's first step (GROUP ids per step)
    DevBuf pslot;            // int32 [ngroups*GROUP]: each piece's place in P (padding: npieces)
    DevBuf cpart;            // int32 [grid+1]: each CTA's parts (a part: one segment's groups)
    DevBuf pseg;             // int32 [nparts]: each part's segment
    DevBuf pch;              // int32 [nparts+1]: each part's chunks (claimed by its CTA's warps)
    DevBuf cb;               // int32 [nchunks+1]: chunk boundaries (group indices)
    DevBuf pair_off;         // int32 [n+1]: row v's pieces in P
    DevBuf P;                // float [npieces+1]: piece sums of the current sweep (+ padding slot)
    DevBuf toff, tcol;       // tail rows: offsets [n+1], int32 ids
    DevBuf fin;              // int32 [nfw]: the rows the finish sums a warp each
    DevBuf ctime;            // int64 [grid]: each CTA's clock cycles in the last sweep
    // host copies for re-splitting the work among the CTAs
    std::vector<int32_t> hglam, hsegg;  // steps of every group; first group of every segment
    std::vector<double> w;            // every group's cost weight
};
}  // namespace mgi

// ---------------------------------------------------------------------------
// algorithm workspaces (defined in their translation units)
// ---------------------------------------------------------------------------
struct FrontierWS;
struct PrWS;
struct CcWS;
struct BcWS;
struct PprWS;
struct WprWS;

struct mg_graph {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // double-buffered input (mg_graph_stage / mg_graph_commit)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_staged = nullptr, ev_consumed = nullptr;
    const mg_host_graph *staged_h = nullptr;
    mgi::DevBuf s_row, s_col, s_wt; // staged next input (caller order); swapped with o_* on commit
    mgi::DevBuf sym_sums;          // commit checks: pair checksum (2 x uint64), rows-differ word
    unsigned long long *sym_host = nullptr;  // pinned readback of sym_sums
    int32_t nv = 0, ne = 0;
    bool symmetric = true;         // transpose == graph (pull uses the same arrays)
    bool bc_ext = false;           // BC path counts overflowed plain FP64 once: extended from then on
    bool weights_symmetric = true; // weight of (u,v) == weight of (v,u)
    // CSR (push side, out-edges)
    mgi::DevBuf row, col, wt;
    // transpose (pull side, in-edges); aliases row/col/wt when symmetric
    mgi::DevBuf trow_own, tcol_own, twt_own;
    const int32_t *trow = nullptr, *tcol = nullptr, *twt = nullptr;
    // degree bins of the pull rows: warp rows (32 < deg <= heavy_deg) and
    // thread rows (deg <= 32), in engine order
    mgi::DevBuf wrows, trows;
    int32_t nwrows = 0, ntrows = 0;
    int32_t nwlong = 0;            // wrows[0, nwlong) have SUBWARP_MAX+ edges (a warp each)
    // heavy pull rows split into chunks: (row, begin, end) triplets
    mgi::DevBuf hchunk;            // int32 [3*nhchunks]
    int32_t nhchunks = 0;
    mgi::DevBuf hrows;             // int32 [nhrows] heavy row ids
    mgi::DevBuf hrow_chunk;        // int32 [nhrows+1] first chunk of each heavy row
    int32_t nhrows = 0;
    int32_t heavy_deg = 0;         // rows with in-degree > heavy_deg are heavy
    int32_t hchunk_size = 0;       // edges per heavy chunk
    int32_t tbin = 0;              // rows up to this in-degree are in the thread bin
    std::vector<int32_t> h_prow;   // pull-side row offsets (engine order), for re-binning
    int32_t n_dangling = 0;        // vertices with out-degree 0
    int32_t min_weight = 0;        // smallest integer edge weight
    // PPR heavy rows: rows with in-degree > PPR_HEAVY split in PPR_CHUNK pieces
    mgi::DevBuf ppr_hchunk, ppr_hrows, ppr_hrow_chunk;
    int32_t ppr_nhchunks = -1, ppr_nhrows = 0;
    // float edge weights for weighted PageRank (CSR order)
    mgi::DevBuf fw;
    bool has_fw = false;
    uint64_t fw_version = 0;       // bumped whenever fw or the CSR changes
    // hub-first relabeling: the engines run on ids ordered by descending
    // log2 degree; results are mapped back before they leave the library
    bool relabeled = false;
    bool pr_prefer_gather = false; // mg_autotune measured the gather PageRank layout faster (MG_PR_LAYOUT_AUTO)
    mgi::DevBuf o_row, o_col, o_wt;        // the CSR in the caller's ids (as uploaded)
    mgi::DevBuf o_fw;                      // float weights in caller CSR order
    mgi::DevBuf old2new, new2old;          // int32 [nv]
    mgi::DevBuf pos_row;                   // int32 [ne/32 + 2]: engine row of position 32k
    mgi::DevBuf cpos;                      // int32 [ne]: caller position of each engine position
    bool pos_valid = false;                // pos_row follows the current row offsets
    std::vector<int32_t> h_old2new;        // host copy for mapping sources
    mgi::DevBuf res_out[8];                // results in the caller's ids
    // PageRank's shared-memory segmented pull (rebuilt when the columns change)
    mgi::HubSplit hub;
    // per-algorithm workspaces
    FrontierWS *fws = nullptr;
    PrWS *pws = nullptr;
    CcWS *cws = nullptr;
    BcWS *bws = nullptr;
    PprWS *ppws = nullptr;
    WprWS *wpws = nullptr;
    mgi::Profiler prof;
    int32_t *pinned_flag = nullptr; // pinned host word for host-loop readbacks
    // result pointers for mg_result_device
    const void *res[8] = {nullptr};
};

namespace mgi {
void free_frontier_ws(mg_graph *g);
void free_pr_ws(mg_graph *g);
void free_cc_ws(mg_graph *g);
void free_bc_ws(mg_graph *g);
void free_ppr_ws(mg_graph *g);
void free_wpr_ws(mg_graph *g);
mg_status begin_run(mg_graph *g, const mg_opts *o, mg_opts &opt, mg_run_info *info);
mg_status end_run(mg_graph *g, const mg_opts &opt, mg_run_info *info);
mg_status copy_out(mg_graph *g, void *host, const void *dev, size_t bytes);
int launch_grid(const mg_graph *g, int threads, int per_sm);
// caller ids <-> engine ids (identity unless the graph was relabeled)
int32_t to_engine(const mg_graph *g, int32_t v);
// result in engine order (rows x nv elements of elem = 4 or 8 bytes) -> a
// buffer in caller order owned by the graph (slot `which`); *out = src when
// the graph is not relabeled
mg_status to_caller(mg_graph *g, int which, const void *src, size_t elem, int32_t rows, const void **out);
mg_status vertices_to_engine(mg_graph *g, const void *src_caller, void *dst_engine);  // 4-byte elements
// CC roots in engine ids -> minimum caller id of each component, per caller vertex
mg_status cc_to_caller(mg_graph *g, const int32_t *parent, const void **out);
// per-edge 4-byte payloads between caller CSR order and engine CSR order
mg_status edges_to_engine(mg_graph *g, const void *src_caller, void *dst_engine);
mg_status edges_to_caller(mg_graph *g, const void *src_engine, void *dst_caller);
// new degree bins / heavy chunks (heavy-row threshold, chunk edges, thread
// bin cutoff) from the
// host copy of the pull-side row offsets; drops the algorithm workspaces
mg_status rebin(mg_graph *g, int32_t heavy, int32_t chunk, int32_t tbin);
// batched multi-source BC over engine-id sources (symmetric graphs); the
// float scores in engine order stay in the graph's BC workspace
mg_status bc_batched(mg_graph *g, const int32_t *src_engine, int32_t nsrc, const mg_opts &opt, mg_run_info *info,
                     const float **bc_dev);
// PageRank segmented pull: build for the current pull columns (when stale),
// enqueue one sweep's pair sums (contributions c0 / c1 picked by *cur; no-op
// once *more is 0 or *off is not), report a bulk-copy wait that ran out, free
mg_status hub_prepare(mg_graph *g);
mg_status hub_launch(mg_graph *g, const float *c0, const float *c1, const int32_t *cur, const int32_t *more,
                     const int32_t *off, cudaStream_t st, int slot_sweep);
mg_status hub_check(mg_graph *g);
bool hub_covers_all(const mg_graph *g);   // the segments hold every vertex id
mg_status hub_rebalance(mg_graph *g);     // re-split the sweep's work from the last sweep's per-CTA times
bool hub_weights(mg_graph *g, std::vector<double> *get, const std::vector<double> *set);
void hub_free(mg_graph *g);

// Launch with programmatic dependent launch on the stream's previous kernel:
// the kernel may start while that one drains and must begin with
// mgd::pdl_enter() (wait for its completion and memory flush).
template <class K, class... Args>
inline mg_status launch_pdl(K kernel, int grid, int block, cudaStream_t st, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    MG_CUDA(cudaLaunchKernelEx(&cfg, kernel, args...));
    return MG_OK;
}
}  // namespace mgi

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
namespace mgd {

// Compensated (Kahan) add: t += x, r carrying the low part lost so far
// (the exact sum is t - r).  A long sum of similar terms then rounds about
// once instead of once per term.
__device__ __forceinline__ void kahan_add(float &t, float &r, float x)
{
    const float y = x - r;
    const float u = t + y;
    r = (u - t) - y;
    t = u;
}

// Warp-wide sum of the lanes' compensated sums (t - r), every lane gets the
// total: an xor tree whose adds carry their exact rounding errors (TwoSum),
// so the total rounds about once.  TwoSum is exact in either operand order,
// so every lane forms the same value.
__device__ __forceinline__ float warp_sum_comp(float t, float r)
{
    float v = t - r, c = 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float vo = __shfl_xor_sync(0xffffffffu, v, o);
        const float co = __shfl_xor_sync(0xffffffffu, c, o);
        const float u = v + vo;
        const float bp = u - v;
        const float e = (v - (u - bp)) + (vo - bp);
        c = (c + co) + e;
        v = u;
    }
    return v + c;
}

// warp-bin rows below this many edges are summed by an 8-lane group (four
// rows per warp in flight, mg_bins.cuh), longer ones by a whole warp
constexpr int32_t SUBWARP_MAX = 128;

// First statement of a kernel launched with mgi::launch_pdl (a no-op under a
// plain launch): wait for the previous kernel to complete and flush
// (griddepcontrol.wait), then let the next one launch as soon as all of
// this kernel's blocks are running (griddepcontrol.launch_dependents).
__device__ __forceinline__ void pdl_enter()
{
    cudaGridDependencySynchronize();
    cudaTriggerProgrammaticLaunchCompletion();
}


__device__ __forceinline__ int lane() { return threadIdx.x & 31; }

// warp-aggregated append: returns this lane's slot in the queue at *ctr
__device__ __forceinline__ int warp_append(int *ctr, bool pred)
{
    unsigned m = __ballot_sync(__activemask(), pred);
    if (!pred) return -1;
    int leader = __ffs(m) - 1;
    int base = 0;
    if (lane() == leader) base = atomicAdd(ctr, __popc(m));
    base = __shfl_sync(m, base, leader);
    return base + __popc(m & ((1u << lane()) - 1u));
}

// inclusive warp scan
__device__ __forceinline__ int warp_scan_incl(int v)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane() >= o) v += t;
    }
    return v;
}

// lane whose exclusive offset range [off, off+deg) contains k, given the
// exclusive offsets held one per lane (monotone).  Binary search by shuffles.
__device__ __forceinline__ int owner_lane(int excl_off, int k)
{
    int lo = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
        int probe = __shfl_sync(0xffffffffu, excl_off, lo + step);
        if (probe <= k) lo += step;
    }
    return lo;
}

// Per-warp staging of newly reached vertices: lanes push with a shared
// atomic, then the warp reserves one global slice and copies.
struct WarpStage {
    int32_t *buf;   // >= 32 entries (one per lane between flushes)
    int32_t *cnt;   // shared counter
    __device__ __forceinline__ void push(int32_t v) { buf[atomicAdd(cnt, 1)] = v; }
};

// Grid-wide barrier for persistent kernels launched cooperatively (every
// block resident).  bar[0] counts arrivals and only grows: a block's
// arrival returns the count before it, so its barrier is the one that
// completes when the count reaches the next multiple of gridDim.x, and the
// block waits for that (a block that has already left and arrives at the
// next barrier only raises the count further).  One atomic per block and a
// polled load, with no reset on the critical path (a two-level counter with
// resets and a generation word took about twice as long per barrier).  bar
// is zero before the launch, and every launch on it uses the same grid.
// The fences on both sides order every block's writes before the barrier
// against every block's reads after it.  The wait is bounded: after
// GRID_SYNC_LIMIT cycles (about 2 s) the block sets *err and the barrier
// returns false, so a broken launch ends with an error status instead of a
// hang; callers return at once on false.
constexpr long long GRID_SYNC_LIMIT = 4000000000ll;
constexpr long long GRID_SYNC_TEST_LIMIT = 20000000ll;  // ~10 ms: the injected-failure wait
constexpr unsigned GRID_SYNC_GROUPS = 32;               // words reserved after the counter

// `never` (failure injection, MG_FAIL_BARRIER): every block waits for one
// more grid's worth of arrivals than will come, so every block waits out
// GRID_SYNC_TEST_LIMIT and the barrier fails the way a lost block would
// make it fail.
__device__ __forceinline__ bool grid_sync(unsigned *bar, int *err, int never = 0)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned G = gridDim.x;
        __threadfence();
        const unsigned before = atomicAdd(&bar[0], 1u);
        const unsigned target = (before / G + 1u + (never ? 1u : 0u)) * G;
        const volatile unsigned *count = bar;
        const long long limit = never ? GRID_SYNC_TEST_LIMIT : GRID_SYNC_LIMIT;
        int ok = 1;
        const long long t0 = clock64();
        while ((int)(*count - target) < 0) {
            if (clock64() - t0 > limit) {
                ok = 0;
                atomicExch(err, 1);
                break;
            }
            __nanosleep(16);
        }
        __threadfence();
        s_ok = ok && *(volatile int *)err == 0;
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ bool bm_test(const uint32_t *bm, int v) { return (bm[v >> 5] >> (v & 31)) & 1u; }
__device__ __forceinline__ bool bm_set(uint32_t *bm, int v)  // returns true if this call set it
{
    uint32_t bit = 1u << (v & 31);
    return (atomicOr(&bm[v >> 5], bit) & bit) == 0;
}

}  // namespace mgd
