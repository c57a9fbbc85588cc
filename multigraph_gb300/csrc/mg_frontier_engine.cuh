// mg_frontier_engine.cuh -- the hybrid push/pull frontier engine, a
// template over the operator (include/mg_ops.cuh): BFS, SSSP and the BC
// forward sweep are instantiations, and so is any operator a caller defines
// with the same hooks and capability flags (include/mg_plugin.cuh).
//
// Replaces MultiGraph_V_E_V (process.cu:1079-1368) with its kernels
// process_f1 / make_frontier / phase1 / phase11 / phase2 and the sampling
// heuristic; the reference selects the operator by macro (user_function.h).
//
// The loop lives inside a CUDA graph with a device-side WHILE node; one
// pass of its body is four launches with fixed grids:
//   k_sparse_levels  (cooperative, persistent) every consecutive push level:
//            frontier queue -> neighbours (warp load-balanced search over the
//            degrees of 32 queue entries; vertices above PUSH_HEAVY split over
//            the whole grid), claims / relaxes destinations with the
//            operator hooks, appends the next queue with warp-aggregated
//            atomics and sets the next-frontier bitmap; one grid barrier
//            per level, after which every block takes the end-of-level
//            decision itself from the level's counters;
//   k_pull   (when the frontier is dense) every candidate row scans its
//            in-edges against the frontier bitmap (first-parent operators
//            stop at the first parent; the others fold every frontier
//            offer), light rows in degree bins (warp / thread per row),
//            heavy rows in 2048-edge chunks;
//   k_compact (after a pull) next queue from the next-frontier bitmap;
//   k_decide 1 warp: next size, direction switch (frontier edges against
//            unvisited edges, Beamer), iteration cap, loop condition.
// The push phase returns as soon as the switch picks pull; k_pull /
// k_compact / k_decide then run one dense level and the body repeats.
// Frontier bitmaps are triple-buffered: the active kernel clears the buffer
// the next iteration will write.
#pragma once

#include "mg_device.cuh"
#include "mg_ops.cuh"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <type_traits>

namespace {

constexpr int MODE_PUSH = 0, MODE_PULL = 1;
constexpr int32_t PUSH_HEAVY = 4096;
constexpr int THREADS = 256;
constexpr int PTHREADS = 1024;  // persistent kernels: 2 CTAs of 1024 per SM (fewer barrier arrivals)
// grid barrier words (2 + GRID_SYNC_GROUPS), the barrier error flag, the BC
// path-count overflow flag, rounded up
constexpr size_t BAR_BYTES = 4 * (2 + mgd::GRID_SYNC_GROUPS + 1 + 7);
constexpr int OVF_WORD = 2 + mgd::GRID_SYNC_GROUPS + 1;
constexpr int FMIN_WORD = OVF_WORD + 1;  // SSSP: least distance on the current frontier (pull levels)

struct FCtl {
    int32_t more;       // continue flag (host loop readback)
    int32_t iter;       // level / round being expanded
    int32_t mode;       // MODE_PUSH / MODE_PULL
    int32_t cur;        // current bitmap buffer 0..2
    int32_t qoff, qsize;  // current queue slice
    int32_t nqoff, nq;    // next queue slice (nq: atomic counter)
    int32_t hcur, nhcur;  // heavy list sizes: current / next (atomic)
    int32_t hpar;         // heavy list parity
    int32_t status;       // 0 ok, 1 iteration cap
    int32_t pull_iters;
    int32_t max_iter;
    int32_t dirmode;      // MG_DIR_*
    int32_t alpha, beta;
    int32_t nlevels;      // BC: levels archived
    int32_t archive;      // 1: queue slices are appended (BFS/BC), 0: ping-pong (SSSP)
    int32_t pad0;
    long long nf_edges;      // out-edges of the next frontier (atomic)
    long long visited_edges; // out-edges of every vertex visited so far
    long long scanned;       // edges scanned (statistics, atomic)
};

struct Args {
    int32_t n;
    int32_t m;
    const int32_t *row, *col, *wt;     // push side
    const int32_t *trow, *tcol, *twt;  // pull side
    const int32_t *wrows, *trows;  // degree bins of the pull rows
    int32_t nwrows, ntrows, nwlong;
    const int32_t *hchunk;
    int32_t nhchunks;
    int32_t heavy_deg;
    int32_t *label;
    mgops::PathCount *sigma;
    int32_t bc_ext;      // BC path counts in extended mode (mgops::PathCount)
    int32_t *bc_ovf;     // set when a plain-mode path count reaches mgops::PC_PLAIN_MAX
    int32_t *fmin;       // SSSP pull levels: least distance on the frontier (k_fmin)
    int32_t wmin;        // least edge weight
    uint32_t *bm;        // 3 * words
    uint32_t *visited;
    int32_t words;
    int32_t *queue;
    int32_t *heavy;      // 2 * n (parity)
    int32_t *lvl_off;
    FCtl *ctl;
    unsigned *bar;       // grid barrier words of the persistent kernels
    int *bar_err;        // set when a grid barrier wait times out
    int bar_never;       // failure injection: barriers never complete (MG_FAIL_BARRIER)
    struct LevelCnt *cnt;  // persistent push phase: per-level counters, 4 rotating slots
};

// Counters one push level produces (next queue size, heavy entries, next
// frontier's out-edges).  The persistent push phase keeps them in 4 slots
// by level mod 4, so every block can read level L's counters after the one
// barrier while level L+1 appends to the next slot; block 0 clears slot
// L+2 during level L (its last readers finished before the barrier that
// began level L).
struct LevelCnt {
    int32_t nq;
    int32_t nhcur;
    long long nfe;
};

__device__ __forceinline__ uint32_t *bm_buf(const Args &a, int idx) { return a.bm + (size_t)idx * a.words; }

// The loop state as the persistent kernel re-reads it after every grid
// barrier: through L2, never from a stale L1 line.
static_assert(sizeof(FCtl) % 8 == 0, "FCtl is copied as 8-byte words");
__device__ __forceinline__ FCtl load_ctl(const FCtl *p)
{
    FCtl c;
    const int2 *s = reinterpret_cast<const int2 *>(p);
    int2 *d = reinterpret_cast<int2 *>(&c);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(FCtl) / 8); i++) d[i] = __ldcg(s + i);
    return c;
}

// warp-wide: add v (64-bit) from every lane to *dst with one atomic
__device__ __forceinline__ void warp_add64(long long *dst, long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (mgd::lane() == 0 && v) atomicAdd((unsigned long long *)dst, (unsigned long long)v);
}

// record a newly reached vertex in the next frontier (push sweeps; all lanes
// call).  A relaxed operator has already set the vertex's bit when it
// improved it.
template <class Op>
__device__ __forceinline__ void emit_next(const Args &a, const FCtl &c, int nextbuf, bool found, int32_t v,
                                          long long &dsum, int32_t *nq, int32_t *nhcur)
{
    int slot = mgd::warp_append(nq, found);
    if (found) {
        a.queue[c.nqoff + slot] = v;
        if (Op::kLevelSync) mgd::bm_set(bm_buf(a, nextbuf), v);
        int32_t dg = a.row[v + 1] - a.row[v];
        dsum += dg;
        if (dg > PUSH_HEAVY) {
            int h = atomicAdd(nhcur, 1);
            a.heavy[(size_t)(c.hpar ^ 1) * a.n + h] = v;
        }
    }
}

// ----------------------------------------------------------------------------
// push: one edge (u -> v) with the source's payload
// ----------------------------------------------------------------------------
template <class Op>
__device__ __forceinline__ bool push_edge(const Args &a, int it1, int32_t v, int32_t payload_i,
                                          mgops::PathCount payload_d, int32_t w, uint32_t *next_bm)
{
    if constexpr (Op::kPathCounts) {
        // claim at this level, or collect the path count on it
        bool on_level;
        bool claimed = Op::fused_update_condition(&a.label[v], it1, on_level);
        if (on_level) Op::accumulate(&a.sigma[v], payload_d, a.bc_ext != 0, a.bc_ovf);
        if (claimed) mgd::bm_set(a.visited, v);
        return claimed;
    } else if constexpr (Op::kLevelSync) {
        // the visited bitmap claims the vertex once; its label is the level
        if (mgd::bm_test(a.visited, v)) return false;
        if (!mgd::bm_set(a.visited, v)) return false;
        a.label[v] = Op::get_partial_result(it1 - 1, w);
        return true;
    } else {
        // relaxation: the offer folded in with one atomic; an improved
        // vertex enters the next frontier once (its bit)
        const int32_t nd = Op::get_partial_result(payload_i, w);
        if (!Op::update_condition(a.label[v], nd, it1)) return false;
        if (!Op::fused_update_condition(&a.label[v], nd, it1)) return false;
        return mgd::bm_set(next_bm, v);
    }
}

// One push level.  Queue entries, heavy entries and the frontier's labels /
// path counts were written by other blocks in the previous level, so they
// are loaded through L2 (__ldcg): the persistent kernel runs many levels in
// one launch.
template <class Op>
__device__ __forceinline__ void push_level(const Args &a, const FCtl &c, LevelCnt *lc)
{
    const int it1 = c.iter + 1;
    const int nextbuf = (c.cur + 1) % 3, sparebuf = (c.cur + 2) % 3;
    // clear the buffer the next iteration writes
    {
        uint32_t *sp = bm_buf(a, sparebuf);
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.words; i += gridDim.x * blockDim.x) sp[i] = 0;
    }
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    long long scanned = 0, dsum = 0;
    // heavy frontier vertices: every thread of the grid strides over their edges
    for (int h = 0; h < c.hcur; h++) {
        int32_t u = __ldcg(&a.heavy[(size_t)c.hpar * a.n + h]);
        int32_t b = a.row[u], e = a.row[u + 1];
        int32_t pi = __ldcg(&a.label[u]);
        const mgops::PathCount pd = Op::kPathCounts ? mgops::pc_load_cg(&a.sigma[u]) : mgops::pc_zero();
        if (Op::kPathCounts && !a.bc_ext && pd.m >= mgops::PC_PLAIN_MAX) *a.bc_ovf = 1;
        int32_t span = e - b;
        int32_t rounds = (span + gridDim.x * blockDim.x - 1) / (gridDim.x * blockDim.x);
        for (int r = 0; r < rounds; r++) {
            int32_t k = b + r * gridDim.x * blockDim.x + blockIdx.x * blockDim.x + threadIdx.x;
            bool found = false;
            int32_t v = 0;
            if (k < e) {
                v = a.col[k];
                found = push_edge<Op>(a, it1, v, pi, pd, Op::kWeighted ? a.wt[k] : 0, bm_buf(a, nextbuf));
            }
            emit_next<Op>(a, c, nextbuf, found, v, dsum, &lc->nq, &lc->nhcur);
        }
        scanned += (threadIdx.x == 0 && blockIdx.x == 0) ? span : 0;
    }
    // light frontier vertices: vpw per warp (32, or fewer when the frontier
    // would leave warps idle), load-balanced over their edges
    int vpw = 32;
    if (c.qsize < nwarps * 32) {
        const int want = max(1, c.qsize / nwarps);
        vpw = 1;
        while (vpw * 2 <= want) vpw *= 2;
    }
    for (int base = gwarp * vpw; base < c.qsize; base += nwarps * vpw) {
        int32_t u = -1, start = 0, deg = 0, pi = 0;
        mgops::PathCount pd = mgops::pc_zero();
        if (lane < vpw && base + lane < c.qsize) {
            u = __ldcg(&a.queue[c.qoff + base + lane]);
            start = a.row[u];
            deg = a.row[u + 1] - start;
            if (deg > PUSH_HEAVY) deg = 0;
            pi = __ldcg(&a.label[u]);
            if (Op::kPathCounts) {
                pd = mgops::pc_load_cg(&a.sigma[u]);
                if (!a.bc_ext && pd.m >= mgops::PC_PLAIN_MAX) *a.bc_ovf = 1;
            }
        }
        int incl = mgd::warp_scan_incl(deg);
        int excl = incl - deg;
        int total = __shfl_sync(0xffffffffu, incl, 31);
        scanned += (lane == 0) ? total : 0;
        for (int k0 = 0; k0 < total; k0 += 32) {
            int k = k0 + lane;
            int kk = k < total ? k : total - 1;
            int own = mgd::owner_lane(excl, kk);
            int32_t e = __shfl_sync(0xffffffffu, start, own) + (kk - __shfl_sync(0xffffffffu, excl, own));
            int32_t opi = __shfl_sync(0xffffffffu, pi, own);
            const mgops::PathCount opd = Op::kPathCounts ? mgops::shfl_val(pd, own) : pd;
            bool found = false;
            int32_t v = 0;
            if (k < total) {
                v = a.col[e];
                found = push_edge<Op>(a, it1, v, opi, opd, Op::kWeighted ? a.wt[e] : 0, bm_buf(a, nextbuf));
            }
            emit_next<Op>(a, c, nextbuf, found, v, dsum, &lc->nq, &lc->nhcur);
        }
    }
    warp_add64(&lc->nfe, dsum);
    if (lane == 0 && scanned) atomicAdd((unsigned long long *)&a.ctl->scanned, (unsigned long long)scanned);
}

// ----------------------------------------------------------------------------
// pull: row reductions over in-edges against the frontier bitmap
// ----------------------------------------------------------------------------
// A pull sweep only marks the rows it reaches in the next-frontier bitmap
// (atomicOr on distinct words, no shared counter); k_compact then builds the
// queue, the frontier's edge count and its heavy list from the bitmap.
struct PullEmit {
    const Args &a;
    uint32_t *next_bm;
    __device__ void flush() {}
};

// Relaxed operators: fold the offers of frontier in-neighbours in row order
// (accumulate_nonAtomics), then one fused update + next-frontier bit on the
// row.  With a dense frontier (all_in) every in-neighbour's offer is folded
// without the bitmap test: operators are monotone (mg_ops.cuh), so offers of
// unreached or earlier-relaxed vertices never spoil a label, labels still
// converge to the same fixed point, and one dependent load per edge goes away.
//
// Min-plus operators (kMinPlusBound) skip rows whose label is at most (least
// frontier label + least weight): every offer is label[u] + w from a
// frontier vertex u, or from a vertex whose edges an earlier level already
// relaxed, so such a row cannot improve this level.  On R-MAT the hubs
// settle first, so the later pull levels read a fraction of the edges.
template <class Op>
struct PullRelax : PullEmit {
    using T = int32_t;
    static constexpr bool kRowAware = Op::kMinPlusBound;
    static constexpr bool kWeights = Op::kWeighted;
    const uint32_t *fb;
    int it1;
    bool all_in;
    int32_t bound;
    __device__ T identity() const { return Op::initialize(); }
    __device__ bool skip(int32_t v) const { return a.label[v] <= bound; }
    __device__ T edge(int32_t, int32_t, int32_t u, int32_t w) const
    {
        if (!all_in && !mgd::bm_test(fb, u)) return Op::initialize();
        return Op::get_partial_result(a.label[u], w);
    }
    __device__ T combine(T x, T y) const
    {
        Op::accumulate_nonAtomics(x, y, it1);
        return x;
    }
    __device__ void finish(int32_t v, T best)
    {
        if (Op::update_condition(a.label[v], best, it1) && Op::fused_update_condition(&a.label[v], best, it1))
            mgd::bm_set(next_bm, v);
    }
};

// Path-count operators (BC forward): unvisited rows sum the path counts of
// frontier in-neighbours
template <class Op>
struct PullCounts : PullEmit {
    using T = mgops::PathCount;
    static constexpr bool kRowAware = true;  // visited rows are skipped
    static constexpr bool kWeights = false;
    const uint32_t *fb;
    int it1;
    bool all_in;
    int32_t bound;
    __device__ T identity() const { return mgops::pc_zero(); }
    __device__ bool skip(int32_t v) const { return mgd::bm_test(a.visited, v); }
    __device__ T edge(int32_t, int32_t, int32_t u, int32_t) const
    {
        return mgd::bm_test(fb, u) ? a.sigma[u] : mgops::pc_zero();
    }
    __device__ T combine(T x, T y) const
    {
        Op::accumulate_nonAtomics(x, y, a.bc_ext != 0);
        return x;
    }
    __device__ void finish(int32_t v, T s)
    {
        if (s.m > 0.0) {
            a.label[v] = it1;
            a.sigma[v] = s;
            if (!a.bc_ext && s.m >= mgops::PC_PLAIN_MAX) *a.bc_ovf = 1;
            mgd::bm_set(a.visited, v);
            mgd::bm_set(next_bm, v);
        }
    }
};

template <class Op>
using PullOp = std::conditional_t<Op::kPathCounts, PullCounts<Op>, PullRelax<Op>>;

// min-plus pull levels: rows at or below this label cannot improve
__device__ __forceinline__ int32_t sssp_bound(const Args &a)
{
    const int32_t f = *a.fmin;
    return f >= INT32_MAX - a.wmin ? INT32_MAX : f + a.wmin;
}

// least label over the frontier queue (before a min-plus pull level)
__global__ void __launch_bounds__(THREADS) k_fmin(Args a)
{
    const FCtl c = *a.ctl;
    if (c.mode != MODE_PULL || c.more == 0) return;
    int32_t mn = INT32_MAX;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < c.qsize; i += gridDim.x * blockDim.x)
        mn = min(mn, a.label[a.queue[c.qoff + i]]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    if (mgd::lane() == 0 && mn < INT32_MAX) atomicMin(a.fmin, mn);
}

template <class Op>
__global__ void __launch_bounds__(THREADS) k_pull(Args a)
{
    const FCtl c = *a.ctl;
    if (c.mode != MODE_PULL || c.more == 0) return;
    const int it1 = c.iter + 1;
    const int nextbuf = (c.cur + 1) % 3, sparebuf = (c.cur + 2) % 3;
    const uint32_t *fb = bm_buf(a, c.cur);
    {
        uint32_t *sp = bm_buf(a, sparebuf);
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.words; i += gridDim.x * blockDim.x) sp[i] = 0;
    }
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    long long scanned = 0;

    if constexpr (Op::kFirstParent) {
        // bottom-up: a thread per unvisited light row, first frontier parent wins
        const int32_t stride = gridDim.x * blockDim.x;
        const int32_t nround = (a.n + stride - 1) / stride;
        for (int32_t r = 0; r < nround; r++) {
            int32_t v = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
            bool found = false;
            if (v < a.n && !mgd::bm_test(a.visited, v)) {
                int32_t b = a.trow[v], e = a.trow[v + 1];
                if (e - b <= a.heavy_deg) {
                    for (int32_t p = b; p < e; p++) {
                        scanned++;
                        if (mgd::bm_test(fb, a.tcol[p])) { found = true; break; }
                    }
                    if (found) {
                        a.label[v] = it1;
                        mgd::bm_set(a.visited, v);
                        mgd::bm_set(bm_buf(a, nextbuf), v);
                    }
                }
            }
        }
    } else {
        // degree-binned rows; reached rows marked in the next-frontier bitmap
        PullOp<Op> op{{a, bm_buf(a, nextbuf)}, fb, it1, false, 0};
        if constexpr (!Op::kLevelSync) op.all_in = (long long)c.qsize * 8 > a.n;
        if constexpr (Op::kMinPlusBound) op.bound = sssp_bound(a);
        mgd::bins_reduce(op, a.trow, a.tcol, a.twt, a.wrows, a.nwrows, a.nwlong, a.trows, a.ntrows);
        (void)gwarp;
        (void)nwarps;
    }

    // heavy rows: one CTA per 2048-edge chunk
    __shared__ int32_t s_min[THREADS / 32];
    __shared__ mgops::PathCount s_sum[THREADS / 32];
    __shared__ int s_hit, s_skip;
    for (int32_t ch = blockIdx.x; ch < a.nhchunks; ch += gridDim.x) {
        int32_t v = a.hchunk[3 * ch], b = a.hchunk[3 * ch + 1], e = a.hchunk[3 * ch + 2];
        // thread 0 decides for the block (the row may be claimed concurrently
        // by another chunk, so a per-thread test could diverge).  BFS / BC
        // skip only rows reached at an earlier level; the label is read from
        // L2: hub-first ids put the heavy rows' labels in a few lines, and an
        // L1 copy from an earlier chunk can predate this level's claim, which
        // would drop this chunk's share of the row's path count
        if (threadIdx.x == 0) {
            if constexpr (!Op::kLevelSync) {
                s_skip = Op::kMinPlusBound && a.label[v] <= sssp_bound(a);
            } else {
                const int32_t lv = __ldcg(&a.label[v]);
                s_skip = lv != mgops::UNSET && lv != it1;
            }
        }
        __syncthreads();
        const bool skip = s_skip;
        __syncthreads();
        if (skip) continue;
        int32_t best = Op::initialize();
        mgops::PathCount ssum = mgops::pc_zero();
        const bool ext = a.bc_ext != 0;
        int hit = 0;
        const bool all_in = !Op::kLevelSync && (long long)c.qsize * 8 > a.n;  // as PullRelax
        for (int32_t p = b + threadIdx.x; p < e; p += blockDim.x) {
            int32_t u = __ldcs(&a.tcol[p]);  // streamed once: evict-first
            if (all_in || mgd::bm_test(fb, u)) {
                hit = 1;
                if constexpr (!Op::kLevelSync)
                    Op::accumulate_nonAtomics(best, Op::get_partial_result(a.label[u], Op::kWeighted ? a.twt[p] : 0),
                                              it1);
                if constexpr (Op::kPathCounts) ssum = mgops::pc_add(ssum, a.sigma[u], ext);
            }
        }
        if (threadIdx.x == 0) s_hit = 0;
        __syncthreads();
        if (hit) s_hit = 1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            if constexpr (!Op::kLevelSync) Op::accumulate_nonAtomics(best, __shfl_xor_sync(0xffffffffu, best, o), it1);
            if constexpr (Op::kPathCounts) ssum = mgops::pc_add(ssum, mgops::shfl_xor_val(ssum, o), ext);
        }
        if (lane == 0) { s_min[threadIdx.x >> 5] = best; s_sum[threadIdx.x >> 5] = ssum; }
        __syncthreads();
        if (threadIdx.x == 0) {
            int32_t bm = Op::initialize();
            mgops::PathCount bs = mgops::pc_zero();
            for (int w = 0; w < THREADS / 32; w++) {
                if constexpr (!Op::kLevelSync) Op::accumulate_nonAtomics(bm, s_min[w], it1);
                if constexpr (Op::kPathCounts) bs = mgops::pc_add(bs, s_sum[w], ext);
            }
            uint32_t *nb = bm_buf(a, nextbuf);
            if (s_hit) {
                if constexpr (Op::kFirstParent) {
                    if (atomicCAS(&a.label[v], Op::initialize(), it1) == Op::initialize()) {
                        mgd::bm_set(a.visited, v);
                        mgd::bm_set(nb, v);
                    }
                } else if constexpr (!Op::kLevelSync) {
                    if (Op::update_condition(a.label[v], bm, it1) && Op::fused_update_condition(&a.label[v], bm, it1))
                        mgd::bm_set(nb, v);
                } else {
                    bool on_level;
                    bool found = Op::fused_update_condition(&a.label[v], it1, on_level);
                    if (on_level) Op::accumulate(&a.sigma[v], bs, ext, a.bc_ovf);
                    if (found) {
                        mgd::bm_set(a.visited, v);
                        mgd::bm_set(nb, v);
                    }
                }
            }
            scanned += e - b;
        }
        __syncthreads();
    }
    warp_add64(&a.ctl->scanned, scanned);
}

// ----------------------------------------------------------------------------
// compact: after a pull sweep, the next frontier's bitmap -> queue slice,
// edge count and heavy list.  Each warp takes 32 bitmap words (1024
// vertices) and reserves its queue slots with one atomicAdd.
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(THREADS) k_compact(Args a)
{
    const FCtl c = *a.ctl;
    if (c.mode != MODE_PULL || c.more == 0) return;
    const uint32_t *nb = bm_buf(a, (c.cur + 1) % 3);
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    long long dsum = 0;
    for (int32_t w0 = gwarp * 32; w0 < a.words; w0 += nwarps * 32) {
        const int32_t wi = w0 + lane;
        uint32_t bits = wi < a.words ? nb[wi] : 0u;
        const int cnt = __popc(bits);
        const int incl = mgd::warp_scan_incl(cnt);
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        int base = 0;
        if (lane == 31 && total) base = atomicAdd(&a.ctl->nq, total);
        base = __shfl_sync(0xffffffffu, base, 31) + incl - cnt;
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1;
            const int32_t v = wi * 32 + b;
            a.queue[c.nqoff + base++] = v;
            const int32_t dg = a.row[v + 1] - a.row[v];
            dsum += dg;
            if (dg > PUSH_HEAVY) a.heavy[(size_t)(c.hpar ^ 1) * a.n + atomicAdd(&a.ctl->nhcur, 1)] = v;
        }
    }
    warp_add64(&a.ctl->nf_edges, dsum);
}

// ----------------------------------------------------------------------------
// decide: 1 thread
// ----------------------------------------------------------------------------
__device__ __forceinline__ void store_ctl(FCtl *p, const FCtl &c)
{
    int2 *d = reinterpret_cast<int2 *>(p);
    const int2 *s = reinterpret_cast<const int2 *>(&c);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(FCtl) / 8); i++) d[i] = s[i];
}

// The end-of-level decision on a copy of the loop state, given the level's
// counters; block 0 (write_lvl) also records the level offset.
__device__ __forceinline__ int decide_local(const Args &a, FCtl &c, int32_t nq, int32_t nhcur, long long nfe_in,
                                            bool write_lvl)
{
    int more = c.more;
    if (more) {
        if (c.mode == MODE_PULL) c.pull_iters++;
        c.iter += 1;
        if (c.archive && c.iter + 1 < a.n + 3) {
            if (write_lvl) a.lvl_off[c.iter + 1] = c.nqoff + nq;
            if (nq > 0) c.nlevels = c.iter + 1;
        }
        c.qoff = c.nqoff;
        c.qsize = nq;
        c.nqoff = c.archive ? (c.qoff + nq) : (c.qoff == 0 ? a.n : 0);
        c.nq = 0;
        c.hcur = nhcur;
        c.nhcur = 0;
        c.hpar ^= 1;
        c.cur = (c.cur + 1) % 3;
        const long long nfe = nfe_in;
        c.visited_edges += nfe;
        c.nf_edges = 0;
        if (nq == 0) {
            more = 0;
        } else {
            if (c.dirmode == MG_DIR_PUSH) c.mode = MODE_PUSH;
            else if (c.dirmode == MG_DIR_PULL) c.mode = MODE_PULL;
            else if (c.archive) {
                // Beamer: push -> pull when frontier edges exceed unvisited
                // edges / alpha; pull -> push when the frontier is below n / beta
                const long long unvisited = (long long)a.m - c.visited_edges;
                if (c.mode == MODE_PUSH) {
                    if (nfe * (long long)c.alpha > unvisited && nq > 64) c.mode = MODE_PULL;
                } else {
                    if ((long long)nq * c.beta < a.n) c.mode = MODE_PUSH;
                }
            } else {
                // SSSP: pull when the frontier's edges are a large share of m
                c.mode = (nfe * (long long)c.alpha > (long long)a.m) ? MODE_PULL : MODE_PUSH;
            }
            if (c.iter >= c.max_iter) { c.status = 1; more = 0; }
        }
        c.more = more;
    }
    return more;
}

// End of a level (one thread, no other thread touching the loop state):
// next queue slice, direction switch, caps.  Works on a register copy (one
// batch of parallel loads, one batch of stores).  Returns the continue flag.
__device__ __forceinline__ int decide_step(const Args &a)
{
    FCtl c = load_ctl(a.ctl);
    if (c.more == 0) return 0;
    const int more = decide_local(a, c, c.nq, c.nhcur, c.nf_edges, true);
    store_ctl(a.ctl, c);
    return more;
}

__global__ void k_decide(Args a, cudaGraphConditionalHandle h, int use_cond)
{
    if (threadIdx.x != 0) return;
    *a.fmin = INT32_MAX;  // the next pull level's k_fmin starts from here
    const int more = decide_step(a);
    if (use_cond) cudaGraphSetConditional(h, more ? 1u : 0u);
}

// Persistent push phase: consecutive push levels in one cooperative launch,
// one grid barrier per level (push level | barrier | every block decides
// from the level's counters on its own copy of the loop state, the same
// inputs giving the same decision everywhere), until the traversal ends or
// the direction switch picks pull; block 0 writes the loop state back.
// High-diameter graphs (lattices, road networks) spend thousands of levels
// here, each a few microseconds instead of a round of kernel launches.  A
// barrier timeout sets status 3 and ends the traversal.
// Every block reads the loop state once per level: one warp loads it
// (one L2 request per block instead of one per warp) and shares it.
__device__ __forceinline__ FCtl block_load_ctl(const FCtl *p)
{
    __shared__ int2 s_c[sizeof(FCtl) / 8];
    if (threadIdx.x < sizeof(FCtl) / 8) s_c[threadIdx.x] = __ldcg(reinterpret_cast<const int2 *>(p) + threadIdx.x);
    __syncthreads();
    FCtl c;
    int2 *d = reinterpret_cast<int2 *>(&c);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(FCtl) / 8); i++) d[i] = s_c[i];
    __syncthreads();
    return c;
}

template <class Op>
__global__ void __launch_bounds__(PTHREADS, 2) k_sparse_levels(Args a)
{
    __shared__ FCtl s_c;
    __shared__ int4 s_cnt;
    {
        const FCtl c0 = block_load_ctl(a.ctl);
        if (threadIdx.x == 0) s_c = c0;
        __syncthreads();
    }
    bool ran = false;
    for (int32_t lv = 0; lv <= a.n + 2; lv++) {
        if (s_c.more == 0 || s_c.mode != MODE_PUSH) break;
        ran = true;
        LevelCnt *lc = a.cnt + (lv & 3);
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            LevelCnt *z = a.cnt + ((lv + 2) & 3);
            z->nq = 0;
            z->nhcur = 0;
            z->nfe = 0;
        }
        push_level<Op>(a, s_c, lc);
        if (!mgd::grid_sync(a.bar, a.bar_err, a.bar_never)) break;
        if (threadIdx.x == 0) {
            s_cnt = __ldcg(reinterpret_cast<const int4 *>(lc));  // nq, nhcur, nfe (lo, hi)
            FCtl c = s_c;
            const long long nfe = (long long)(((unsigned long long)(unsigned)s_cnt.w << 32) | (unsigned)s_cnt.z);
            decide_local(a, c, s_cnt.x, s_cnt.y, nfe, blockIdx.x == 0);
            s_c = c;
        }
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        FCtl c = s_c;
        if (*(volatile int *)a.bar_err) {
            c.status = 3;
            c.more = 0;
        }
        if (ran || c.status) {
            // the loop state back to global memory for the other kernels,
            // all but the last word (the scanned-edges statistic, which the
            // push levels add to atomically)
            int2 *d = reinterpret_cast<int2 *>(a.ctl);
            const int2 *src = reinterpret_cast<const int2 *>(&c);
            for (int i = 0; i < (int)(sizeof(FCtl) / 8) - 1; i++) d[i] = src[i];
        }
    }
}

// ----------------------------------------------------------------------------
// init: source
// ----------------------------------------------------------------------------
// sources: srcs[0..nsrc) when srcs is non-null, else the single `src`
// (several sources = one traversal of a disjoint union of graphs)
template <class Op>
__global__ void k_init(Args a, int32_t src, const int32_t *srcs, int32_t nsrc, int dirmode, int alpha, int beta,
                       int max_iter)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    FCtl *c = a.ctl;
    std::memset(c, 0, sizeof(FCtl));
    c->more = 1;
    c->archive = Op::kLevelSync;
    c->max_iter = max_iter;
    c->dirmode = dirmode;
    c->alpha = alpha;
    c->beta = beta;
    c->mode = (dirmode == MG_DIR_PULL) ? MODE_PULL : MODE_PUSH;
    int32_t q = 0;
    long long ve = 0;
    for (int32_t i = 0; i < (srcs ? nsrc : 1); i++) {
        int32_t s = srcs ? srcs[i] : src;
        if (!mgd::bm_set(a.visited, s)) continue;  // duplicate source
        a.label[s] = Op::source_value();
        if (Op::kPathCounts) a.sigma[s] = mgops::pc_one();
        mgd::bm_set(a.bm, s);  // buffer 0 is the current frontier
        a.queue[q++] = s;
        int32_t d = a.row[s + 1] - a.row[s];
        ve += d;
        if (d > PUSH_HEAVY) a.heavy[c->hcur++] = s;
    }
    c->qoff = 0;
    c->qsize = q;
    c->nqoff = Op::kLevelSync ? q : a.n;
    c->visited_edges = ve;
    if (Op::kLevelSync) { a.lvl_off[0] = 0; a.lvl_off[1] = q; c->nlevels = 1; }
    *a.fmin = INT32_MAX;
}

// ----------------------------------------------------------------------------

// every vertex's label = the operator's initial value
template <class Op>
__global__ void k_label_init(int32_t *label, int32_t n)
{
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        label[v] = Op::initialize();
}

// per-instantiation tag: its address keys the workspace's captured loop and
// the persistent kernel's resident grid for this operator
template <class Op>
struct OpTag {
    static const char id;
};
template <class Op>
const char OpTag<Op>::id = 0;

}  // namespace

// ----------------------------------------------------------------------------
// workspace (shared by every operator run on a graph; freed with the graph)
// ----------------------------------------------------------------------------
struct FrontierWS {
    mgi::DevBuf label, sigma, sigma_d, bm, visited, queue, heavy, lvl_off, ctl;
    mgi::DevBuf q, delta, bc, bctl, bheavy, srcbuf;
    mgi::DevBuf bar;        // grid barrier words + error flag of the persistent kernels
    mgi::DevBuf cnt;        // LevelCnt[4] of the persistent push phase
    std::map<const void *, int> coop_grid;      // resident blocks of k_sparse_levels<Op>, by operator tag
    int coop_back = 0;                          // resident blocks of k_bc_back_levels
    std::map<const void *, mgi::LoopGraph> lg;  // captured loop per operator tag
};

namespace {

using namespace mgi;

template <class Op>
mg_status ensure_ws(mg_graph *g)
{
    if (!g->fws) g->fws = new FrontierWS();
    FrontierWS *w = g->fws;
    const size_t n = (size_t)std::max(g->nv, 1);
    const size_t words = (n + 31) / 32;
    MG_TRY(dev_alloc(w->label, n * 4));
    MG_TRY(dev_alloc(w->bm, 3 * words * 4));
    MG_TRY(dev_alloc(w->visited, words * 4));
    MG_TRY(dev_alloc(w->queue, 2 * n * 4));
    MG_TRY(dev_alloc(w->heavy, 2 * n * 4));
    MG_TRY(dev_alloc(w->ctl, sizeof(FCtl)));
    MG_TRY(dev_alloc(w->lvl_off, (n + 3) * 4));
    MG_TRY(dev_alloc(w->bar, BAR_BYTES));
    MG_TRY(dev_alloc(w->cnt, 4 * sizeof(LevelCnt)));
    if (Op::kPathCounts) MG_TRY(dev_alloc(w->sigma, n * sizeof(mgops::PathCount)));
    int &cg = w->coop_grid[&OpTag<Op>::id];
    if (cg == 0) {
        int per_sm = 0;
        MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sparse_levels<Op>, PTHREADS, 0));
        if (per_sm < 1) return fail(MG_ERR_CUDA, "persistent push kernel does not fit on an SM");
        cg = std::min(per_sm, 2) * g->num_sms;
    }
    return MG_OK;
}

// cooperative launch (all blocks resident) of the persistent push phase
template <class Op>
mg_status launch_sparse_levels(const Args &a, int grid, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(PTHREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    MG_CUDA(cudaLaunchKernelEx(&cfg, k_sparse_levels<Op>, a));
    return MG_OK;
}

inline Args make_args(mg_graph *g)
{
    FrontierWS *w = g->fws;
    Args a;
    std::memset(&a, 0, sizeof(a));
    a.n = g->nv;
    a.m = g->ne;
    a.row = g->row.as<int32_t>(); a.col = g->col.as<int32_t>(); a.wt = g->wt.as<int32_t>();
    a.trow = g->trow; a.tcol = g->tcol; a.twt = g->twt;
    a.wrows = g->wrows.as<int32_t>(); a.nwrows = g->nwrows; a.nwlong = g->nwlong;
    a.trows = g->trows.as<int32_t>(); a.ntrows = g->ntrows;
    a.hchunk = g->hchunk.as<int32_t>(); a.nhchunks = g->nhchunks;
    a.heavy_deg = g->heavy_deg;
    a.label = w->label.as<int32_t>();
    a.sigma = w->sigma.as<mgops::PathCount>();
    a.bc_ext = g->bc_ext ? 1 : 0;
    a.bc_ovf = reinterpret_cast<int32_t *>(w->bar.as<unsigned>() + OVF_WORD);
    a.fmin = reinterpret_cast<int32_t *>(w->bar.as<unsigned>() + FMIN_WORD);
    a.wmin = std::max(g->min_weight, 0);
    a.bm = w->bm.as<uint32_t>();
    a.visited = w->visited.as<uint32_t>();
    a.words = (std::max(g->nv, 1) + 31) / 32;
    a.queue = w->queue.as<int32_t>();
    a.heavy = w->heavy.as<int32_t>();
    a.lvl_off = w->lvl_off.as<int32_t>();
    a.ctl = w->ctl.as<FCtl>();
    a.bar = w->bar.as<unsigned>();
    a.cnt = w->cnt.as<LevelCnt>();
    a.bar_err = reinterpret_cast<int *>(w->bar.as<unsigned>() + 2 + mgd::GRID_SYNC_GROUPS);
    // failure injection for tests: the persistent kernels' barriers never
    // complete, their bounded waits run out and the run reports an error
    const char *fb = std::getenv("MG_FAIL_BARRIER");
    a.bar_never = (fb && fb[0] == '1') ? 1 : 0;
    return a;
}

// every by-value argument of the captured kernels: the whole Args (pointers,
// sizes, the min-plus skip bound's least weight, the injection flag, the
// path-count mode), the operator and the launch grids
inline LoopKey key_of(const Args &a, const void *op_tag, int grid, int coop_grid)
{
    return LoopKey().add(op_tag).add(a).add(grid).add(coop_grid);
}

// Forward traversal with operator Op from src (or from the nsrc sources in
// srcs_host when it is non-null); results stay in the workspace.
template <class Op>
mg_status frontier_run_impl(mg_graph *g, int32_t src, const int32_t *srcs_host, int32_t nsrc, const mg_opts &opt,
                            mg_run_info *info)
{
    static_assert(!Op::kLevelSync || Op::kFirstParent || Op::kPathCounts,
                  "a level-synchronous operator is first-parent (BFS) or carries path counts (BC)");
    if (!srcs_host && (src < 0 || src >= g->nv)) return fail(MG_ERR_RANGE, "source %d out of range [0,%d)", src, g->nv);
    if (Op::kMinPlusBound && g->min_weight < 0)
        return fail(MG_ERR_INVALID, "%s needs non-negative edge weights (min weight %d)", Op::kTag, g->min_weight);
    MG_TRY(ensure_ws<Op>(g));
    const int32_t *srcs_dev = nullptr;
    if (srcs_host) {
        if (nsrc <= 0 || nsrc > g->nv) return fail(MG_ERR_INVALID, "invalid source count %d", nsrc);
        MG_TRY(dev_alloc(g->fws->srcbuf, (size_t)nsrc * 4));
        MG_CUDA(cudaMemcpyAsync(g->fws->srcbuf.p, srcs_host, (size_t)nsrc * 4, cudaMemcpyHostToDevice, g->stream));
        srcs_dev = g->fws->srcbuf.as<int32_t>();
    }
    FrontierWS *w = g->fws;
    Args a = make_args(g);
    cudaStream_t s = g->stream;
    const size_t n = (size_t)g->nv;
    const int grid = launch_grid(g, THREADS, 8);
    if (n) k_label_init<Op><<<grid, THREADS, 0, s>>>(a.label, (int32_t)n);
    MG_CUDA(cudaMemsetAsync(a.bm, 0, 3 * (size_t)a.words * 4, s));
    MG_CUDA(cudaMemsetAsync(a.visited, 0, (size_t)a.words * 4, s));
    MG_CUDA(cudaMemsetAsync(w->bar.p, 0, BAR_BYTES, s));
    if (Op::kPathCounts) MG_CUDA(cudaMemsetAsync(a.sigma, 0, n * sizeof(mgops::PathCount), s));
    int max_iter = opt.max_iter > 0 ? opt.max_iter : (Op::kLevelSync ? g->nv + 2 : 4 * g->nv + 16);
    int alpha = opt.alpha > 0 ? opt.alpha : (Op::kLevelSync ? 15 : 4), beta = opt.beta > 0 ? opt.beta : 18;
    k_init<Op><<<1, 32, 0, s>>>(a, src, srcs_dev, nsrc, opt.direction, alpha, beta, max_iter);
    MG_CUDA(cudaGetLastError());
    const void *tag = &OpTag<Op>::id;
    const int coop = w->coop_grid[tag];
    Profiler &P = g->prof;
    const std::string t(Op::kTag);
    const int sp = P.slot((t + "_push").c_str());
    const int sl = P.slot((t + "_pull").c_str());
    const int sc = P.slot("frontier_compact");
    const int sf = Op::kMinPlusBound ? P.slot((t + "_fmin").c_str()) : -1;
    const int sd = P.slot("frontier_decide");
    BodyFn body = [&](cudaStream_t st, cudaGraphConditionalHandle h, int use_cond) -> mg_status {
        MG_CUDA(cudaMemsetAsync(a.cnt, 0, 4 * sizeof(LevelCnt), st));
        P.begin(sp);
        MG_TRY(launch_sparse_levels<Op>(a, coop, st));
        P.end();
        if (Op::kMinPlusBound) {
            P.begin(sf);
            k_fmin<<<grid, THREADS, 0, st>>>(a);
            P.end();
        }
        P.begin(sl);
        k_pull<Op><<<grid, THREADS, 0, st>>>(a);
        P.end();
        P.begin(sc);
        k_compact<<<grid, THREADS, 0, st>>>(a);
        P.end();
        P.begin(sd);
        k_decide<<<1, 32, 0, st>>>(a, h, use_cond);
        P.end();
        MG_CUDA(cudaGetLastError());
        return MG_OK;
    };
    MG_TRY(run_loop(opt.profile ? MG_EXEC_HOST : opt.exec, opt.profile != 0, s, w->lg[tag], key_of(a, tag, grid, coop),
                    body, &a.ctl->more, g->pinned_flag, max_iter + 2));
    // status readback
    FCtl hc;
    int32_t ovf = 0;
    MG_CUDA(cudaMemcpyAsync(&hc, a.ctl, sizeof(FCtl), cudaMemcpyDeviceToHost, s));
    if (Op::kPathCounts) MG_CUDA(cudaMemcpyAsync(&ovf, a.bc_ovf, 4, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    if (ovf && !g->bc_ext) {
        // a path count passed FP64's comfortable range: this graph's BC runs
        // use extended path counts from now on, starting with this one
        g->bc_ext = true;
        return frontier_run_impl<Op>(g, src, srcs_host, nsrc, opt, info);
    }
    if (info) {
        info->iterations = hc.iter;
        info->pull_iterations = hc.pull_iters;
        info->edges_scanned = hc.scanned;
    }
    if (hc.status == 3) return fail(MG_ERR_CUDA, "grid barrier of the persistent push kernel timed out");
    if (hc.status != 0) return fail(MG_ERR_ITER_LIMIT, "iteration cap %d reached", max_iter);
    return MG_OK;
}

// result slot `which` in caller ids (mapped on the device before the run ends)
inline mg_status publish(mg_graph *g, int which, const void *src, size_t elem)
{
    const void *p = nullptr;
    MG_TRY(to_caller(g, which, src, elem, 1, &p));
    g->res[which] = p;
    return MG_OK;
}

// One whole run of a label operator through the C ABI's conventions:
// source in caller ids, labels out in caller order (nv int32, when
// label_out is non-NULL), status and run info as mg_bfs / mg_sssp.
template <class Op>
mg_status frontier_operator_run(mg_graph *g, int32_t source, const mg_opts *o, int32_t *label_out,
                                mg_run_info *info)
{
    mg_opts opt;
    MG_TRY(begin_run(g, o, opt, info));
    if (source < 0 || source >= g->nv) return fail(MG_ERR_RANGE, "source %d out of range [0,%d)", source, g->nv);
    MG_TRY(frontier_run_impl<Op>(g, to_engine(g, source), nullptr, 0, opt, info));
    MG_TRY(publish(g, MG_RES_LEVEL, g->fws->label.p, 4));
    MG_TRY(end_run(g, opt, info));
    return copy_out(g, label_out, g->res[MG_RES_LEVEL], (size_t)g->nv * 4);
}

}  // namespace
