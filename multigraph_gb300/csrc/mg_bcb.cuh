// mg_bcb.cuh -- batched multi-source Brandes BC: 32 sources per traversal,
// one lane of a warp per source.  Structures, helpers and the phase bodies
// of the per-level kernels in mg_bcb.cu.
//
// The reference runs one BC source per program invocation (main.cu:52-86:
// MultiGraph_V_E_V forward, then MultiGraph_V_E_V_pull backward over the
// archived levels, process2.cu:263-325).  Here a group of up to 32 sources
// is traversed together, level-synchronously:
//
//   vis[v]   bit s set once v has been reached from source s
//   fm[v]    bit s set when v is on source s's current frontier
//   sig[v*32+s]  path count of v from source s (mgops::PathCount: FP64
//                mantissa m and a 2^512 scale k; plain FP64 until a count
//                reaches mgops::PC_PLAIN_MAX = 2^90, then the run repeats
//                in extended mode)
//   q[v*32+s]    (1 + delta_s[v]) / m   (backward; FP32 with plain counts,
//                FP64 with extended ones)
//   archive  (vertex, mask) entries, grouped by level: entry (v, M) at
//            level d means v is at distance d from exactly the sources in M
//
// Forward level d -> d+1 (three launches, four with heavy rows, looped by a
// CUDA-graph WHILE node):
//   k_bb_mark     sparse levels only: frontier entries scan their out-edges
//                 and collect the distinct candidate destinations (a vertex
//                 not yet reached by some source of the entry's mask)
//   k_bb_pull     each candidate row (sparse) or every row that some source
//                 has not reached (dense) scans its in-edges; a warp loads 32
//                 column ids and their frontier masks at once, keeps the
//                 lanes that hit (ballot), and lane s adds sig[u*32+s] for
//                 each hit of source s.  Rows above heavy_deg go in 2048-edge
//                 chunks whose partials land in hpart.
//   k_bb_heavy    (graphs with heavy rows) folds the chunk partials of heavy
//                 rows in chunk order
//   k_bb_compact  archives the new frontier (one atomic per warp), sums its
//                 out-degrees for the direction switch, clears the old
//                 frontier's masks; the last block to finish decides the
//                 next level (sparse/dense: Beamer, frontier out-edges x
//                 alpha against m) and the loop condition
// Backward level L (two launches, three with heavy rows): level l's masks
// sit in a dense array fm[l % 3]; every level-L entry sums q over
// successors whose level-(L+1) mask shares the source, and lane s finishes
//   delta_s[u] = sig_s[u] * sum,  q_s[u] = (1 + delta_s[u]) / sig_s[u]
// with the per-vertex score bc[u] += sum of delta_s[u] over the entry's
// sources (u excluded as its own source); k_bbb_next then clears level
// L+1's masks, scatters level L-1's into the third buffer and steps L.
//
// On low-degree graphs (average degree <= 8) both pull kernels first give
// each row / entry with at most 8 edges and at most 4 sources at this level
// to one thread, which forms the same per-source sums in the same edge
// order (a lattice level is mostly such rows, with one source each, so a
// warp per row left 31 lanes idle); the rest go to the warp path above.
//
// Every sum runs in a fixed order (the warp's edge order, then chunk order),
// so results do not depend on scheduling; path counts are integers in FP64
// and exact up to 2^53.  The column stream and the frontier-mask gathers are
// shared by the 32 sources of a group, which is where the batch gains over
// one traversal per source.

#pragma once

#include "mg_device.cuh"
#include "mg_ops.cuh"

#include <algorithm>
#include <type_traits>
#include <cstring>
#include <vector>

namespace mgbc {

constexpr int W = 32;                 // sources per group (one per lane)
constexpr int THREADS = 256;
constexpr int32_t MARK_HEAVY = 2048;  // frontier entries above this out-degree are marked by the whole grid
// rows with at most TDEG edges whose level touches at most TBITS sources are
// handled by one thread (low-degree graphs: a lattice row has four or five
// edges and usually one source per level); the rest by a warp, lane per source
constexpr int TDEG = 8;
constexpr int TBITS = 4;
constexpr int TP_AVG_DEG = 8;  // graphs up to this average degree use the thread path

// what one forward level counts (atomics): candidates of a sparse level,
// entries archived for the next level, their heavy entries and out-edges
struct LvlCnt {
    int32_t ncand;
    int32_t nnew;
    int32_t nfh_build;
    int32_t status;            // 2: archive overflow
    unsigned long long nfe;
};

struct BbCtl {
    int32_t more;
    int32_t d;          // forward level being expanded
    int32_t cur;        // fm buffer holding level d
    int32_t dense;      // this level pulls over every row
    int32_t nfh;        // heavy frontier entries at level d
    int32_t nlevels;    // levels 0..nlevels-1 archived (set when the forward sweep ends)
    int32_t L;          // backward level
    int32_t status;     // 1: level cap reached, 2: archive overflow, 3: grid barrier timeout
    int32_t dirmode;    // MG_DIR_*
    int32_t alpha;
    int32_t max_levels;
    uint32_t gmask;     // lanes holding a source
    int32_t dense_levels;
    int32_t done;       // blocks finished (last-block-done step of the level's final kernel)
    int32_t ovf;        // a plain-mode path count reached PC_PLAIN_MAX (ends the sweep)
    int32_t pad;
    unsigned long long nfe_cur;  // out-edges of level d
    LvlCnt k;                    // this level's counters (per-level kernels)
};

// the next level from level d's counters; off_d2 = archive offset of level d+2
__device__ __forceinline__ void bb_decide(BbCtl &n, const LvlCnt &k, int32_t ovf, int32_t off_d1, int32_t &off_d2,
                                          int32_t m)
{
    off_d2 = off_d1 + k.nnew;
    if (k.status) n.status = k.status;
    if (k.nnew == 0 || n.status || ovf) {  // (a path-count overflow ends the sweep for a rerun)
        n.more = 0;
        n.nlevels = n.d + 1;
        if (ovf) n.ovf = 1;
    } else if (n.d + 2 >= n.max_levels) {
        n.more = 0;
        n.status = 1;
        n.nlevels = n.d + 2;
    } else {
        n.d += 1;
        n.cur ^= 1;
        n.nfe_cur = k.nfe;
        n.nfh = k.nfh_build;
        if (n.dirmode == MG_DIR_PUSH) n.dense = 0;
        else if (n.dirmode == MG_DIR_PULL) n.dense = 1;
        else n.dense = n.nfe_cur * (unsigned long long)n.alpha > (unsigned long long)m;
        n.dense_levels += n.dense;
    }
}

struct BbArgs {
    int32_t n;
    int32_t m;
    const int32_t *row, *col;    // out-edges
    const int32_t *trow, *tcol;  // in-edges
    const int32_t *hchunk;       // (row, begin, end) of the heavy in-rows
    int32_t nhchunks;
    const int32_t *hrows, *hrow_chunk;
    int32_t nhrows;
    int32_t heavy_deg;
    uint32_t *vis;
    uint32_t *fm0, *fm1, *fm2;   // frontier masks: forward fm0/fm1, backward level l in fm[l % 3]
    uint32_t *cbm;               // candidate bitmap (sparse levels)
    int32_t *cand;
    int32_t *arch;
    uint32_t *amask;
    size_t cap;                  // archive capacity (32 n)
    int32_t *off;                // level offsets into the archive
    mgops::PathCount *sig;
    void *q;                     // float (plain counts) or double (extended) per (v, source)
    mgops::PathCount *hpart;     // per chunk x 32 lanes (backward reuses it as double)
    int32_t ext;                 // extended path counts
    uint32_t *hmask;
    double *bc;                  // score accumulator (all groups)
    int32_t *fheavy;
    const int32_t *src;          // the group's sources (engine ids), W entries
    BbCtl *ctl;
    // persistent sweeps (low-degree graphs): grid barrier words (zero before
    // each sweep), the barrier's error word, four rotating level counters
    unsigned *bar;
    int *bar_err;
    LvlCnt *pcnt;
};

__device__ __forceinline__ uint32_t *fm_of(const BbArgs &a, int i) { return i ? a.fm1 : a.fm0; }
__device__ __forceinline__ uint32_t *fmb_of(const BbArgs &a, int32_t l)
{
    const int32_t r = l % 3;
    return r == 0 ? a.fm0 : (r == 1 ? a.fm1 : a.fm2);
}

// the control block as other blocks left it (L2, not a stale L1 line)
__device__ __forceinline__ BbCtl load_ctl_l2(const BbCtl *cp)
{
    BbCtl c;
    const int *src = reinterpret_cast<const int *>(cp);
    int *dst = reinterpret_cast<int *>(&c);
#pragma unroll
    for (int k = 0; k < (int)(sizeof(BbCtl) / 4); k++) dst[k] = __ldcg(src + k);
    return c;
}

// true in one thread of the last block of the grid to get here (every
// block's earlier writes and atomics are visible to it)
__device__ __forceinline__ bool last_block_done(int32_t *done)
{
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(done, 1) == (int)gridDim.x - 1;
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        return true;
    }
    return false;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------
// items per warp: `cap`, or fewer (a power of two) when `count` items would
// leave warps idle
__device__ __forceinline__ int entries_per_warp(int32_t count, int nwarps, int cap)
{
    if (count >= nwarps * cap) return cap;
    const int want = max(1, count / nwarps);
    int v = 1;
    while (v * 2 <= want && v * 2 <= cap) v *= 2;
    return v;
}

__device__ __forceinline__ void mark_edge_block(const BbArgs &a, int32_t p, int32_t e, uint32_t f, int32_t *ncand)
{
    bool pred = false;
    int32_t v = 0;
    if (p < e) {
        v = __ldg(&a.col[p]);
        pred = (f & ~a.vis[v]) != 0 && mgd::bm_set(a.cbm, v);
    }
    int slot = mgd::warp_append(ncand, pred);
    if (pred) a.cand[slot] = v;
}

// sparse level d (archive entries [b0, b1)): collect the candidate rows
__device__ __forceinline__ void bb_mark_phase(const BbArgs &a, const BbCtl &c, int32_t b0, int32_t b1, int32_t *ncand)
{
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    // up to 32 entries per warp (fewer when the level would leave warps
    // idle), their out-edges spread over the lanes by a load-balanced search
    const int vpw = entries_per_warp(b1 - b0, nwarps, 32);
    for (int32_t base = b0 + gwarp * vpw; base < b1; base += nwarps * vpw) {
        int32_t start = 0, deg = 0;
        uint32_t f = 0;
        if (lane < vpw && base + lane < b1) {
            const int32_t u = a.arch[base + lane];
            f = a.amask[base + lane];
            start = __ldg(&a.row[u]);
            deg = __ldg(&a.row[u + 1]) - start;
            if (deg > MARK_HEAVY) deg = 0;  // the grid-wide loop below
        }
        const int incl = mgd::warp_scan_incl(deg);
        const int excl = incl - deg;
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        for (int k0 = 0; k0 < total; k0 += 32) {
            const int k = k0 + lane;
            const int kk = k < total ? k : total - 1;
            const int own = mgd::owner_lane(excl, kk);
            const int32_t p = __shfl_sync(0xffffffffu, start, own) + (kk - __shfl_sync(0xffffffffu, excl, own));
            const uint32_t fo = __shfl_sync(0xffffffffu, f, own);
            mark_edge_block(a, k < total ? p : 0, k < total ? p + 1 : 0, fo, ncand);
        }
    }
    // heavy frontier entries: every warp of the grid takes 32-edge slices
    const uint32_t *fcur = fm_of(a, c.cur);
    for (int32_t h = 0; h < c.nfh; h++) {
        const int32_t u = a.fheavy[h];
        const uint32_t f = fcur[u];
        const int32_t b = __ldg(&a.row[u]), e = __ldg(&a.row[u + 1]);
        for (int32_t base = b + gwarp * 32; base < e; base += nwarps * 32) mark_edge_block(a, base + lane, e, f, ncand);
    }
}

// One row's in-edges [b, e) against the frontier masks: lane s returns the
// sum of sig over in-neighbours on source s's frontier; *hit gets the union
// of the masks that hit (restricted to `want`).
template <bool EXT>
__device__ __forceinline__ mgops::PathCount pull_span(const BbArgs &a, const uint32_t *fcur, int32_t b, int32_t e,
                                                      uint32_t want, uint32_t &hit)
{
    const int lane = mgd::lane();
    mgops::PathCount acc = mgops::pc_zero();  // extended counts
    double accp = 0.0;                        // plain counts
    uint32_t newm = 0;
    for (int32_t base = b; base < e; base += 32) {
        const int32_t p = base + lane;
        int32_t u = 0;
        uint32_t f = 0;
        if (p < e) {
            u = __ldcs(&a.tcol[p]);
            f = fcur[u] & want;
        }
        unsigned hits = __ballot_sync(0xffffffffu, f != 0);
        while (hits) {
            const int j = __ffs(hits) - 1;
            hits &= hits - 1;
            const int32_t uj = __shfl_sync(0xffffffffu, u, j);
            const uint32_t fj = __shfl_sync(0xffffffffu, f, j);
            newm |= fj;
            if ((fj >> lane) & 1u) {
                if (EXT) acc = mgops::pc_add(acc, a.sig[(size_t)uj * W + lane], true);
                else accp += a.sig[(size_t)uj * W + lane].m;
            }
        }
    }
    hit = newm;
    if (!EXT) acc.m = accp;
    return acc;
}

__device__ __forceinline__ void settle_row(const BbArgs &a, uint32_t *fnext, int32_t v, uint32_t newm,
                                           mgops::PathCount acc)
{
    const int lane = mgd::lane();
    if ((newm >> lane) & 1u) {
        a.sig[(size_t)v * W + lane] = acc;
        if (!a.ext && acc.m >= mgops::PC_PLAIN_MAX) a.ctl->ovf = 1;
    }
    if (lane == 0) {
        a.vis[v] |= newm;
        fnext[v] = newm;
    }
}

// One thread, one row v with at most TDEG in-edges: per source s in the
// sources that reach v at this level (at most TBITS of them, else false is
// returned and the row goes to the warp path), the sum of sig over the
// in-neighbours on s's frontier, in edge order as pull_span forms it.
__device__ __forceinline__ bool pull_row_thread(const BbArgs &a, const uint32_t *fcur, uint32_t *fnext, int32_t v,
                                                uint32_t want)
{
    const int32_t b = __ldg(&a.trow[v]), e = __ldg(&a.trow[v + 1]);
    if (e - b > TDEG) return false;
    uint32_t newm = 0;
    for (int32_t p = b; p < e; p++) newm |= fcur[__ldg(&a.tcol[p])];
    newm &= want;
    if (__popc(newm) > TBITS) return false;
    if (newm == 0) return true;
    uint32_t mm = newm;
    while (mm) {  // the row's edges again per source (L1 hits)
        const int s = __ffs(mm) - 1;
        mm &= mm - 1;
        mgops::PathCount acc = mgops::pc_zero();
        for (int32_t p = b; p < e; p++) {
            const int32_t u = __ldg(&a.tcol[p]);
            if ((fcur[u] >> s) & 1u) acc = mgops::pc_add(acc, a.sig[(size_t)u * W + s], a.ext != 0);
        }
        a.sig[(size_t)v * W + s] = acc;
        if (!a.ext && acc.m >= mgops::PC_PLAIN_MAX) a.ctl->ovf = 1;
    }
    a.vis[v] |= newm;
    fnext[v] = newm;
    return true;
}

// level d -> d+1 over nrows rows (every row when dense, else the candidates)
template <bool TP, bool EXT>
__device__ __forceinline__ void bb_pull_phase(const BbArgs &a, const BbCtl &c, int32_t nrows)
{
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t *fcur = fm_of(a, c.cur);
    uint32_t *fnext = fm_of(a, c.cur ^ 1);
    if constexpr (TP) {
        // up to 32 rows per warp, one per lane; rows the thread path
        // declines are then pulled by the whole warp, one at a time
        const int vpw = entries_per_warp(nrows, nwarps, 32);
        for (int32_t base = gwarp * vpw; base < nrows; base += nwarps * vpw) {
            const int32_t i = base + lane;
            int32_t v = 0;
            uint32_t want = 0;
            bool deferred = false;
            if (lane < vpw && i < nrows) {
                v = c.dense ? i : a.cand[i];
                want = ~a.vis[v] & c.gmask;
                if (want) deferred = !pull_row_thread(a, fcur, fnext, v, want);
            }
            unsigned dm = __ballot_sync(0xffffffffu, deferred);
            while (dm) {
                const int j = __ffs(dm) - 1;
                dm &= dm - 1;
                const int32_t vj = __shfl_sync(0xffffffffu, v, j);
                const uint32_t wj = __shfl_sync(0xffffffffu, want, j);
                const int32_t b = __ldg(&a.trow[vj]), e = __ldg(&a.trow[vj + 1]);
                if (e - b > a.heavy_deg) continue;  // chunk path below
                uint32_t newm;
                const mgops::PathCount acc = pull_span<EXT>(a, fcur, b, e, wj, newm);
                if (newm) settle_row(a, fnext, vj, newm, acc);
            }
        }
    } else {
        for (int32_t i = gwarp; i < nrows; i += nwarps) {  // a warp per row
            const int32_t v = c.dense ? i : a.cand[i];
            const uint32_t want = ~a.vis[v] & c.gmask;
            if (want == 0) continue;
            const int32_t b = __ldg(&a.trow[v]), e = __ldg(&a.trow[v + 1]);
            if (e - b > a.heavy_deg) continue;  // chunk path below
            uint32_t newm;
            const mgops::PathCount acc = pull_span<EXT>(a, fcur, b, e, want, newm);
            if (newm) settle_row(a, fnext, v, newm, acc);
        }
    }
    for (int32_t ch = gwarp; ch < a.nhchunks; ch += nwarps) {
        const int32_t v = __ldg(&a.hchunk[3 * ch]), b = __ldg(&a.hchunk[3 * ch + 1]), e = __ldg(&a.hchunk[3 * ch + 2]);
        uint32_t want = ~a.vis[v] & c.gmask;
        if (!c.dense && !mgd::bm_test(a.cbm, v)) want = 0;
        uint32_t newm = 0;
        mgops::PathCount acc = mgops::pc_zero();
        if (want) acc = pull_span<EXT>(a, fcur, b, e, want, newm);
        if (newm) a.hpart[(size_t)ch * W + lane] = acc;
        if (lane == 0) a.hmask[ch] = newm;
    }
}

__device__ __forceinline__ void bb_heavy_phase(const BbArgs &a, const BbCtl &c)
{
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    uint32_t *fnext = fm_of(a, c.cur ^ 1);
    for (int32_t i = gwarp; i < a.nhrows; i += nwarps) {
        const int32_t v = __ldg(&a.hrows[i]), k0 = __ldg(&a.hrow_chunk[i]), k1 = __ldg(&a.hrow_chunk[i + 1]);
        uint32_t newm = 0;
        mgops::PathCount acc = mgops::pc_zero();
        for (int32_t k = k0; k < k1; k++) {
            const uint32_t hm = a.hmask[k];
            newm |= hm;
            if ((hm >> lane) & 1u) acc = mgops::pc_add(acc, a.hpart[(size_t)k * W + lane], a.ext != 0);
        }
        if (newm) settle_row(a, fnext, v, newm, acc);
    }
}

// Archives level d+1 (entries from off_d1 on), clears level d's masks
// (entries [off_d, off_d1)), counts into *k
__device__ __forceinline__ void bb_compact_phase(const BbArgs &a, const BbCtl &c, int32_t off_d, int32_t off_d1,
                                                 int32_t nrows, LvlCnt *k)
{
    const int lane = mgd::lane();
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gwarp = gtid >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    uint32_t *fcur = fm_of(a, c.cur);
    const uint32_t *fnext = fm_of(a, c.cur ^ 1);
    // the old frontier's masks (every reader of level d has finished)
    for (int32_t i = off_d + gtid; i < off_d1; i += gridDim.x * blockDim.x) fcur[a.arch[i]] = 0;
    const int32_t base_out = off_d1;
    for (int32_t base = gwarp * 32; base < nrows; base += nwarps * 32) {
        const int32_t i = base + lane;
        int32_t v = -1;
        uint32_t msk = 0;
        if (i < nrows) {
            v = c.dense ? i : a.cand[i];
            if (!c.dense) atomicAnd(&a.cbm[v >> 5], ~(1u << (v & 31)));
            msk = fnext[v];
        }
        const bool pred = msk != 0;
        int32_t deg = 0;
        if (pred) deg = __ldg(&a.row[v + 1]) - __ldg(&a.row[v]);
        const int slot = mgd::warp_append(&k->nnew, pred);
        if (pred) {
            const size_t at = (size_t)base_out + (size_t)slot;
            if (at < a.cap) {
                a.arch[at] = v;
                a.amask[at] = msk;
            } else {
                k->status = 2;
            }
            if (deg > MARK_HEAVY) a.fheavy[atomicAdd(&k->nfh_build, 1)] = v;
        }
        const unsigned long long s = warp_sum_u64((unsigned long long)deg);
        if (lane == 0 && s) atomicAdd(&k->nfe, s);
    }
}

// ---------------------------------------------------------------------------
// backward
// ---------------------------------------------------------------------------
// Backward start at the deepest level L: the masks of levels L and L-1
// into their buffers (all three are zero after the forward sweep).
__device__ __forceinline__ void bbb_start_phase(const BbArgs &a, int32_t L)
{
    const int32_t stride = gridDim.x * blockDim.x;
    for (int32_t l = L - 1; l <= L; l++) {
        uint32_t *buf = fmb_of(a, l);
        for (int32_t i = a.off[l] + blockIdx.x * blockDim.x + threadIdx.x; i < a.off[l + 1]; i += stride)
            buf[a.arch[i]] = a.amask[i];
    }
}

template <bool EXT>
using QT = typename std::conditional<EXT, double, float>::type;

template <bool EXT>
__device__ __forceinline__ QT<EXT> *q_of(const BbArgs &a)
{
    return reinterpret_cast<QT<EXT> *>(a.q);
}

// successor v's term for lane s of an entry whose count has scale ku
template <bool EXT>
__device__ __forceinline__ QT<EXT> back_term(const BbArgs &a, int32_t v, int s, int32_t ku)
{
    QT<EXT> t = q_of<EXT>(a)[(size_t)v * W + s];
    if (EXT) t *= (QT<EXT>)mgops::pc_scale(ku - a.sig[(size_t)v * W + s].k);
    return t;
}

// successors' q summed for the sources in `want`: out-edges [b, e); ku is
// this lane's scale of the entry's path count
template <bool EXT>
__device__ __forceinline__ QT<EXT> back_span(const BbArgs &a, const uint32_t *nxt, const int32_t *col, int32_t b,
                                             int32_t e, uint32_t want, int32_t ku)
{
    const int lane = mgd::lane();
    QT<EXT> acc = 0;
    for (int32_t base = b; base < e; base += 32) {
        const int32_t p = base + lane;
        int32_t v = 0;
        uint32_t f = 0;
        if (p < e) {
            v = __ldcs(&col[p]);
            f = nxt[v] & want;
        }
        unsigned hits = __ballot_sync(0xffffffffu, f != 0);
        while (hits) {
            const int j = __ffs(hits) - 1;
            hits &= hits - 1;
            const int32_t vj = __shfl_sync(0xffffffffu, v, j);
            const uint32_t fj = __shfl_sync(0xffffffffu, f, j);
            if ((fj >> lane) & 1u) acc += back_term<EXT>(a, vj, lane, ku);
        }
    }
    return acc;
}

// lane's scale of u's path count (0 in plain mode)
template <bool EXT>
__device__ __forceinline__ int32_t lane_scale(const BbArgs &a, int32_t u, uint32_t msk)
{
    const int lane = mgd::lane();
    return (EXT && ((msk >> lane) & 1u)) ? a.sig[(size_t)u * W + lane].k : 0;
}

template <bool EXT>
__device__ __forceinline__ void back_finish(const BbArgs &a, int32_t u, uint32_t msk, QT<EXT> s)
{
    const int lane = mgd::lane();
    double contrib = 0.0;
    if ((msk >> lane) & 1u) {
        const double sg = a.sig[(size_t)u * W + lane].m;
        const float dv = (float)(sg * (double)s);
        q_of<EXT>(a)[(size_t)u * W + lane] = (QT<EXT>)((1.0 + (double)dv) / sg);
        if (__ldg(&a.src[lane]) != u) contrib = (double)dv;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
    if (lane == 0) a.bc[u] += contrib;
}

// One thread, one level-L entry (u, msk) with at most TDEG out-edges and
// at most TBITS sources: back_span and back_finish for each source of the
// entry in turn (the same sums in the same edge order; the entry's score
// contributions are added in source order).
template <bool EXT>
__device__ __forceinline__ bool back_entry_thread(const BbArgs &a, const uint32_t *nxt, int32_t u, uint32_t msk)
{
    if (__popc(msk) > TBITS) return false;
    const int32_t b = __ldg(&a.row[u]), e = __ldg(&a.row[u + 1]);
    if (e - b > TDEG) return false;
    double contrib = 0.0;
    uint32_t mm = msk;
    while (mm) {
        const int s = __ffs(mm) - 1;
        mm &= mm - 1;
        const mgops::PathCount su = a.sig[(size_t)u * W + s];
        QT<EXT> acc = 0;
        for (int32_t p = b; p < e; p++) {
            const int32_t v = __ldg(&a.col[p]);
            if ((nxt[v] >> s) & 1u) acc += back_term<EXT>(a, v, s, su.k);
        }
        const float dv = (float)(su.m * (double)acc);
        q_of<EXT>(a)[(size_t)u * W + s] = (QT<EXT>)((1.0 + (double)dv) / su.m);
        if (__ldg(&a.src[s]) != u) contrib += (double)dv;
    }
    a.bc[u] += contrib;
    return true;
}

// backward level L: every level-L entry from its level-(L+1) successors
template <bool TP, bool EXT>
__device__ __forceinline__ void bbb_pull_phase(const BbArgs &a, int32_t L)
{
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t *cur = fmb_of(a, L);
    const uint32_t *nxt = fmb_of(a, L + 1);
    if constexpr (TP) {
        const int32_t lo = a.off[L], hi = a.off[L + 1];
        // up to 32 entries per warp, one per lane; entries the thread path
        // declines are then handled by the whole warp (lane per source)
        const int vpw = entries_per_warp(hi - lo, nwarps, 32);
        for (int32_t base = lo + gwarp * vpw; base < hi; base += nwarps * vpw) {
            const int32_t i = base + lane;
            int32_t u = 0;
            uint32_t msk = 0;
            bool deferred = false;
            if (lane < vpw && i < hi) {
                u = a.arch[i];
                msk = a.amask[i];
                deferred = !back_entry_thread<EXT>(a, nxt, u, msk);
            }
            unsigned dm = __ballot_sync(0xffffffffu, deferred);
            while (dm) {
                const int j = __ffs(dm) - 1;
                dm &= dm - 1;
                const int32_t uj = __shfl_sync(0xffffffffu, u, j);
                const uint32_t mj = __shfl_sync(0xffffffffu, msk, j);
                const int32_t b = __ldg(&a.row[uj]), e = __ldg(&a.row[uj + 1]);
                if (e - b > a.heavy_deg) continue;  // chunk path below
                const QT<EXT> sj = back_span<EXT>(a, nxt, a.col, b, e, mj, lane_scale<EXT>(a, uj, mj));
                back_finish<EXT>(a, uj, mj, sj);
            }
        }
    } else {
        for (int32_t i = a.off[L] + gwarp; i < a.off[L + 1]; i += nwarps) {  // a warp per entry
            const int32_t u = a.arch[i];
            const uint32_t msk = a.amask[i];
            const int32_t b = __ldg(&a.row[u]), e = __ldg(&a.row[u + 1]);
            if (e - b > a.heavy_deg) continue;  // chunk path below
            const QT<EXT> s = back_span<EXT>(a, nxt, a.col, b, e, msk, lane_scale<EXT>(a, u, msk));
            back_finish<EXT>(a, u, msk, s);
        }
    }
    // heavy rows: the in-row chunks double as out-row chunks (symmetric graphs)
    QT<EXT> *hp = reinterpret_cast<QT<EXT> *>(a.hpart);
    for (int32_t ch = gwarp; ch < a.nhchunks; ch += nwarps) {
        const int32_t u = __ldg(&a.hchunk[3 * ch]);
        const uint32_t msk = cur[u];
        if (msk == 0) continue;
        hp[(size_t)ch * W + lane] = back_span<EXT>(a, nxt, a.tcol, __ldg(&a.hchunk[3 * ch + 1]), __ldg(&a.hchunk[3 * ch + 2]), msk,
                                                   lane_scale<EXT>(a, u, msk));
    }
}

// heavy rows: chunk partials folded in chunk order (graphs with heavy rows)
template <bool EXT>
__device__ __forceinline__ void bbb_heavy_phase(const BbArgs &a, int32_t L)
{
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t *cur = fmb_of(a, L);
    const QT<EXT> *hp = reinterpret_cast<const QT<EXT> *>(a.hpart);
    for (int32_t i = gwarp; i < a.nhrows; i += nwarps) {
        const int32_t u = __ldg(&a.hrows[i]);
        const uint32_t msk = cur[u];
        if (msk == 0) continue;
        QT<EXT> s = 0;
        for (int32_t k = __ldg(&a.hrow_chunk[i]); k < __ldg(&a.hrow_chunk[i + 1]); k++) s += hp[(size_t)k * W + lane];
        back_finish<EXT>(a, u, msk, s);
    }
}

// End of backward level L: level L+1's masks are no longer read (cleared),
// level L-1's go into their buffer ((L-1) % 3, cleared at the end of level
// L+1)
__device__ __forceinline__ void bbb_next_phase(const BbArgs &a, int32_t L)
{
    const int32_t stride = gridDim.x * blockDim.x;
    const int32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t *nxt = fmb_of(a, L + 1);
    for (int32_t i = a.off[L + 1] + gtid; i < a.off[L + 2]; i += stride) nxt[a.arch[i]] = 0;
    if (L >= 2) {
        uint32_t *prv = fmb_of(a, L - 1);
        for (int32_t i = a.off[L - 1] + gtid; i < a.off[L]; i += stride) prv[a.arch[i]] = a.amask[i];
    }
}

}  // namespace mgbc

