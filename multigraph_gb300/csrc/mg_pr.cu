// mg_pr.cu -- PageRank engines: the reference's PR_T / PR_D recurrences,
// normalised topology- and data-driven PageRank, batched personalised
// PageRank, weighted PageRank and its adjoint (edge-weight gradient).
//
// Replaces MultiGraph_V_E_V_NOTIDEM (processi.cu:682-894) with _phase1 /
// _phase11 / _phase2.  The reference scatters pr/deg with FP32 atomicAdd into
// an intermediate buffer and gathers it in shared memory (order-dependent
// sums, ~12.5 B/edge).  Here every sweep is a pull over in-edges, in one of
// two layouts (mg_opts.pr_layout; MG_PR_LAYOUT_AUTO picks):
//   segmented (the default where the segments hold every id): k_hub_sweep
//               (mg_hub.cu) sums every in-edge from a source segment staged
//               in shared memory into per-(row, segment) piece sums, then
//   k_pr_seg    sums each row's pieces in order, applies the update and
//               (last block) closes the sweep;
//   gather (contribution gathers through L2):
//   k_pr_light  degree bins (mg_bins.cuh): a warp per row of tbin+1..heavy
//               in-edges (lanes read one 128 B line of column ids per step,
//               a fixed shuffle tree sums them), a thread per row of <= tbin
//               in-edges; then rows above heavy in-edges in chunks, one CTA
//               each, partial sums written per chunk (tbin / heavy / chunk
//               default to 32 / 512 / 2048, mg_autotune re-picks them);
//   k_pr_apply  heavy rows summed chunk by chunk in order (thread per row),
//               then the last block to finish sums every block's residual
//               partials in slot order: convergence test, loop condition.
// Sums are therefore deterministic (fixed order) run to run.
// Algorithmic bytes per sweep: 4m (column ids) + 4(n+1) (offsets) + 12n
// (old value read, new value and contribution written); in the gather
// layout the contribution gathers (4n bytes) are served by L2.

#include "mg_device.cuh"
#include "mg_ops.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace {

constexpr int THREADS = 256;


struct PCtl {
    int32_t more;
    int32_t iter;
    int32_t cur;
    int32_t status;
    int32_t max_iter;
    int32_t any;          // a vertex changed beyond tolerance / is active
    int32_t done;         // blocks of k_pr_apply that have finished this sweep
    int32_t pad2;
    double resid;         // L1 change of the last sweep
    double dangling;      // sum of x over zero out-degree vertices (current iterate)
    double lam_mean;      // adjoint: mean of lambda (dangling rows)
    float damping, tol;
    int32_t n;
    float base;           // (1-d)/n + d*dangling/n of the current sweep (set once per sweep)
    float tol_row;        // tol / n: per-vertex activity threshold of the data-driven form
    float lam_meanf;      // lam_mean as float
    // data-driven form, frontier sweeps: once the active vertices' in-edges
    // fall below m / SPARSE_ALPHA the sweeps run over a queue of them and
    // update x[cur] / c[cur] in place (frozen vertices keep their values)
    int32_t sparse;       // 1: queue sweeps
    int32_t need_compact; // the queue is to be built from the active flags
    int32_t qc;           // current queue (0 / 1)
    int32_t dense_iters;  // sweeps that ran over every row
    int32_t qn[2];        // queue sizes (qn[qc ^ 1]: appends of this sweep)
    double dang_frozen;   // dangling mass of frozen vertices
    long long act_edges;  // in-edges of the vertices still active
};

// per-sweep constants derived once (FP64 math stays out of the per-row path)
__device__ __forceinline__ void pctl_derive(PCtl *c)
{
    c->base = (float)((1.0 - (double)c->damping) / c->n + (double)c->damping * c->dangling / c->n);
    c->tol_row = c->tol / (float)c->n;
    c->lam_meanf = (float)c->lam_mean;
}

struct PArgs {
    int32_t n;
    const int32_t *prow;     // rows scanned (in-edges for PR, out-edges for the adjoint)
    const int32_t *pcol;
    const float *pw;         // per-entry weights of the scanned rows (weighted / adjoint), or null
    const int32_t *outrow;   // push-side offsets (out-degrees)
    float *S;                // weighted: out-weight sums
    const int32_t *wrows, *trows;  // degree bins
    int32_t nwrows, ntrows, nwlong;
    const int32_t *hchunk;
    int32_t nhchunks;
    const int32_t *hrows;
    const int32_t *hrow_chunk;
    int32_t nhrows;
    int32_t heavy_deg;
    // segmented pull (unweighted forms on graphs where it covers enough
    // edges): prow / pcol hold the tail part, P the sweep's per-(row,
    // segment) sums, row v's at P[pair_off[v] .. pair_off[v+1]); heavy
    // chunks keep their full-row numbering (prow_full, chunk)
    const float *P;
    const int32_t *pair_off;
    const int32_t *prow_full;
    int32_t chunk;
    int32_t seg_only;        // every in-edge sits in a segment: rows finish in k_pr_seg
    const int32_t *fin;      // k_pr_seg's warp rows (more than fin_warp pieces)
    int32_t nfw, fin_warp;
    float *x[2];             // iterate (ping-pong)
    float *c[2];             // gathered quantity: contribution x/deg (PR) or lambda (adjoint)
    const float *gvec;       // adjoint: g
    int32_t *active;         // data-driven masks
    float *hpart;            // heavy chunk partial sums
    double *bpart;           // per-block partials: [NPART*slots] (resid, dangling, any, active edges, frozen dangling)
    int32_t nblocks;
    int32_t qblocks;          // grid of the queue sweeps (k_prd_gather / k_prd_apply)
    PCtl *ctl;
    // data-driven frontier sweeps: the full pull rows (the hub split keeps
    // only the tail in prow / pcol), two queues, the queue sweep's new values
    const int32_t *frow, *fcol;
    int32_t *queue[2];
    float *qval;
    int64_t m;
};

constexpr int NPART = 5;       // partials per block slot
constexpr int SPARSE_ALPHA = 16;  // queue sweeps once active in-edges < m / SPARSE_ALPHA

// ---------------------------------------------------------------------------
// PageRank operators: the engine (k_pr_light / k_pr_apply / k_prd_*) is a
// template over one of these.  Hooks:
//   apply(a, c, v, s, any, dang)  row v's update from its gathered sum s:
//                                 writes the next iterate and contribution,
//                                 returns |change|, sets any when the row
//                                 counts as changed / active, dang = the new
//                                 value when the row is dangling
//   init(a, v, x0)                start value and contribution of row v
//   more(any, R, tol)             continue after a sweep with any / L1 change R
// Flags: kDataDriven (inactive rows frozen and skipped; queue sweeps),
// kWeights (gathers scaled by the staged per-edge weight; the others take
// the shared-memory hub split), kAdjoint (the iterate lives in c; its mean
// replaces the dangling mass); kSlot: the workspace's captured-loop slot.
// ---------------------------------------------------------------------------
// PR_T: the reference recurrence (processi.cu:631-638 / validate.cu:59-70)
struct PrTopologyRef {
    static constexpr bool kDataDriven = false, kWeights = false, kAdjoint = false;
    static constexpr int kSlot = 0;
    __device__ static __forceinline__ float apply(const PArgs &a, const PCtl &c, int32_t v, float s, int &any, float &)
    {
        const int cur = c.cur, nxt = cur ^ 1;
        const float xo = a.x[cur][v];
        const int32_t od = a.outrow[v + 1] - a.outrow[v];
        const float f1 = mgops::PrRef::apply(s);
        float xn = xo;
        if (fabsf(f1 - xo) > mgops::PrRef::TOL) { xn = f1; any = 1; }
        a.x[nxt][v] = xn;
        a.c[nxt][v] = mgops::PrRef::get_partial_result(xn, od);
        return fabsf(xn - xo);
    }
    __device__ static __forceinline__ int more(int any, double, float) { return any; }
};

// PR_D: the reference recurrence with the sticky per-vertex mask
// (processi.cu:640-655 / validate.cu:71-84): values always move, the mask
// only decides termination
struct PrDataRef {
    static constexpr bool kDataDriven = false, kWeights = false, kAdjoint = false;
    static constexpr int kSlot = 1;
    __device__ static __forceinline__ float apply(const PArgs &a, const PCtl &c, int32_t v, float s, int &any, float &)
    {
        const int cur = c.cur, nxt = cur ^ 1;
        const float xo = a.x[cur][v];
        const int32_t od = a.outrow[v + 1] - a.outrow[v];
        const float f1 = mgops::PrRef::apply(s);
        if (a.active[v] == 1 && fabsf(f1 - xo) > mgops::PrRef::TOL * xo) any = 1;
        else a.active[v] = 0;
        a.x[nxt][v] = f1;
        a.c[nxt][v] = mgops::PrRef::get_partial_result(f1, od);
        return fabsf(f1 - xo);
    }
    __device__ static __forceinline__ int more(int any, double, float) { return any; }
};

// normalised topology-driven: (1-d)/n + d (sum + dangling/n) for every row
struct PrTopology {
    static constexpr bool kDataDriven = false, kWeights = false, kAdjoint = false;
    static constexpr int kSlot = 2;
    __device__ static __forceinline__ float apply(const PArgs &a, const PCtl &c, int32_t v, float s, int &,
                                                  float &dang)
    {
        const int cur = c.cur, nxt = cur ^ 1;
        const float xo = a.x[cur][v];
        const int32_t od = a.outrow[v + 1] - a.outrow[v];
        const float xn = c.base + c.damping * s;
        a.x[nxt][v] = xn;
        a.c[nxt][v] = od > 0 ? xn / (float)od : 0.0f;
        if (od == 0) dang = xn;
        return fabsf(xn - xo);
    }
    __device__ static __forceinline__ int more(int, double R, float tol) { return R > (double)tol; }
};

// normalised data-driven: a row freezes (for good) once its change is at
// most tol / n; frozen rows keep their value and are skipped
struct PrData {
    static constexpr bool kDataDriven = true, kWeights = false, kAdjoint = false;
    static constexpr int kSlot = 3;
    __device__ static __forceinline__ float apply(const PArgs &a, const PCtl &c, int32_t v, float s, int &any,
                                                  float &dang)
    {
        const int cur = c.cur, nxt = cur ^ 1;
        const float xo = a.x[cur][v];
        const int32_t od = a.outrow[v + 1] - a.outrow[v];
        float xn = xo;   // frozen
        if (a.active[v] != 0) {
            xn = c.base + c.damping * s;
            if (fabsf(xn - xo) <= c.tol_row) a.active[v] = 0;
            else any = 1;
        }
        a.x[nxt][v] = xn;
        a.c[nxt][v] = od > 0 ? xn / (float)od : 0.0f;
        if (od == 0) dang = xn;
        return fabsf(xn - xo);
    }
    __device__ static __forceinline__ int more(int any, double R, float tol) { return any && R > (double)tol; }
};

// weighted: P_uv = w_uv / S_u
struct PrWeighted {
    static constexpr bool kDataDriven = false, kWeights = true, kAdjoint = false;
    static constexpr int kSlot = 4;
    __device__ static __forceinline__ float apply(const PArgs &a, const PCtl &c, int32_t v, float s, int &,
                                                  float &dang)
    {
        const int cur = c.cur, nxt = cur ^ 1;
        const float xo = a.x[cur][v];
        const float xn = c.base + c.damping * s;
        a.x[nxt][v] = xn;
        const float Su = a.S[v];
        a.c[nxt][v] = Su > 0.0f ? xn / Su : 0.0f;
        if (!(Su > 0.0f)) dang = xn;
        return fabsf(xn - xo);
    }
    __device__ static __forceinline__ int more(int, double R, float tol) { return R > (double)tol; }
};

// adjoint: lambda_new = g + d * (t + [S_u == 0] * mean(lambda))
struct PrAdjoint {
    static constexpr bool kDataDriven = false, kWeights = true, kAdjoint = true;
    static constexpr int kSlot = 5;
    __device__ static __forceinline__ float apply(const PArgs &a, const PCtl &c, int32_t v, float s, int &,
                                                  float &dang)
    {
        const int cur = c.cur, nxt = cur ^ 1;
        const float Su = a.S[v];
        const float t = Su > 0.0f ? s / Su : c.lam_meanf;
        const float xn = a.gvec[v] + c.damping * t;
        const float xo = a.c[cur][v];
        a.c[nxt][v] = xn;
        dang = xn;  // sum of lambda for the mean
        return fabsf(xn - xo);
    }
    __device__ static __forceinline__ int more(int, double R, float tol) { return R > (double)tol; }
};

// start values: x = x0, contributions (lambda = g for the adjoint), masks
template <class Op>
__device__ __forceinline__ void pr_init_row(const PArgs &a, int32_t v, float x0)
{
    if constexpr (Op::kAdjoint) {
        a.c[0][v] = a.gvec[v];
        return;
    }
    a.x[0][v] = x0;
    if constexpr (Op::kWeights) {
        const float Su = a.S[v];
        a.c[0][v] = Su > 0.0f ? x0 / Su : 0.0f;
    } else {
        const int32_t od = a.outrow[v + 1] - a.outrow[v];
        a.c[0][v] = od > 0 ? x0 / (float)od : 0.0f;
    }
    if (a.active) a.active[v] = 1;
}

// gathered value for edge e from source u
template <class Op>
__device__ __forceinline__ float pr_gather(const PArgs &a, int cur, int32_t e, int32_t u)
{
    float cv = a.c[cur][u];
    if (Op::kWeights) cv *= a.pw[e];
    return cv;
}

template <class Op>
__device__ __forceinline__ bool pr_row_skipped(const PArgs &a, int32_t v)
{
    return Op::kDataDriven && a.active[v] == 0;
}

// Per-block partials to bpart[slot]: the L1 change and the dangling mass
// summed in FP32 within each warp (FP64 arithmetic is slow on this part; a
// warp adds 32 per-thread FP32 sums), then in FP64 across warps; the
// data-driven form's active in-edge count and frozen dangling mass stay FP64
// throughout.
template <bool kDD>
__device__ __forceinline__ void block_partials(const PArgs &a, int slot, float r, float dg, int any,
                                               double act = 0.0, double dfz = 0.0)
{
    __shared__ double sp[NPART - 1][THREADS / 32];
    __shared__ int sa[THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_xor_sync(0xffffffffu, r, o);
        dg += __shfl_xor_sync(0xffffffffu, dg, o);
        any |= __shfl_xor_sync(0xffffffffu, any, o);
        if (kDD) {
            act += __shfl_xor_sync(0xffffffffu, act, o);
            dfz += __shfl_xor_sync(0xffffffffu, dfz, o);
        }
    }
    if ((threadIdx.x & 31) == 0) {
        sp[0][threadIdx.x >> 5] = (double)r;
        sp[1][threadIdx.x >> 5] = (double)dg;
        sp[2][threadIdx.x >> 5] = kDD ? act : 0.0;
        sp[3][threadIdx.x >> 5] = kDD ? dfz : 0.0;
        sa[threadIdx.x >> 5] = any;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double T[NPART - 1] = {0, 0, 0, 0};
        int A = 0;
        for (int w = 0; w < THREADS / 32; w++) {
#pragma unroll
            for (int k = 0; k < NPART - 1; k++) T[k] += sp[k][w];
            A |= sa[w];
        }
        double *o = a.bpart + (size_t)NPART * slot;
        o[0] = T[0];
        o[1] = T[1];
        o[2] = (double)A;
        o[3] = T[2];
        o[4] = T[3];
    }
}

// the row's segment partial sums (segments ascending; 0 without the split)
__device__ __forceinline__ float seg_sum(const PArgs &a, int32_t v)
{
    float s = 0.0f;
    if (a.P)
        for (int32_t p = __ldg(&a.pair_off[v]), e = __ldg(&a.pair_off[v + 1]); p < e; p++) s += __ldcg(&a.P[p]);
    return s;
}

// row reduction for one PageRank sweep (bins_reduce interface)
template <class Op>
struct PrRowOp {
    using T = float;
    static constexpr bool kRowAware = Op::kDataDriven;  // inactive rows are skipped
    static constexpr bool kWeights = Op::kWeights;      // staged float weight bits
    const PArgs &a;
    const PCtl &c;
    float resid = 0.0f, dangs = 0.0f;  // per-thread partials (blocks sum in FP64)
    float dfz = 0.0f;                  // data-driven: dangling mass of frozen rows
    double act = 0.0;                  // data-driven: in-edges of rows still active
    int any = 0;
    __device__ float identity() const { return 0.0f; }
    __device__ bool skip(int32_t v) const { return pr_row_skipped<Op>(a, v); }
    __device__ float edge(int32_t, int32_t, int32_t u, int32_t w) const
    {
        float cv = a.c[c.cur][u];
        if (kWeights) cv *= __int_as_float(w);
        return cv;
    }
    __device__ float combine(float x, float y) const { return x + y; }
    __device__ void flush() {}
    __device__ void finish(int32_t v, float s) { finish_row(v, s + seg_sum(a, v)); }
    // the row's whole in-edge sum s
    __device__ void finish_row(int32_t v, float s)
    {
        float dg = 0.0f;
        resid += Op::apply(a, c, v, s, any, dg);
        dangs += dg;
        if (Op::kDataDriven) {
            if (a.active[v]) act += (double)(a.frow[v + 1] - a.frow[v]);
            else dfz += dg;
        }
    }
};

template <class Op>
__global__ void __launch_bounds__(THREADS) k_pr_light(PArgs a)
{
    // lets k_pr_apply (launched with programmatic dependent launch) be
    // scheduled while this sweep runs; it waits for the sweep's completion
    mgd::pdl_enter();
    const PCtl c = *a.ctl;
    if (c.more == 0 || c.sparse) return;
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    PrRowOp<Op> op{a, c};
    (void)lane;
    (void)gwarp;
    (void)nwarps;
    const int32_t *pwt = reinterpret_cast<const int32_t *>(a.pw);
    mgd::bins_reduce(op, a.prow, a.pcol, pwt, a.wrows, a.nwrows, a.nwlong, a.trows, a.ntrows);
    // heavy-row chunks, one per CTA, in batches of 8 * THREADS edges: each
    // thread issues its 8 column loads, then its 8 gathers (one batch for
    // the default 2048-edge chunks)
    __shared__ float s_part[THREADS / 32];
    for (int32_t ch = blockIdx.x; ch < a.nhchunks; ch += gridDim.x) {
        int32_t v = a.hchunk[3 * ch], b = a.hchunk[3 * ch + 1], e = a.hchunk[3 * ch + 2];
        if (a.P) {
            // the same piece of the row's tail part: piece k of the full
            // row covers tail positions [k * chunk, (k + 1) * chunk)
            const int32_t k = (b - a.prow_full[v]) / a.chunk;
            const int32_t tb = a.prow[v], te = a.prow[v + 1];
            b = min(te, tb + k * a.chunk);
            e = min(te, b + a.chunk);
        }
        float acc = 0.0f;
        if (!pr_row_skipped<Op>(a, v)) {
            for (int32_t b0 = b; b0 < e; b0 += 8 * THREADS) {
                int32_t u[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    int32_t p = b0 + threadIdx.x + j * THREADS;
                    u[j] = p < e ? __ldcs(&a.pcol[p]) : -1;  // streamed once: evict-first
                }
#pragma unroll
                for (int j = 0; j < 8; j++)
                    if (u[j] >= 0) acc += pr_gather<Op>(a, c.cur, b0 + threadIdx.x + j * THREADS, u[j]);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            float s = 0.0f;
            for (int w = 0; w < THREADS / 32; w++) s += s_part[w];
            a.hpart[ch] = s;
        }
        __syncthreads();
    }
    block_partials<Op::kDataDriven>(a, blockIdx.x, op.resid, op.dangs, op.any, op.act, op.dfz);
}

// Sum of the partials of slots [s0, s1): lane-strided in slot order, then a
// fixed shuffle tree and warp order (thread 0 gets T[0..3] and A).
__device__ __forceinline__ void reduce_slots(const double *bpart, int s0, int s1, double T[NPART - 1], int &A)
{
    __shared__ double sp[NPART - 1][THREADS / 32];
    __shared__ int sa[THREADS / 32];
    double v[NPART - 1] = {0, 0, 0, 0};
    int any = 0;
    int b = s0 + (int)threadIdx.x;
    // four slots' loads in flight, then added in slot order (the same sums
    // as one slot at a time)
    for (; b + 3 * (int)blockDim.x < s1; b += 4 * blockDim.x) {
        double r[4][NPART];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const double *o = bpart + (size_t)NPART * (b + j * blockDim.x);
#pragma unroll
            for (int k = 0; k < NPART; k++) r[j][k] = __ldcg(&o[k]);
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            v[0] += r[j][0];
            v[1] += r[j][1];
            any |= r[j][2] != 0.0;
            v[2] += r[j][3];
            v[3] += r[j][4];
        }
    }
    for (; b < s1; b += blockDim.x) {
        const double *o = bpart + (size_t)NPART * b;
        v[0] += __ldcg(&o[0]);
        v[1] += __ldcg(&o[1]);
        any |= __ldcg(&o[2]) != 0.0;
        v[2] += __ldcg(&o[3]);
        v[3] += __ldcg(&o[4]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < NPART - 1; k++) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
        any |= __shfl_xor_sync(0xffffffffu, any, o);
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < NPART - 1; k++) sp[k][threadIdx.x >> 5] = v[k];
        sa[threadIdx.x >> 5] = any;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < NPART - 1; k++) T[k] = 0.0;
        A = 0;
        for (int w = 0; w < THREADS / 32; w++) {
            for (int k = 0; k < NPART - 1; k++) T[k] += sp[k][w];
            A |= sa[w];
        }
    }
}

// last block to arrive (per-launch counter ctl->done) returns true
__device__ __forceinline__ bool last_block(PCtl *cp)
{
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(&cp->done, 1) == (int)gridDim.x - 1);
    __syncthreads();
    return s_last != 0;
}

// End of a sweep over every row: the last block to arrive sums the blocks'
// partials of slots [0, nslots) in slot order and updates the loop state
// (iterate index, residual, dangling mass, continue flag and the graph's
// loop condition; the data-driven form's switch to queue sweeps).
template <class Op>
__device__ __forceinline__ void close_sweep(const PArgs &a, const PCtl &c, int nslots, cudaGraphConditionalHandle h,
                                            int use_cond)
{
    PCtl *cp = a.ctl;
    if (!last_block(cp)) return;
    double T[NPART - 1];
    int A;
    reduce_slots(a.bpart, 0, nslots, T, A);
    if (threadIdx.x == 0) {
        const double R = T[0], D = T[1];
        int more = 1;
        cp->done = 0;
        cp->iter = c.iter + 1;
        cp->cur = c.cur ^ 1;
        cp->resid = R;
        cp->any = A;
        if (Op::kAdjoint) cp->lam_mean = D / c.n;
        else cp->dangling = D;
        pctl_derive(cp);
        more = Op::more(A, R, c.tol) ? 1 : 0;
        if (more && cp->iter >= c.max_iter) { cp->status = 1; more = 0; }
        cp->more = more;
        if (Op::kDataDriven) {
            cp->dense_iters = c.dense_iters + 1;
            cp->act_edges = (long long)T[2];
            cp->dang_frozen = T[3];
            if (more && T[2] * SPARSE_ALPHA < (double)a.m) {
                cp->sparse = 1;
                cp->need_compact = 1;
                cp->qc = 0;
                cp->qn[0] = cp->qn[1] = 0;
            }
        }
        if (use_cond) cudaGraphSetConditional(h, more ? 1u : 0u);
    }
}

// Row finish when every in-edge sits in a segment (no tail, no heavy-row
// chunks): each row sums its pieces' partials (P[pair_off[v] ..], segments
// ascending) and applies the update.  Rows are binned by piece count at
// layout time: long rows a warp each (lane-strided, then a fixed xor tree;
// listed), the rest a thread each in row order (compensated FP32; a warp's
// 32 rows read their piece sums as one coalesced window staged in shared
// memory) -- fixed orders, so sweeps stay reproducible.
template <class Op>
__global__ void __launch_bounds__(THREADS, 8) k_pr_seg(PArgs a, cudaGraphConditionalHandle h, int use_cond)
{
    const PCtl c = *a.ctl;
    if (c.more == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0 && use_cond) cudaGraphSetConditional(h, 0u);
        return;
    }
    if (c.sparse) return;   // queue sweeps (k_prd_*) drive the loop
    PrRowOp<Op> op{a, c};
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int32_t *fw = a.fin;
    for (int32_t i = gwarp; i < a.nfw; i += nwarps) {
        const int32_t v = __ldg(&fw[i]);
        // compensated sums, lane-strided then a compensated xor tree: a
        // long row's total stays steady between sweeps
        float s = 0.0f, r = 0.0f;
        if (!op.skip(v)) {
            // four loads in flight per lane (the longest rows hold about a
            // thousand pieces), added in order
            int32_t p = __ldg(&a.pair_off[v]) + lane;
            const int32_t e = __ldg(&a.pair_off[v + 1]);
            for (; p + 96 < e; p += 128) {
                const float f0 = __ldcg(&a.P[p]), f1 = __ldcg(&a.P[p + 32]), f2 = __ldcg(&a.P[p + 64]),
                            f3 = __ldcg(&a.P[p + 96]);
                mgd::kahan_add(s, r, f0);
                mgd::kahan_add(s, r, f1);
                mgd::kahan_add(s, r, f2);
                mgd::kahan_add(s, r, f3);
            }
            for (; p < e; p += 32) mgd::kahan_add(s, r, __ldcg(&a.P[p]));
        }
        const float tot = mgd::warp_sum_comp(s, r);
        if (lane == 0) op.finish_row(v, tot);
    }
    // every other row a thread each, rows in order (the warp rows skipped):
    // a warp takes 32 consecutive rows, copies their piece sums (one
    // contiguous window of P) into shared memory with coalesced loads, and
    // each lane sums its row from there; windows longer than SEG_WIN (rows
    // near the hubs) are read from P directly.  Same adds in the same order
    // either way.
    constexpr int SEG_WIN = 512;
    __shared__ float s_win[THREADS / 32][SEG_WIN];
    float *win = s_win[threadIdx.x >> 5];
    for (int32_t vb = gwarp * 32; vb < a.n; vb += nwarps * 32) {
        const int32_t v = vb + lane;
        const bool act = v < a.n;
        const int32_t p0 = act ? __ldg(&a.pair_off[v]) : 0;
        const int32_t p1 = act ? __ldg(&a.pair_off[v + 1]) : 0;
        const int32_t last = min(a.n - vb, 32) - 1;
        const int32_t base = __shfl_sync(0xffffffffu, p0, 0), wend = __shfl_sync(0xffffffffu, p1, last);
        const int32_t len = wend - base;
        const bool in_win = len <= SEG_WIN;
        if (in_win) {
            int32_t i = lane;
            for (; i + 96 < len; i += 128) {
                const float f0 = __ldcg(&a.P[base + i]), f1 = __ldcg(&a.P[base + i + 32]),
                            f2 = __ldcg(&a.P[base + i + 64]), f3 = __ldcg(&a.P[base + i + 96]);
                win[i] = f0;
                win[i + 32] = f1;
                win[i + 64] = f2;
                win[i + 96] = f3;
            }
            for (; i < len; i += 32) win[i] = __ldcg(&a.P[base + i]);
        }
        __syncwarp();
        if (act && p1 - p0 <= a.fin_warp) {
            float s = 0.0f, r = 0.0f;
            if (!op.skip(v)) {
                if (in_win) {
                    for (int32_t p = p0 - base; p < p1 - base; p++) mgd::kahan_add(s, r, win[p]);
                } else {
                    int32_t p = p0;
                    for (; p + 4 <= p1; p += 4) {
                        const float f0 = __ldcg(&a.P[p]), f1 = __ldcg(&a.P[p + 1]), f2 = __ldcg(&a.P[p + 2]),
                                    f3 = __ldcg(&a.P[p + 3]);
                        mgd::kahan_add(s, r, f0);
                        mgd::kahan_add(s, r, f1);
                        mgd::kahan_add(s, r, f2);
                        mgd::kahan_add(s, r, f3);
                    }
                    for (; p < p1; p++) mgd::kahan_add(s, r, __ldcg(&a.P[p]));
                }
            }
            op.finish_row(v, s - r);
        }
        __syncwarp();   // the window is reused by the next 32 rows
    }
    block_partials<Op::kDataDriven>(a, blockIdx.x, op.resid, op.dangs, op.any, op.act, op.dfz);
    close_sweep<Op>(a, c, gridDim.x, h, use_cond);
}

// Heavy rows (warp per row, chunk partials summed lane-strided then by a
// fixed shuffle tree), then the last block to arrive reduces every block's
// partials in slot order and updates the loop state -- no block waits.
// The data-driven form switches to queue sweeps here once the active
// vertices' in-edges fall below m / SPARSE_ALPHA.
template <class Op>
__global__ void __launch_bounds__(THREADS) k_pr_apply(PArgs a, cudaGraphConditionalHandle h, int use_cond)
{
    mgd::pdl_enter();
    PCtl *cp = a.ctl;
    const PCtl c = *cp;
    if (c.more == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0 && use_cond) cudaGraphSetConditional(h, 0u);
        return;
    }
    if (c.sparse) return;   // queue sweeps (k_prd_*) drive the loop
    double resid = 0.0, dangs = 0.0, act = 0.0, dfz = 0.0;
    int any = 0;
    // a thread per heavy row: its chunk partials summed in chunk order, four
    // loads in flight (a row has a few chunks; every row's chain of loads
    // runs side by side instead of one warp walking two rows in turn)
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nhrows; i += gridDim.x * blockDim.x) {
        const int32_t v = a.hrows[i];
        const int32_t k1 = a.hrow_chunk[i + 1];
        int32_t k = a.hrow_chunk[i];
        float s = 0.0f;
        for (; k + 4 <= k1; k += 4) {
            const float p0 = a.hpart[k], p1 = a.hpart[k + 1], p2 = a.hpart[k + 2], p3 = a.hpart[k + 3];
            s += p0;
            s += p1;
            s += p2;
            s += p3;
        }
        for (; k < k1; k++) s += a.hpart[k];
        float dg = 0.0f;
        s += seg_sum(a, v);
        resid += Op::apply(a, c, v, s, any, dg);
        dangs += dg;
        if (Op::kDataDriven) {
            if (a.active[v]) act += (double)(a.frow[v + 1] - a.frow[v]);
            else dfz += dg;
        }
    }
    block_partials<Op::kDataDriven>(a, a.nblocks + blockIdx.x, (float)resid, (float)dangs, any, act, dfz);
    close_sweep<Op>(a, c, a.nblocks + gridDim.x, h, use_cond);
}

// ---------------------------------------------------------------------------
// data-driven frontier sweeps (processi.cu:182-407: _process_f1 works from
// the active vertices, process_f3 applies and requeues those still above
// the per-vertex tolerance).  Pull form over the queue of active vertices;
// the sweep's new values go to qval first and are applied in place by the
// next kernel, so every gather of a sweep reads the previous iterate.
// ---------------------------------------------------------------------------
// queue = every still-active vertex (once, at the switch)
__global__ void __launch_bounds__(THREADS) k_prd_compact(PArgs a)
{
    const PCtl c = *a.ctl;
    if (!c.more || !c.sparse || !c.need_compact) return;
    const int lane = mgd::lane();
    for (int32_t b0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; b0 < a.n; b0 += gridDim.x * blockDim.x) {
        const int32_t v = b0 + lane;
        const bool p = v < a.n && a.active[v] != 0;
        const unsigned m = __ballot_sync(0xffffffffu, p);
        int base = 0;
        if (lane == 0 && m) base = atomicAdd(&a.ctl->qn[0], __popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (p) a.queue[0][base + __popc(m & ((1u << lane) - 1u))] = v;
    }
}

// one queue sweep: an 8-lane group per queued vertex (four per warp), its
// full in-edge row summed lane-strided then by a fixed shuffle tree
__global__ void __launch_bounds__(THREADS) k_prd_gather(PArgs a)
{
    const PCtl c = *a.ctl;
    if (!c.more || !c.sparse) return;
    const int lane = mgd::lane(), grp = lane >> 3, gl = lane & 7;
    const int32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const int32_t nq = c.qn[c.qc];
    const int32_t *q = a.queue[c.qc];
    int32_t *nextq = a.queue[c.qc ^ 1];
    const float *cc = a.c[c.cur];
    const float *xc = a.x[c.cur];
    const float d = c.damping;
    double resid = 0.0, dangs = 0.0, act = 0.0, dfz = 0.0;
    int any = 0;
    for (int32_t base = gwarp * 4; base < nq; base += nwarps * 4) {
        const int32_t i = base + grp;
        int32_t v = -1, b = 0, e = 0;
        if (i < nq) {
            v = q[i];
            b = a.frow[v];
            e = a.frow[v + 1];
        }
        float sum = 0.0f;
        for (int32_t p = b + gl; p < e; p += 8) sum += cc[__ldg(&a.fcol[p])];
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        bool keep = false;
        if (v >= 0 && gl == 0) {
            const float xo = xc[v];
            const float xn = c.base + d * sum;
            const float diff = fabsf(xn - xo);
            const int32_t od = a.outrow[v + 1] - a.outrow[v];
            a.qval[i] = xn;
            resid += diff;
            if (od == 0) dangs += xn;
            if (diff > c.tol_row) {
                keep = true;
                any = 1;
                act += (double)(e - b);
            } else {
                a.active[v] = 0;   // frozen from now on, at xn
                if (od == 0) dfz += xn;
            }
        }
        // the group leaders that stay active requeue with one atomic per warp
        const unsigned km = __ballot_sync(0xffffffffu, keep);
        int qb = 0;
        if (lane == 0 && km) qb = atomicAdd(&a.ctl->qn[c.qc ^ 1], __popc(km));
        qb = __shfl_sync(0xffffffffu, qb, 0);
        if (keep) nextq[qb + __popc(km & ((1u << lane) - 1u))] = v;
    }
    block_partials<true>(a, blockIdx.x, (float)resid, (float)dangs, any, act, dfz);
}

// apply the queue sweep's values in place, then the last block updates the
// loop state (the iterate stays in x[cur] / c[cur])
__global__ void __launch_bounds__(THREADS) k_prd_apply(PArgs a, cudaGraphConditionalHandle h, int use_cond)
{
    PCtl *cp = a.ctl;
    const PCtl c = *cp;
    if (!c.more || !c.sparse) return;   // the dense apply set the loop condition
    const int32_t nq = c.qn[c.qc];
    const int32_t *q = a.queue[c.qc];
    float *xc = a.x[c.cur];
    float *cc = a.c[c.cur];
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x) {
        const int32_t v = q[i];
        const float xn = a.qval[i];
        const int32_t od = a.outrow[v + 1] - a.outrow[v];
        xc[v] = xn;
        cc[v] = od > 0 ? xn / (float)od : 0.0f;
    }
    if (!last_block(cp)) return;
    double T[NPART - 1];
    int A;
    reduce_slots(a.bpart, 0, gridDim.x, T, A);
    if (threadIdx.x == 0) {
        cp->done = 0;
        cp->iter = c.iter + 1;
        cp->resid = T[0];
        cp->any = A;
        cp->dangling = c.dang_frozen + T[1];
        cp->dang_frozen = c.dang_frozen + T[3];
        cp->act_edges = (long long)T[2];
        cp->need_compact = 0;
        cp->qn[c.qc] = 0;
        cp->qc = c.qc ^ 1;
        pctl_derive(cp);
        int more = (A && T[0] > (double)c.tol) ? 1 : 0;
        if (more && cp->iter >= c.max_iter) { cp->status = 1; more = 0; }
        cp->more = more;
        if (use_cond) cudaGraphSetConditional(h, more ? 1u : 0u);
    }
}

// init: x = x0, contributions, masks
template <class Op>
__global__ void k_pr_init(PArgs a, float x0)
{
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.n; v += gridDim.x * blockDim.x)
        pr_init_row<Op>(a, v, x0);
}

__global__ void k_pr_ctl_init(PCtl *c, int32_t n, int32_t max_iter, float damping, float tol, double dangling0,
                              double lam_mean0)
{
    if (threadIdx.x != 0) return;
    std::memset(c, 0, sizeof(PCtl));
    c->more = 1;
    c->max_iter = max_iter;
    c->damping = damping;
    c->tol = tol;
    c->n = n;
    c->dangling = dangling0;
    c->lam_mean = lam_mean0;
    pctl_derive(c);
}

// weighted: out-weight sums S[u] = sum_e w[e] (CSR order)
__global__ void k_row_sums(int32_t n, const int32_t *row, const float *w, float *S)
{
    for (int32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int32_t p = row[u]; p < row[u + 1]; p++) s += w[p];
        S[u] = s;
    }
}

// adjoint edge scatter: grad[e] = d x_u / S_u * (lambda_v - t_u),
// t_u = sum_k P_uk lambda_k recomputed over the row (warp per row)
__global__ void __launch_bounds__(THREADS) k_wpr_grad(int32_t n, const int32_t *row, const int32_t *col,
                                                      const float *w, const float *S, const float *x,
                                                      const float *lam, float damping, float *grad)
{
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int32_t u = gwarp; u < n; u += nwarps) {
        int32_t b = row[u], e = row[u + 1];
        float Su = S[u];
        float t = 0.0f;
        for (int32_t p = b + lane; p < e; p += 32) t += w[p] * lam[col[p]];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        float coef = Su > 0.0f ? damping * x[u] / Su : 0.0f;
        float tu = Su > 0.0f ? t / Su : 0.0f;
        for (int32_t p = b + lane; p < e; p += 32) grad[p] = coef * (lam[col[p]] - tu);
    }
}

// personalised PageRank, 32 seeds per pass: lane = seed, X / C are [n][32]
// for the current seed block (one 128 B line per vertex).  Rows with more
// than PPR_HEAVY in-edges are split into PPR_HEAVY-edge chunks (warp per
// chunk, partial sums per chunk) and combined in order by k_ppr_heavy.
constexpr int32_t PPR_HEAVY = 256;

struct PPCtl {
    int32_t more, iter, cur, status, max_iter, pad;
    double resid[32];
};

struct PPArgs {
    int32_t n;
    const int32_t *prow, *pcol, *outrow;
    const int32_t *seeds;
    int32_t nseed;
    const int32_t *hchunk;   // (row, begin, end)
    int32_t nhchunks;
    const int32_t *hrows, *hrow_chunk;
    int32_t nhrows;
    float *X0, *C0, *X1, *C1;
    float *hpart;            // [nhchunks][32]
    double *bpart;           // [2*grid][32][2]
    double *dang;            // [32] dangling mass of the current iterate
    PPCtl *ctl;
    float damping;
};

__global__ void k_ppr_init(PPArgs a, int32_t max_iter)
{
    const size_t total = (size_t)a.n * 32;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        int32_t v = (int32_t)(i >> 5);
        int s = (int)(i & 31);
        float x = (s < a.nseed && a.seeds[s] == v) ? 1.0f : 0.0f;
        a.X0[i] = x;
        int32_t od = a.outrow[v + 1] - a.outrow[v];
        a.C0[i] = od > 0 ? x / (float)od : 0.0f;
    }
    if (blockIdx.x == 0 && threadIdx.x < 32) {
        int s = threadIdx.x;
        double dg = 0.0;
        if (s < a.nseed) { int32_t v = a.seeds[s]; dg = (a.outrow[v + 1] == a.outrow[v]) ? 1.0 : 0.0; }
        a.dang[s] = dg;
        if (s == 0) {
            std::memset(a.ctl, 0, sizeof(PPCtl));
            a.ctl->more = 1;
            a.ctl->max_iter = max_iter;
        }
    }
}

__device__ __forceinline__ void ppr_apply(const PPArgs &a, const PPCtl &c, int32_t v, float s, int lane, float dang,
                                          int32_t seed, double &resid, double &dnext)
{
    const float *Xc = c.cur ? a.X1 : a.X0;
    float *Xn = c.cur ? a.X0 : a.X1;
    float *Cn = c.cur ? a.C0 : a.C1;
    float base = (v == seed) ? (1.0f - a.damping) + a.damping * dang : 0.0f;
    float xn = base + a.damping * s;
    float xo = Xc[(size_t)v * 32 + lane];
    Xn[(size_t)v * 32 + lane] = xn;
    int32_t od = a.outrow[v + 1] - a.outrow[v];
    Cn[(size_t)v * 32 + lane] = od > 0 ? xn / (float)od : 0.0f;
    if (od == 0) dnext += xn;
    resid += fabsf(xn - xo);
}

__device__ __forceinline__ void ppr_block_partials(const PPArgs &a, int slot, double resid, double dnext)
{
    __shared__ double sr[THREADS / 32][32], sd[THREADS / 32][32];
    const int lane = mgd::lane();
    sr[threadIdx.x >> 5][lane] = resid;
    sd[threadIdx.x >> 5][lane] = dnext;
    __syncthreads();
    if (threadIdx.x < 32) {
        double R = 0, D = 0;
        for (int w = 0; w < THREADS / 32; w++) { R += sr[w][threadIdx.x]; D += sd[w][threadIdx.x]; }
        a.bpart[((size_t)slot * 32 + threadIdx.x) * 2] = R;
        a.bpart[((size_t)slot * 32 + threadIdx.x) * 2 + 1] = D;
    }
}

// gather sum of C[u][lane] over [b, e)
__device__ __forceinline__ float ppr_gather(const float *Cc, const int32_t *pcol, int32_t b, int32_t e, int lane)
{
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int32_t p = b;
    for (; p + 8 <= e; p += 8) {
        int32_t u[8];
#pragma unroll
        for (int j = 0; j < 8; j++) u[j] = pcol[p + j];
        float t[8];
#pragma unroll
        for (int j = 0; j < 8; j++) t[j] = Cc[(size_t)u[j] * 32 + lane];
        s0 += t[0] + t[4];
        s1 += t[1] + t[5];
        s2 += t[2] + t[6];
        s3 += t[3] + t[7];
    }
    for (; p < e; p++) s0 += Cc[(size_t)pcol[p] * 32 + lane];
    return (s0 + s1) + (s2 + s3);
}

__global__ void __launch_bounds__(THREADS) k_ppr_sweep(PPArgs a)
{
    const PPCtl c = *a.ctl;
    if (c.more == 0) return;
    const float *Cc = c.cur ? a.C1 : a.C0;
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int32_t seed = lane < a.nseed ? a.seeds[lane] : -1;
    const float dang = (float)a.dang[lane];
    double resid = 0.0, dnext = 0.0;
    for (int32_t v = gwarp; v < a.n; v += nwarps) {
        int32_t b = a.prow[v], e = a.prow[v + 1];
        if (e - b > PPR_HEAVY) continue;  // warp-uniform
        float s = ppr_gather(Cc, a.pcol, b, e, lane);
        ppr_apply(a, c, v, s, lane, dang, seed, resid, dnext);
    }
    for (int32_t ch = gwarp; ch < a.nhchunks; ch += nwarps) {
        int32_t b = a.hchunk[3 * ch + 1], e = a.hchunk[3 * ch + 2];
        a.hpart[(size_t)ch * 32 + lane] = ppr_gather(Cc, a.pcol, b, e, lane);
    }
    ppr_block_partials(a, blockIdx.x, resid, dnext);
}

__global__ void __launch_bounds__(THREADS) k_ppr_heavy(PPArgs a)
{
    const PPCtl c = *a.ctl;
    if (c.more == 0) return;
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int32_t seed = lane < a.nseed ? a.seeds[lane] : -1;
    const float dang = (float)a.dang[lane];
    double resid = 0.0, dnext = 0.0;
    for (int32_t i = gwarp; i < a.nhrows; i += nwarps) {
        int32_t v = a.hrows[i];
        float s = 0.0f;
        for (int32_t k = a.hrow_chunk[i]; k < a.hrow_chunk[i + 1]; k++) s += a.hpart[(size_t)k * 32 + lane];
        ppr_apply(a, c, v, s, lane, dang, seed, resid, dnext);
    }
    ppr_block_partials(a, gridDim.x + blockIdx.x, resid, dnext);
}

__global__ void k_ppr_finish(PPArgs a, int nslots, float tol, cudaGraphConditionalHandle h, int use_cond)
{
    const int lane = threadIdx.x;  // 32 threads, lane = seed
    PPCtl *ctl = a.ctl;
    int more = ctl->more;
    if (more) {
        double R = 0, D = 0;
        for (int b = 0; b < nslots; b++) {
            R += a.bpart[((size_t)b * 32 + lane) * 2];
            D += a.bpart[((size_t)b * 32 + lane) * 2 + 1];
        }
        ctl->resid[lane] = R;
        a.dang[lane] = D;
        int cont = (lane < a.nseed) && (R > (double)tol);
        cont = __any_sync(0xffffffffu, cont);
        if (lane == 0) {
            ctl->iter += 1;
            ctl->cur ^= 1;
            if (cont && ctl->iter >= ctl->max_iter) { ctl->status = 1; cont = 0; }
            ctl->more = cont;
        }
        more = cont;
    }
    if (lane == 0 && use_cond) cudaGraphSetConditional(h, more ? 1u : 0u);
}

__global__ void k_ppr_store(int32_t n, const float *X, int32_t nseed, int32_t s0, float *out)
{
    const size_t total = (size_t)n * 32;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        int s = (int)(i & 31);
        if (s < nseed) out[(size_t)(s0 + s) * n + (i >> 5)] = X[i];
    }
}

}  // namespace

struct PrWS {
    mgi::DevBuf x0, x1, c0, c1, active, hpart, bpart, ctl, S, wT, gvec, grad, lam_keep, xkeep;
    mgi::DevBuf wT_caller, gvec_caller, grad_caller;  // caller-order staging of a relabeled graph
    mgi::DevBuf q0, q1, qval;  // data-driven queue sweeps
    uint64_t wT_version = 0;  // fw_version that S and wT were derived from (0: none)
    mgi::LoopGraph lg[6];
};

struct PprWS {
    mgi::DevBuf X0, X1, C0, C1, seeds, ctl, bpart, dang, hpart, out;
    mgi::LoopGraph lg;
};

struct WprWS {};

namespace mgi {

void free_pr_ws(mg_graph *g)
{
    if (!g->pws) return;
    PrWS *w = g->pws;
    DevBuf *bufs[] = {&w->x0, &w->x1, &w->c0, &w->c1, &w->active, &w->hpart, &w->bpart, &w->ctl, &w->S,
                      &w->wT, &w->gvec, &w->grad, &w->lam_keep, &w->xkeep, &w->wT_caller, &w->gvec_caller,
                      &w->grad_caller, &w->q0, &w->q1, &w->qval};
    for (DevBuf *b : bufs) dev_free(*b);
    for (auto &l : w->lg) l.destroy();
    delete w;
    g->pws = nullptr;
}

void free_ppr_ws(mg_graph *g)
{
    if (!g->ppws) return;
    PprWS *w = g->ppws;
    DevBuf *bufs[] = {&w->X0, &w->X1, &w->C0, &w->C1, &w->seeds, &w->ctl, &w->bpart, &w->dang, &w->hpart, &w->out};
    for (DevBuf *b : bufs) dev_free(*b);
    w->lg.destroy();
    delete w;
    g->ppws = nullptr;
}

void free_wpr_ws(mg_graph *g) { (void)g; }


// Runs sweeps of variant V until convergence; the result is x[ctl.cur]
// (c[ctl.cur] for the adjoint).
// apply CTAs per SM: more blocks shorten nothing (one heavy row per warp is
// already in flight) but lengthen the last-block-done reduction and its
// counter (R-MAT 22: 27 us per apply at 8, 20 us at 4)
constexpr int APPLY_PER_SM = 4;

template <class Op>
static mg_status pr_loop(mg_graph *g, PArgs &a, const mg_opts &opt, const char *name, mg_run_info *info,
                         int *final_cur)
{
    cudaStream_t s = g->stream;
    const int grid = a.nblocks;
    Profiler &P = g->prof;
    const int sl = P.slot(name);
    std::string hn = std::string(name) + "_apply";
    const int sh = P.slot(hn.c_str());
    const int apply_grid = std::max(1, std::min(std::min(grid, (a.nhrows + THREADS - 1) / THREADS),
                                                g->num_sms * APPLY_PER_SM));
    const int shs = a.P ? P.slot("pr_hub") : -1;
    const int sqc = Op::kDataDriven ? P.slot("prd_compact") : -1, sqg = Op::kDataDriven ? P.slot("prd_gather") : -1,
              sqa = Op::kDataDriven ? P.slot("prd_apply") : -1;
    BodyFn body = [&](cudaStream_t st, cudaGraphConditionalHandle h, int use_cond) -> mg_status {
        if (a.P) MG_TRY(hub_launch(g, a.c[0], a.c[1], &a.ctl->cur, &a.ctl->more, &a.ctl->sparse, st, shs));
        P.begin(sl);
        if (a.seg_only) {
            // every row finishes in k_pr_seg, which also closes the sweep
            k_pr_seg<Op><<<grid, THREADS, 0, st>>>(a, h, use_cond);
            P.end();
        } else {
            k_pr_light<Op><<<grid, THREADS, 0, st>>>(a);
            P.end();
            P.begin(sh);
            MG_TRY(launch_pdl(k_pr_apply<Op>, apply_grid, THREADS, st, a, h, use_cond));
            P.end();
        }
        if (Op::kDataDriven) {
            // queue sweeps once the switch has happened (no-ops before)
            P.begin(sqc);
            k_prd_compact<<<grid, THREADS, 0, st>>>(a);
            P.end();
            P.begin(sqg);
            k_prd_gather<<<a.qblocks, THREADS, 0, st>>>(a);
            P.end();
            P.begin(sqa);
            k_prd_apply<<<a.qblocks, THREADS, 0, st>>>(a, h, use_cond);
            P.end();
        }
        MG_CUDA(cudaGetLastError());
        return MG_OK;
    };
    int max_iter = opt.max_iter > 0 ? opt.max_iter : 10000;
    // the key holds every by-value argument of the captured kernels
    // (and the hub split's build, whose sizes the hub kernels take by value)
    const LoopKey key = LoopKey().add(Op::kSlot).add(a).add(grid).add(apply_grid).add(a.P ? g->hub.gen : 0ull);
    MG_TRY(run_loop(opt.profile ? MG_EXEC_HOST : opt.exec, opt.profile != 0, s, g->pws->lg[Op::kSlot], key, body,
                    &a.ctl->more, g->pinned_flag, max_iter + 2));
    PCtl hc;
    MG_CUDA(cudaMemcpyAsync(&hc, a.ctl, sizeof(PCtl), cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    if (a.P) MG_TRY(hub_check(g));
    if (info) {
        info->iterations = hc.iter;
        info->pull_iterations = Op::kDataDriven ? hc.dense_iters : hc.iter;   // sweeps over every row
        info->residual = hc.resid;
        info->edges_scanned = (int64_t)hc.iter * g->ne;
    }
    *final_cur = hc.cur;
    if (hc.status != 0) return fail(MG_ERR_ITER_LIMIT, "PageRank did not converge in %d sweeps (residual %g)", max_iter, hc.resid);
    return MG_OK;
}

static mg_status pr_setup(mg_graph *g, PArgs &a, bool weighted_or_adj, int32_t layout = MG_PR_LAYOUT_GATHER)
{
    if (!g->pws) g->pws = new PrWS();
    PrWS *w = g->pws;
    const size_t n = (size_t)std::max(g->nv, 1);
    const int grid = launch_grid(g, THREADS, 8);
    MG_TRY(dev_alloc(w->x0, n * 4));
    MG_TRY(dev_alloc(w->x1, n * 4));
    // 16 bytes of slack: the segmented sweep stages contributions in
    // 16-byte units, up to 12 bytes past the last vertex
    MG_TRY(dev_alloc(w->c0, n * 4 + 16));
    MG_TRY(dev_alloc(w->c1, n * 4 + 16));
    MG_TRY(dev_alloc(w->active, n * 4));
    MG_TRY(dev_alloc(w->hpart, (size_t)std::max(g->nhchunks, 1) * 4));
    MG_TRY(dev_alloc(w->bpart, (size_t)grid * 2 * NPART * 8));  // sweep blocks + apply blocks
    MG_TRY(dev_alloc(w->q0, n * 4));
    MG_TRY(dev_alloc(w->q1, n * 4));
    MG_TRY(dev_alloc(w->qval, n * 4));
    MG_TRY(dev_alloc(w->ctl, sizeof(PCtl)));
    std::memset(&a, 0, sizeof(a));
    a.n = g->nv;
    a.prow = g->trow;
    a.pcol = g->tcol;
    a.outrow = g->row.as<int32_t>();
    a.wrows = g->wrows.as<int32_t>(); a.nwrows = g->nwrows; a.nwlong = g->nwlong;
    a.trows = g->trows.as<int32_t>(); a.ntrows = g->ntrows;
    a.hchunk = g->hchunk.as<int32_t>(); a.nhchunks = g->nhchunks;
    a.hrows = g->hrows.as<int32_t>(); a.hrow_chunk = g->hrow_chunk.as<int32_t>(); a.nhrows = g->nhrows;
    a.heavy_deg = g->heavy_deg;
    a.x[0] = w->x0.as<float>(); a.x[1] = w->x1.as<float>();
    a.c[0] = w->c0.as<float>(); a.c[1] = w->c1.as<float>();
    a.active = w->active.as<int32_t>();
    a.hpart = w->hpart.as<float>();
    a.bpart = w->bpart.as<double>();
    a.nblocks = grid;
    // queue sweeps run while the active in-edges are below m / SPARSE_ALPHA:
    // two blocks per SM keep their block partials and the last block's
    // reduction small
    a.qblocks = std::min(grid, 2 * g->num_sms);
    a.ctl = w->ctl.as<PCtl>();
    a.frow = g->trow;
    a.fcol = g->tcol;
    a.queue[0] = w->q0.as<int32_t>();
    a.queue[1] = w->q1.as<int32_t>();
    a.qval = w->qval.as<float>();
    a.m = g->ne;
    // AUTO: segmented when the segments hold every source id (a graph with
    // ids past them gathers the rest through L2 and sums each row's parts
    // one by one, slower than the binned gather sweep), unless mg_autotune
    // measured otherwise
    if (layout == MG_PR_LAYOUT_AUTO)
        layout = (!g->pr_prefer_gather && hub_covers_all(g)) ? MG_PR_LAYOUT_SEGMENTED : MG_PR_LAYOUT_GATHER;
    if (!weighted_or_adj && layout == MG_PR_LAYOUT_SEGMENTED) {
        MG_TRY(hub_prepare(g));
        if (g->hub.use) {
            a.prow = g->hub.toff.as<int32_t>();
            a.pcol = g->hub.tcol.as<int32_t>();
            a.P = g->hub.P.as<float>();
            a.pair_off = g->hub.pair_off.as<int32_t>();
            if (g->hub.ntail == 0) {
                // rows finish in k_pr_seg; k_pr_apply only reduces
                a.seg_only = 1;
                a.fin = g->hub.fin.as<int32_t>();
                a.nfw = g->hub.nfw;
                a.fin_warp = g->hub.fin_warp;
                a.nhchunks = 0;
                a.nhrows = 0;
            }
            a.prow_full = g->trow;
            a.chunk = g->hchunk_size;
        }
    }
    if (weighted_or_adj) {
        if (!g->has_fw) return fail(MG_ERR_UNSUPPORTED, "float edge weights not set (mg_graph_set_float_weights)");
        if (!g->symmetric) return fail(MG_ERR_UNSUPPORTED, "weighted PageRank needs a structurally symmetric graph");
        MG_TRY(dev_alloc(w->S, n * 4));
        a.S = w->S.as<float>();
    }
    return MG_OK;
}

// transposed float weights: wT[pos of (v,u) in row v] = w[pos of (u,v) in row u].
// One thread per edge: the owner row u of position p by binary search over
// the row offsets, then u among row v's (ascending) columns.
__global__ void k_transpose_weights(int32_t n, int32_t m, const int32_t *row, const int32_t *col, const float *w,
                                    float *wT)
{
    for (int32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < m; p += gridDim.x * blockDim.x) {
        int32_t lo = 0, hi = n - 1;  // last u with row[u] <= p
        while (lo < hi) {
            const int32_t mid = (lo + hi + 1) >> 1;
            if (__ldg(&row[mid]) <= p) lo = mid; else hi = mid - 1;
        }
        const int32_t u = lo, v = __ldg(&col[p]);
        int32_t a = __ldg(&row[v]), b = __ldg(&row[v + 1]) - 1, q = -1;
        while (a <= b) {
            const int32_t mid = (a + b) >> 1;
            const int32_t cm = __ldg(&col[mid]);
            if (cm == u) { q = mid; break; }
            if (cm < u) a = mid + 1; else b = mid - 1;
        }
        if (q >= 0) wT[q] = __ldg(&w[p]);
    }
}

}  // namespace mgi

using namespace mgi;

extern "C" {

mg_status mg_pagerank(mg_graph *g, int32_t variant, const mg_opts *o, float *rank_out, mg_run_info *info)
{
    mg_opts opt;
    MG_TRY(begin_run(g, o, opt, info));
    if (variant < 0 || variant > 3) return fail(MG_ERR_INVALID, "unknown PageRank variant %d", variant);
    if (opt.pr_layout != MG_PR_LAYOUT_GATHER && opt.pr_layout != MG_PR_LAYOUT_SEGMENTED &&
        opt.pr_layout != MG_PR_LAYOUT_AUTO)
        return fail(MG_ERR_INVALID, "unknown PageRank layout %d", opt.pr_layout);
    PArgs a;
    MG_TRY(pr_setup(g, a, false, opt.pr_layout));
    cudaStream_t s = g->stream;
    const int grid = a.nblocks;
    const bool ref = variant == MG_PR_TOPOLOGY_REF || variant == MG_PR_DATA_REF;
    float d = opt.damping > 0 ? opt.damping : 0.85f;
    float tol = opt.tol > 0 ? opt.tol : 1e-6f;
    int max_iter = opt.max_iter > 0 ? opt.max_iter : 10000;
    // dangling mass of the start vector: (#zero out-degree) / n
    double dang0 = (!ref && g->nv > 0) ? (double)g->n_dangling / g->nv : 0.0;
    float x0 = ref ? 0.0f : (g->nv > 0 ? 1.0f / g->nv : 0.0f);
    k_pr_ctl_init<<<1, 32, 0, s>>>(a.ctl, g->nv, max_iter, d, tol, dang0, 0.0);
    int cur = 0;
    switch (variant) {
    case MG_PR_TOPOLOGY_REF:
        k_pr_init<PrTopologyRef><<<grid, THREADS, 0, s>>>(a, x0);
        MG_TRY(pr_loop<PrTopologyRef>(g, a, opt, "pr_pull", info, &cur));
        break;
    case MG_PR_DATA_REF:
        k_pr_init<PrDataRef><<<grid, THREADS, 0, s>>>(a, x0);
        MG_TRY(pr_loop<PrDataRef>(g, a, opt, "pr_pull", info, &cur));
        break;
    case MG_PR_TOPOLOGY:
        k_pr_init<PrTopology><<<grid, THREADS, 0, s>>>(a, x0);
        MG_TRY(pr_loop<PrTopology>(g, a, opt, "pr_pull", info, &cur));
        break;
    default:
        k_pr_init<PrData><<<grid, THREADS, 0, s>>>(a, x0);
        MG_TRY(pr_loop<PrData>(g, a, opt, "pr_pull", info, &cur));
        break;
    }
    MG_TRY(to_caller(g, MG_RES_RANK, a.x[cur], 4, 1, &g->res[MG_RES_RANK]));
    MG_TRY(end_run(g, opt, info));
    return copy_out(g, rank_out, g->res[MG_RES_RANK], (size_t)g->nv * 4);
}

mg_status mg_wpagerank(mg_graph *g, const mg_opts *o, float *x_out, mg_run_info *info)
{
    mg_opts opt;
    MG_TRY(begin_run(g, o, opt, info));
    PArgs a;
    MG_TRY(pr_setup(g, a, true));
    PrWS *w = g->pws;
    cudaStream_t s = g->stream;
    const int grid = a.nblocks;
    const size_t n = (size_t)std::max(g->nv, 1), m = (size_t)std::max(g->ne, 1);
    MG_TRY(dev_alloc(w->wT, m * 4 + 16));  // 16 bytes of tail padding, as the column arrays
    MG_TRY(dev_alloc(w->xkeep, n * 4));
    if (w->wT_version != g->fw_version) {
        // out-weight sums and transposed weights, once per set of weights
        const int egrid = launch_grid(g, THREADS, 16);
        k_row_sums<<<grid, THREADS, 0, s>>>(g->nv, g->row.as<int32_t>(), g->fw.as<float>(), a.S);
        if (g->relabeled) {
            // transposed weights are located in the caller's CSR (ascending
            // columns), then carried to engine order like the column ids
            MG_TRY(dev_alloc(w->wT_caller, m * 4 + 16));
            k_transpose_weights<<<egrid, THREADS, 0, s>>>(g->nv, g->ne, g->o_row.as<int32_t>(),
                                                          g->o_col.as<int32_t>(), g->o_fw.as<float>(),
                                                          w->wT_caller.as<float>());
            MG_TRY(edges_to_engine(g, w->wT_caller.p, w->wT.p));
        } else {
            k_transpose_weights<<<egrid, THREADS, 0, s>>>(g->nv, g->ne, g->row.as<int32_t>(), g->col.as<int32_t>(),
                                                          g->fw.as<float>(), w->wT.as<float>());
        }
        MG_CUDA(cudaGetLastError());
        w->wT_version = g->fw_version;
    }
    a.pw = w->wT.as<float>();
    float d = opt.damping > 0 ? opt.damping : 0.85f;
    float tol = opt.tol > 0 ? opt.tol : 1e-6f;
    int max_iter = opt.max_iter > 0 ? opt.max_iter : 10000;
    // rows without out-edges are dangling (their mass is spread uniformly)
    float x0 = g->nv > 0 ? 1.0f / g->nv : 0.0f;
    k_pr_ctl_init<<<1, 32, 0, s>>>(a.ctl, g->nv, max_iter, d, tol, g->nv ? (double)g->n_dangling / g->nv : 0.0, 0.0);
    k_pr_init<PrWeighted><<<grid, THREADS, 0, s>>>(a, x0);
    int cur = 0;
    MG_TRY(pr_loop<PrWeighted>(g, a, opt, "wpr_pull", info, &cur));
    MG_CUDA(cudaMemcpyAsync(w->xkeep.p, a.x[cur], (size_t)g->nv * 4, cudaMemcpyDeviceToDevice, s));
    MG_TRY(to_caller(g, MG_RES_RANK, w->xkeep.p, 4, 1, &g->res[MG_RES_RANK]));
    MG_TRY(end_run(g, opt, info));
    return copy_out(g, x_out, g->res[MG_RES_RANK], (size_t)g->nv * 4);
}

mg_status mg_wpagerank_backward(mg_graph *g, const float *g_host, const mg_opts *o, float *grad_w_out,
                                float *lambda_out, mg_run_info *info)
{
    mg_opts opt;
    MG_TRY(begin_run(g, o, opt, info));
    if (!g_host && g->nv > 0) return fail(MG_ERR_INVALID, "null loss weights");
    if (!g->pws || !g->pws->xkeep.p || !g->pws->wT.p) return fail(MG_ERR_INVALID, "run mg_wpagerank first");
    PArgs a;
    MG_TRY(pr_setup(g, a, true));
    PrWS *w = g->pws;
    cudaStream_t s = g->stream;
    const int grid = a.nblocks;
    const size_t n = (size_t)std::max(g->nv, 1), m = (size_t)std::max(g->ne, 1);
    MG_TRY(dev_alloc(w->gvec, n * 4));
    MG_TRY(dev_alloc(w->grad, m * 4));
    MG_TRY(dev_alloc(w->lam_keep, n * 4));
    MG_TRY(dev_alloc(w->gvec_caller, n * 4));
    MG_TRY(dev_alloc(w->grad_caller, m * 4));
    if (g->nv) MG_CUDA(cudaMemcpyAsync(w->gvec_caller.p, g_host, (size_t)g->nv * 4, cudaMemcpyHostToDevice, s));
    MG_TRY(vertices_to_engine(g, w->gvec_caller.p, w->gvec.p));
    k_row_sums<<<grid, THREADS, 0, s>>>(g->nv, g->row.as<int32_t>(), g->fw.as<float>(), a.S);
    // lambda = g + d * P lambda : rows of P are the CSR rows (out-edges) with weights w
    a.prow = g->row.as<int32_t>();
    a.pcol = g->col.as<int32_t>();
    a.pw = g->fw.as<float>();
    a.gvec = w->gvec.as<float>();
    float d = opt.damping > 0 ? opt.damping : 0.85f;
    float tol = opt.tol > 0 ? opt.tol : 1e-6f;
    int max_iter = opt.max_iter > 0 ? opt.max_iter : 10000;
    // initial mean of lambda = mean of g (for dangling rows)
    // and the stopping threshold, relative to |g|_1: lambda scales with g,
    // and an absolute L1 threshold would sit below FP32 resolution for
    // large n
    double gm = 0.0, g1 = 0.0;
    for (int32_t i = 0; i < g->nv; i++) {
        gm += g_host[i];
        g1 += std::fabs((double)g_host[i]);
    }
    gm = g->nv ? gm / g->nv : 0.0;
    const float tol_abs = (float)(tol * std::max(g1, 1e-30));
    k_pr_ctl_init<<<1, 32, 0, s>>>(a.ctl, g->nv, max_iter, d, tol_abs, 0.0, gm);
    k_pr_init<PrAdjoint><<<grid, THREADS, 0, s>>>(a, 0.0f);
    int cur = 0;
    MG_TRY(pr_loop<PrAdjoint>(g, a, opt, "wpr_adjoint", info, &cur));
    float *lam = a.c[cur];
    MG_CUDA(cudaMemcpyAsync(w->lam_keep.p, lam, (size_t)g->nv * 4, cudaMemcpyDeviceToDevice, s));
    int sg = g->prof.slot("wpr_grad");
    g->prof.begin(sg);
    k_wpr_grad<<<grid, THREADS, 0, s>>>(g->nv, g->row.as<int32_t>(), g->col.as<int32_t>(), g->fw.as<float>(), a.S,
                                        w->xkeep.as<float>(), w->lam_keep.as<float>(), d, w->grad.as<float>());
    g->prof.end();
    MG_CUDA(cudaGetLastError());
    const void *lam_out = nullptr;
    MG_TRY(to_caller(g, MG_RES_DELTA, w->lam_keep.p, 4, 1, &lam_out));
    MG_TRY(edges_to_caller(g, w->grad.p, w->grad_caller.p));
    MG_TRY(end_run(g, opt, info));
    MG_TRY(copy_out(g, lambda_out, lam_out, (size_t)g->nv * 4));
    return copy_out(g, grad_w_out, w->grad_caller.p, (size_t)g->ne * 4);
}

mg_status mg_ppr_batch(mg_graph *g, const int32_t *seeds, int32_t nseeds, const mg_opts *o, float *out,
                       mg_run_info *info)
{
    mg_opts opt;
    MG_TRY(begin_run(g, o, opt, info));
    if (nseeds < 0 || (nseeds > 0 && !seeds)) return fail(MG_ERR_INVALID, "invalid seeds");
    for (int32_t i = 0; i < nseeds; i++)
        if (seeds[i] < 0 || seeds[i] >= g->nv) return fail(MG_ERR_RANGE, "seed %d out of range", seeds[i]);
    if (!g->ppws) g->ppws = new PprWS();
    PprWS *w = g->ppws;
    const size_t n = (size_t)std::max(g->nv, 1);
    const int grid = launch_grid(g, THREADS, 8);
    cudaStream_t s = g->stream;
    // heavy-row chunk table for PPR (built once per graph from the pull offsets)
    if (g->ppr_nhchunks < 0) {
        std::vector<int32_t> pr(n + 1);
        MG_CUDA(cudaMemcpyAsync(pr.data(), g->trow, (size_t)(g->nv + 1) * 4, cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaStreamSynchronize(s));
        std::vector<int32_t> hc, hr, hrc{0};
        for (int32_t v = 0; v < g->nv; v++) {
            if (pr[v + 1] - pr[v] <= PPR_HEAVY) continue;
            hr.push_back(v);
            for (int32_t b = pr[v]; b < pr[v + 1]; b += PPR_HEAVY) {
                hc.push_back(v); hc.push_back(b); hc.push_back(std::min(pr[v + 1], b + PPR_HEAVY));
            }
            hrc.push_back((int32_t)(hc.size() / 3));
        }
        MG_TRY(dev_alloc(g->ppr_hchunk, std::max<size_t>(hc.size(), 3) * 4));
        MG_TRY(dev_alloc(g->ppr_hrows, std::max<size_t>(hr.size(), 1) * 4));
        MG_TRY(dev_alloc(g->ppr_hrow_chunk, hrc.size() * 4));
        if (!hc.empty()) MG_CUDA(cudaMemcpyAsync(g->ppr_hchunk.p, hc.data(), hc.size() * 4, cudaMemcpyHostToDevice, s));
        if (!hr.empty()) MG_CUDA(cudaMemcpyAsync(g->ppr_hrows.p, hr.data(), hr.size() * 4, cudaMemcpyHostToDevice, s));
        MG_CUDA(cudaMemcpyAsync(g->ppr_hrow_chunk.p, hrc.data(), hrc.size() * 4, cudaMemcpyHostToDevice, s));
        MG_CUDA(cudaStreamSynchronize(s));
        g->ppr_nhchunks = (int32_t)(hc.size() / 3);
        g->ppr_nhrows = (int32_t)hr.size();
    }
    MG_TRY(dev_alloc(w->X0, n * 32 * 4));
    MG_TRY(dev_alloc(w->X1, n * 32 * 4));
    MG_TRY(dev_alloc(w->C0, n * 32 * 4));
    MG_TRY(dev_alloc(w->C1, n * 32 * 4));
    MG_TRY(dev_alloc(w->seeds, (size_t)std::max(nseeds, 1) * 4));
    MG_TRY(dev_alloc(w->ctl, sizeof(PPCtl)));
    MG_TRY(dev_alloc(w->bpart, (size_t)2 * grid * 32 * 2 * 8));
    MG_TRY(dev_alloc(w->dang, 32 * 8));
    MG_TRY(dev_alloc(w->hpart, (size_t)std::max(g->ppr_nhchunks, 1) * 32 * 4));
    MG_TRY(dev_alloc(w->out, (size_t)std::max(nseeds, 1) * n * 4));
    std::vector<int32_t> eseeds(seeds, seeds + nseeds);
    for (int32_t &v : eseeds) v = to_engine(g, v);
    if (nseeds) MG_CUDA(cudaMemcpyAsync(w->seeds.p, eseeds.data(), (size_t)nseeds * 4, cudaMemcpyHostToDevice, s));
    float tol = opt.tol > 0 ? opt.tol : 1e-6f;
    int max_iter = opt.max_iter > 0 ? opt.max_iter : 10000;
    PPArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n = g->nv;
    a.prow = g->trow; a.pcol = g->tcol; a.outrow = g->row.as<int32_t>();
    a.hchunk = g->ppr_hchunk.as<int32_t>(); a.nhchunks = g->ppr_nhchunks;
    a.hrows = g->ppr_hrows.as<int32_t>(); a.hrow_chunk = g->ppr_hrow_chunk.as<int32_t>(); a.nhrows = g->ppr_nhrows;
    a.X0 = w->X0.as<float>(); a.X1 = w->X1.as<float>(); a.C0 = w->C0.as<float>(); a.C1 = w->C1.as<float>();
    a.hpart = w->hpart.as<float>();
    a.bpart = w->bpart.as<double>();
    a.dang = w->dang.as<double>();
    a.ctl = w->ctl.as<PPCtl>();
    a.damping = opt.damping > 0 ? opt.damping : 0.85f;
    Profiler &P = g->prof;
    const int sl = P.slot("ppr_pull"), sh = P.slot("ppr_heavy"), sf = P.slot("ppr_finish");
    int32_t total_iters = 0;
    double max_resid = 0.0;
    for (int32_t s0 = 0; s0 < nseeds; s0 += 32) {
        a.nseed = std::min(32, nseeds - s0);
        a.seeds = w->seeds.as<int32_t>() + s0;
        k_ppr_init<<<grid, THREADS, 0, s>>>(a, max_iter);
        BodyFn body = [&](cudaStream_t st, cudaGraphConditionalHandle h, int use_cond) -> mg_status {
            P.begin(sl);
            k_ppr_sweep<<<grid, THREADS, 0, st>>>(a);
            P.end();
            P.begin(sh);
            k_ppr_heavy<<<grid, THREADS, 0, st>>>(a);
            P.end();
            P.begin(sf);
            k_ppr_finish<<<1, 32, 0, st>>>(a, 2 * grid, tol, h, use_cond);
            P.end();
            MG_CUDA(cudaGetLastError());
            return MG_OK;
        };
        // the captured kernels take the whole PPArgs (pointers, counts, the
        // heavy-row table, damping), the tolerance and the grid by value
        const LoopKey key = LoopKey().add(a).add(tol).add(grid);
        MG_TRY(run_loop(opt.profile ? MG_EXEC_HOST : opt.exec, opt.profile != 0, s, w->lg, key, body, &a.ctl->more,
                        g->pinned_flag, max_iter + 2));
        PPCtl hc;
        MG_CUDA(cudaMemcpyAsync(&hc, w->ctl.p, sizeof(PPCtl), cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaStreamSynchronize(s));
        if (hc.status) return fail(MG_ERR_ITER_LIMIT, "PPR did not converge in %d sweeps", max_iter);
        total_iters += hc.iter;
        for (int i = 0; i < a.nseed; i++) max_resid = std::max(max_resid, hc.resid[i]);
        const float *X = hc.cur ? a.X1 : a.X0;
        k_ppr_store<<<grid, THREADS, 0, s>>>(g->nv, X, a.nseed, s0, w->out.as<float>());
        MG_CUDA(cudaGetLastError());
    }
    const void *res = nullptr;
    MG_TRY(to_caller(g, 7, w->out.p, 4, nseeds, &res));
    MG_TRY(end_run(g, opt, info));
    if (info) { info->iterations = total_iters; info->residual = max_resid; }
    return copy_out(g, out, res, (size_t)nseeds * g->nv * 4);
}
}  // extern "C"
