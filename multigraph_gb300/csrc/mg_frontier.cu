// mg_frontier.cu -- the built-in frontier operators (BFS, SSSP, the BC
// forward sweep) on the engine of mg_frontier_engine.cuh; the BC backward
// sweep; multi-source BC for directed graphs; their C ABI.
//
// MultiGraph_V_E_V_pull (process2.cu:263-325) becomes k_bc_back_levels.

#include "mg_frontier_engine.cuh"

namespace {

// BC backward: delta[v] = sigma[v] * sum_{w succ, level[w] = L} q[w],
// q[w] = (1 + delta[w]) / sigma[w]  (bc_phase1/2 of process2.cu:135-261 and
// process_fbc :5-132 in one pull form over the archived level lists).
// With path counts sigma = m * 2^(512 k), q is kept as (1 + delta) / m
// (FP64) and a successor's term is scaled by 2^(512 (k_v - k_w)).
// ----------------------------------------------------------------------------
struct BCtl {
    int32_t L0;       // deepest level; levels L0 .. 1 finalise their predecessors
    int32_t src;      // source of this sweep (excluded from the BC sum)
    int32_t hcnt[2];  // heavy entries listed at a level, by level parity
};

// q and the successor sums: FP32 with plain counts (below 2^100, so
// (1 + delta) / sigma stays a normal FP32 number); FP64 with extended counts,
// whose mantissas reach 2^512.
template <bool EXT>
using QT = typename std::conditional<EXT, double, float>::type;

template <bool EXT>
__global__ void k_bc_q_init(int32_t n, const mgops::PathCount *sigma, const int32_t *label, QT<EXT> *q, float *delta)
{
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        delta[v] = 0.0f;
        const double m = sigma[v].m;
        q[v] = (label[v] != mgops::UNSET && m > 0.0) ? (QT<EXT>)(1.0 / m) : (QT<EXT>)0;
    }
}

// successor w's term of a level-(L-1) entry with scale kv
template <bool EXT>
__device__ __forceinline__ QT<EXT> bc_succ_term(const Args &a, const QT<EXT> *q, int32_t w, int32_t kv)
{
    QT<EXT> t = __ldcg(&q[w]);
    if (EXT) t *= (QT<EXT>)mgops::pc_scale(kv - a.sigma[w].k);
    return t;
}

template <bool EXT>
__device__ __forceinline__ void bc_finish_vertex(int32_t v, QT<EXT> s, const mgops::PathCount *sigma, float *delta,
                                                 QT<EXT> *q, float *bc, int32_t src)
{
    const double m = sigma[v].m;
    const float dv = (float)(m * (double)s);
    delta[v] = dv;
    q[v] = (QT<EXT>)((1.0 + (double)dv) / m);
    if (bc && v != src) bc[v] += dv;
}

// Level L-1 entries pull (1+delta)/sigma from their level-L successors.
// q of the successors was written by other blocks in the previous level,
// so it is loaded through L2 (the persistent kernel runs every level in one
// launch).  Entries above PUSH_HEAVY are listed for bc_back_heavy_level.
template <bool EXT>
__device__ __forceinline__ void bc_back_level(const Args &a, int32_t L, int32_t src, int32_t *hcount, QT<EXT> *q,
                                              float *delta, float *bcacc, int32_t *heavy_list)
{
    const int32_t b0 = a.lvl_off[L - 1], b1 = a.lvl_off[L];
    const int lane = mgd::lane();
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    // vpw entries per warp: 32, or fewer when the level would leave warps idle
    int vpw = 32;
    if (b1 - b0 < nwarps * 32) {
        const int want = max(1, (b1 - b0) / nwarps);
        vpw = 1;
        while (vpw * 2 <= want) vpw *= 2;
    }
    if (vpw == 1) {
        // one entry per warp: lanes stride its edges, a shuffle tree sums
        for (int i = b0 + gwarp; i < b1; i += nwarps) {
            const int32_t v = a.queue[i];
            const int32_t b = a.row[v], e = a.row[v + 1];
            if (e - b > PUSH_HEAVY) {
                if (lane == 0) heavy_list[atomicAdd(hcount, 1)] = v;
                continue;
            }
            const int32_t kv = EXT ? a.sigma[v].k : 0;
            QT<EXT> acc = 0;
            for (int32_t p = b + lane; p < e; p += 32) {
                const int32_t w = a.col[p];
                if (a.label[w] == L) acc += bc_succ_term<EXT>(a, q, w, kv);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) bc_finish_vertex<EXT>(v, acc, a.sigma, delta, q, bcacc, src);
        }
        return;
    }
    for (int base = b0 + gwarp * vpw; base < b1; base += nwarps * vpw) {
        int32_t v = -1, start = 0, deg = 0, kv = 0;
        if (lane < vpw && base + lane < b1) {
            v = a.queue[base + lane];
            start = a.row[v];
            deg = a.row[v + 1] - start;
            if (EXT) kv = a.sigma[v].k;
            if (deg > PUSH_HEAVY) {
                int h = atomicAdd(hcount, 1);
                heavy_list[h] = v;
                deg = 0;
                v = -1;
            }
        }
        int incl = mgd::warp_scan_incl(deg);
        int excl = incl - deg;
        int total = __shfl_sync(0xffffffffu, incl, 31);
        QT<EXT> acc = 0;
        for (int k0 = 0; k0 < total; k0 += 32) {
            int k = k0 + lane;
            int kk = k < total ? k : total - 1;
            int own = mgd::owner_lane(excl, kk);
            int32_t e = __shfl_sync(0xffffffffu, start, own) + (kk - __shfl_sync(0xffffffffu, excl, own));
            const int32_t kown = __shfl_sync(0xffffffffu, kv, own);
            QT<EXT> t = 0;
            if (k < total) {
                int32_t w = a.col[e];
                if (a.label[w] == L) t = bc_succ_term<EXT>(a, q, w, kown);
            } else {
                own = -1;
            }
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int oo = __shfl_down_sync(0xffffffffu, own, o);
                QT<EXT> ot = __shfl_down_sync(0xffffffffu, t, o);
                if (lane + o < 32 && oo == own) t += ot;
            }
            int prev_own = __shfl_up_sync(0xffffffffu, own, 1);
            bool head = (own >= 0) && (lane == 0 || prev_own != own);
            unsigned heads = __ballot_sync(0xffffffffu, head);
            while (heads) {
                int hl = __ffs(heads) - 1;
                heads &= heads - 1;
                int ho = __shfl_sync(0xffffffffu, own, hl);
                QT<EXT> ht = __shfl_sync(0xffffffffu, t, hl);
                if (lane == ho) acc += ht;
            }
        }
        if (v >= 0) bc_finish_vertex<EXT>(v, acc, a.sigma, delta, q, bcacc, src);
    }
}

// heavy entries of the level: a CTA each, fixed-order block sum
template <bool EXT>
__device__ __forceinline__ void bc_back_heavy_level(const Args &a, int32_t L, int32_t src, int32_t nheavy, QT<EXT> *q,
                                                    float *delta, float *bcacc, const int32_t *heavy_list)
{
    __shared__ QT<EXT> s_part[32];
    for (int32_t h = blockIdx.x; h < nheavy; h += gridDim.x) {
        int32_t v = __ldcg(&heavy_list[h]);
        int32_t b = a.row[v], e = a.row[v + 1];
        const int32_t kv = EXT ? a.sigma[v].k : 0;
        QT<EXT> acc = 0;
        for (int32_t p = b + threadIdx.x; p < e; p += blockDim.x) {
            int32_t w = a.col[p];
            if (a.label[w] == L) acc += bc_succ_term<EXT>(a, q, w, kv);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            QT<EXT> s = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += s_part[w];
            bc_finish_vertex<EXT>(v, s, a.sigma, delta, q, bcacc, src);
        }
        __syncthreads();
    }
}

// Persistent backward sweep: every level in one cooperative launch, one or
// two grid barriers per level (light entries | barrier | heavy entries |
// barrier, the second half only when the level listed heavy entries).  Every block walks L = L0 .. 1 itself; the heavy-entry counter
// alternates with the level's parity, and block 0 clears the one the next
// level will use while the current level runs (its last readers finished
// before the previous barrier).  A barrier timeout sets the error flag; the
// host reads it and fails the run.
template <bool EXT>
__global__ void __launch_bounds__(PTHREADS, 2) k_bc_back_levels(Args a, BCtl *bc_ctl, QT<EXT> *q, float *delta,
                                                                float *bcacc, int32_t *heavy_list)
{
    __shared__ int4 s_b;
    __shared__ int s_nheavy;
    if (threadIdx.x == 0) s_b = __ldcg(reinterpret_cast<const int4 *>(bc_ctl));
    __syncthreads();
    const int32_t L0 = s_b.x, src = s_b.y;
    for (int32_t L = L0; L >= 1; L--) {
        const int par = L & 1;
        if (blockIdx.x == 0 && threadIdx.x == 0) bc_ctl->hcnt[par ^ 1] = 0;
        bc_back_level<EXT>(a, L, src, &bc_ctl->hcnt[par], q, delta, bcacc, heavy_list);
        if (!mgd::grid_sync(a.bar, a.bar_err, a.bar_never)) return;
        if (threadIdx.x == 0) s_nheavy = __ldcg(&bc_ctl->hcnt[par]);
        __syncthreads();
        const int32_t nheavy = s_nheavy;
        // most levels list no heavy entry: every block sees the same count
        // and skips the heavy phase and its barrier together (block 0's
        // early clear of this counter then leaves it at the 0 it holds)
        if (nheavy == 0) continue;
        bc_back_heavy_level<EXT>(a, L, src, nheavy, q, delta, bcacc, heavy_list);
        if (!mgd::grid_sync(a.bar, a.bar_err, a.bar_never)) return;
    }
}

__global__ void k_pc_to_double(int32_t n, const mgops::PathCount *sigma, double *out)
{
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        out[v] = mgops::pc_to_double(sigma[v]);
}

__global__ void k_bc_back_init(const FCtl *fc, BCtl *bc_ctl, int32_t src)
{
    if (threadIdx.x != 0) return;
    bc_ctl->src = src;
    bc_ctl->L0 = fc->nlevels - 1;
    bc_ctl->hcnt[0] = 0;
    bc_ctl->hcnt[1] = 0;
}

}  // namespace

namespace mgi {

void free_frontier_ws(mg_graph *g)
{
    if (!g->fws) return;
    FrontierWS *w = g->fws;
    DevBuf *bufs[] = {&w->label, &w->sigma, &w->sigma_d, &w->bm, &w->visited, &w->queue, &w->heavy,
                      &w->lvl_off, &w->ctl, &w->q, &w->delta, &w->bc, &w->bctl, &w->bheavy, &w->srcbuf, &w->bar,
                      &w->cnt};
    for (DevBuf *b : bufs) dev_free(*b);
    for (auto &kv : w->lg) kv.second.destroy();
    delete w;
    g->fws = nullptr;
}

// BFS from several sources at once (one traversal of a disjoint union of
// graphs: the multi-graph batch)
mg_status frontier_bfs_multi(mg_graph *g, const int32_t *srcs_host, int32_t nsrc, const mg_opts &opt,
                             mg_run_info *info)
{
    return frontier_run_impl<mgops::Bfs>(g, 0, srcs_host, nsrc, opt, info);
}

const void *frontier_label(mg_graph *g) { return g->fws ? g->fws->label.p : nullptr; }


mg_status bc_backward(mg_graph *g, int32_t src, const mg_opts &opt, float *bcacc)
{
    FrontierWS *w = g->fws;
    const size_t n = (size_t)std::max(g->nv, 1);
    MG_TRY(dev_alloc(w->q, n * 8));
    MG_TRY(dev_alloc(w->delta, n * 4));
    MG_TRY(dev_alloc(w->bctl, sizeof(BCtl)));
    MG_TRY(dev_alloc(w->bheavy, n * 4));
    Args a = make_args(g);
    cudaStream_t s = g->stream;
    void *q = w->q.p;
    float *delta = w->delta.as<float>();
    BCtl *bc = w->bctl.as<BCtl>();
    int32_t *hl = w->bheavy.as<int32_t>();
    const int grid = launch_grid(g, THREADS, 8);
    if (w->coop_back == 0) {
        int per_sm = 0;
        int per_sm_x = 0;
        MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bc_back_levels<false>, PTHREADS, 0));
        MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_x, k_bc_back_levels<true>, PTHREADS, 0));
        per_sm = std::min(per_sm, per_sm_x);
        if (per_sm < 1) return fail(MG_ERR_CUDA, "persistent backward kernel does not fit on an SM");
        w->coop_back = std::min(per_sm, 2) * g->num_sms;
    }
    if (a.bc_ext) k_bc_q_init<true><<<grid, THREADS, 0, s>>>(g->nv, a.sigma, a.label, (double *)q, delta);
    else k_bc_q_init<false><<<grid, THREADS, 0, s>>>(g->nv, a.sigma, a.label, (float *)q, delta);
    k_bc_back_init<<<1, 32, 0, s>>>(a.ctl, bc, src);
    MG_CUDA(cudaMemsetAsync(w->bar.p, 0, BAR_BYTES, s));
    MG_CUDA(cudaGetLastError());
    // every level in one cooperative launch
    Profiler &P = g->prof;
    const int sb = P.slot("bc_back");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)w->coop_back);
    cfg.blockDim = dim3(PTHREADS);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    P.begin(sb);
    if (a.bc_ext) MG_CUDA(cudaLaunchKernelEx(&cfg, k_bc_back_levels<true>, a, bc, (double *)q, delta, bcacc, hl));
    else MG_CUDA(cudaLaunchKernelEx(&cfg, k_bc_back_levels<false>, a, bc, (float *)q, delta, bcacc, hl));
    P.end();
    int err = 0;
    MG_CUDA(cudaMemcpyAsync(&err, a.bar_err, 4, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    if (err) return fail(MG_ERR_CUDA, "grid barrier of the persistent backward kernel timed out");
    (void)opt;
    return MG_OK;
}

}  // namespace mgi

using namespace mgi;

extern "C" {

static mg_status check_source(const mg_graph *g, int32_t s)
{
    if (s < 0 || s >= g->nv) return fail(MG_ERR_RANGE, "source %d out of range [0,%d)", s, g->nv);
    return MG_OK;
}

mg_status mg_bfs(mg_graph *g, int32_t source, const mg_opts *o, int32_t *level_out, mg_run_info *info)
{
    mg_opts opt;
    MG_TRY(begin_run(g, o, opt, info));
    MG_TRY(check_source(g, source));
    MG_TRY(frontier_run_impl<mgops::Bfs>(g, to_engine(g, source), nullptr, 0, opt, info));
    MG_TRY(publish(g, MG_RES_LEVEL, g->fws->label.p, 4));
    MG_TRY(end_run(g, opt, info));
    return copy_out(g, level_out, g->res[MG_RES_LEVEL], (size_t)g->nv * 4);
}

mg_status mg_sssp(mg_graph *g, int32_t source, const mg_opts *o, int32_t *dist_out, mg_run_info *info)
{
    mg_opts opt;
    MG_TRY(begin_run(g, o, opt, info));
    MG_TRY(check_source(g, source));
    MG_TRY(frontier_run_impl<mgops::Sssp>(g, to_engine(g, source), nullptr, 0, opt, info));
    MG_TRY(publish(g, MG_RES_DIST, g->fws->label.p, 4));
    MG_TRY(end_run(g, opt, info));
    return copy_out(g, dist_out, g->res[MG_RES_DIST], (size_t)g->nv * 4);
}

mg_status mg_bc(mg_graph *g, int32_t source, const mg_opts *o, int32_t *level_out, double *sigma_out,
                float *delta_out, mg_run_info *info)
{
    mg_opts opt;
    MG_TRY(begin_run(g, o, opt, info));
    MG_TRY(check_source(g, source));
    const int32_t s = to_engine(g, source);
    MG_TRY(frontier_run_impl<mgops::BcForward>(g, s, nullptr, 0, opt, info));
    MG_TRY(bc_backward(g, s, opt, nullptr));
    FrontierWS *w = g->fws;
    MG_TRY(publish(g, MG_RES_LEVEL, w->label.p, 4));
    // path counts as FP64 values (infinity where a count exceeds the FP64 range)
    MG_TRY(dev_alloc(w->sigma_d, (size_t)std::max(g->nv, 1) * 8));
    k_pc_to_double<<<launch_grid(g, THREADS, 8), THREADS, 0, g->stream>>>(g->nv, w->sigma.as<mgops::PathCount>(),
                                                                           w->sigma_d.as<double>());
    MG_CUDA(cudaGetLastError());
    MG_TRY(publish(g, MG_RES_SIGMA, w->sigma_d.p, 8));
    MG_TRY(publish(g, MG_RES_DELTA, w->delta.p, 4));
    MG_TRY(end_run(g, opt, info));
    MG_TRY(copy_out(g, level_out, g->res[MG_RES_LEVEL], (size_t)g->nv * 4));
    MG_TRY(copy_out(g, sigma_out, g->res[MG_RES_SIGMA], (size_t)g->nv * 8));
    return copy_out(g, delta_out, g->res[MG_RES_DELTA], (size_t)g->nv * 4);
}

mg_status mg_bc_multi(mg_graph *g, const int32_t *sources, int32_t nsrc, const mg_opts *o, float *bc_out,
                      mg_run_info *info)
{
    mg_opts opt;
    MG_TRY(begin_run(g, o, opt, info));
    if (nsrc < 0 || (nsrc > 0 && !sources)) return fail(MG_ERR_INVALID, "invalid sources");
    for (int32_t i = 0; i < nsrc; i++)
        if (sources[i] < 0 || sources[i] >= g->nv) return fail(MG_ERR_RANGE, "source %d out of range", sources[i]);
    if (g->symmetric) {
        // 32 sources per traversal (mg_bcb.cu)
        std::vector<int32_t> eng((size_t)nsrc);
        for (int32_t i = 0; i < nsrc; i++) eng[(size_t)i] = to_engine(g, sources[i]);
        const float *bcd = nullptr;
        MG_TRY(bc_batched(g, eng.data(), nsrc, opt, info, &bcd));
        MG_TRY(publish(g, MG_RES_BC, bcd, 4));
        mg_run_info keep;
        if (info) keep = *info;
        MG_TRY(end_run(g, opt, info));
        if (info) { info->iterations = keep.iterations; info->pull_iterations = keep.pull_iterations; }
        return copy_out(g, bc_out, g->res[MG_RES_BC], (size_t)g->nv * 4);
    }
    // directed graphs: one forward/backward traversal per source
    MG_TRY(ensure_ws<mgops::BcForward>(g));
    FrontierWS *w = g->fws;
    MG_TRY(dev_alloc(w->bc, (size_t)std::max(g->nv, 1) * 4));
    MG_CUDA(cudaMemsetAsync(w->bc.p, 0, (size_t)g->nv * 4, g->stream));
    int32_t iters = 0;
    for (int32_t i = 0; i < nsrc; i++) {
        mg_run_info sub;
        const int32_t s = to_engine(g, sources[i]);
        MG_TRY(frontier_run_impl<mgops::BcForward>(g, s, nullptr, 0, opt, &sub));
        MG_TRY(bc_backward(g, s, opt, w->bc.as<float>()));
        iters += sub.iterations;
    }
    MG_TRY(publish(g, MG_RES_BC, w->bc.p, 4));
    MG_TRY(end_run(g, opt, info));
    if (info) info->iterations = iters;
    return copy_out(g, bc_out, g->res[MG_RES_BC], (size_t)g->nv * 4);
}

}  // extern "C"
