// mg_bcb.cu -- batched multi-source Brandes BC, per-level kernels and the
// host driver.  The algorithm, the data layout and the phase bodies are in
// mg_bcb.cuh.
//
// One CUDA-graph WHILE loop per sweep: forward level d is k_bb_mark (sparse
// levels) -> k_bb_pull -> k_bb_heavy (graphs with heavy rows) ->
// k_bb_compact, whose last block to finish decides the next level; backward
// level L is k_bbb_pull -> k_bbb_heavy -> k_bbb_next, whose last block
// steps L.

#include "mg_bcb.cuh"

namespace {

using namespace mgbc;

__global__ void k_bb_init(BbArgs a, int32_t nsrc, int32_t dirmode, int32_t alpha, int32_t max_levels)
{
    const int lane = threadIdx.x;
    const bool valid = lane < nsrc;
    const int32_t v = valid ? a.src[lane] : -1 - lane;
    const uint32_t same = __match_any_sync(0xffffffffu, v);
    const bool leader = valid && lane == __ffs(same) - 1;
    if (valid) a.sig[(size_t)v * W + lane] = mgops::pc_one();
    const uint32_t leaders = __ballot_sync(0xffffffffu, leader);
    unsigned long long deg = 0;
    int heavy = 0;
    if (leader) {
        const int pos = __popc(leaders & ((1u << lane) - 1u));
        a.vis[v] = same;
        a.fm0[v] = same;
        a.arch[pos] = v;
        a.amask[pos] = same;
        const int32_t d = a.row[v + 1] - a.row[v];
        deg = (unsigned long long)d;
        heavy = d > MARK_HEAVY;
    }
    const uint32_t hv = __ballot_sync(0xffffffffu, heavy);
    if (heavy) a.fheavy[__popc(hv & ((1u << lane) - 1u))] = v;
    deg = warp_sum_u64(deg);
    if (lane == 0) {
        BbCtl c;
        memset(&c, 0, sizeof(c));
        const int cnt = __popc(leaders);
        c.more = cnt > 0;
        c.d = 0;
        c.cur = 0;
        c.dirmode = dirmode;
        c.alpha = alpha;
        c.max_levels = max_levels;
        c.gmask = nsrc >= 32 ? 0xffffffffu : ((1u << nsrc) - 1u);
        c.nfh = __popc(hv);
        c.nfe_cur = deg;
        c.dense = dirmode == MG_DIR_PULL;
        c.dense_levels = c.dense;
        a.off[0] = 0;
        a.off[1] = cnt;
        *a.ctl = c;
    }
}


// The kernels of one level run back to back with programmatic dependent
// launch (mgi::launch_pdl / mgd::pdl_enter), so a level's launch latencies
// overlap the previous kernel's tail.
using mgd::pdl_enter;

__global__ void __launch_bounds__(THREADS) k_bb_mark(BbArgs a)
{
    pdl_enter();
    const BbCtl c = *a.ctl;
    if (c.more == 0 || c.dense) return;
    bb_mark_phase(a, c, a.off[c.d], a.off[c.d + 1], &a.ctl->k.ncand);
}

template <bool TP, bool EXT>
__global__ void __launch_bounds__(THREADS) k_bb_pull(BbArgs a)
{
    pdl_enter();
    const BbCtl c = *a.ctl;
    if (c.more == 0) return;
    bb_pull_phase<TP, EXT>(a, c, c.dense ? a.n : c.k.ncand);
}

__global__ void __launch_bounds__(THREADS) k_bb_heavy(BbArgs a)
{
    pdl_enter();
    const BbCtl c = *a.ctl;
    if (c.more == 0) return;
    bb_heavy_phase(a, c);
}

// Archives level d+1 and, in the last block to finish, decides the next
// level (Beamer's direction test, loop condition)
__global__ void __launch_bounds__(THREADS) k_bb_compact(BbArgs a, cudaGraphConditionalHandle h, int use_cond)
{
    pdl_enter();
    BbCtl *cp = a.ctl;
    const BbCtl c = *cp;
    if (c.more == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0 && use_cond) cudaGraphSetConditional(h, 0u);
        return;
    }
    bb_compact_phase(a, c, a.off[c.d], a.off[c.d + 1], c.dense ? a.n : c.k.ncand, &cp->k);
    if (!last_block_done(&cp->done)) return;
    BbCtl n = load_ctl_l2(cp);
    const LvlCnt k = n.k;
    const int32_t d = n.d;
    int32_t off_d2;
    bb_decide(n, k, n.ovf, a.off[d + 1], off_d2, a.m);
    a.off[d + 2] = off_d2;
    n.k = LvlCnt{0, 0, 0, 0, 0ull};
    n.done = 0;
    *cp = n;
    if (use_cond) cudaGraphSetConditional(h, n.more ? 1u : 0u);
}

// Backward start: L = deepest level, the masks of levels L and L-1 scattered
__global__ void k_bbb_start(BbArgs a)
{
    const BbCtl c = *a.ctl;
    const int32_t L = c.nlevels - 1;
    const bool run = c.status == 0 && c.ovf == 0 && L >= 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ctl->L = L;
        a.ctl->more = run;
        a.ctl->done = 0;
    }
    if (run) bbb_start_phase(a, L);
}

template <bool TP, bool EXT>
__global__ void __launch_bounds__(THREADS) k_bbb_pull(BbArgs a)
{
    pdl_enter();
    const BbCtl c = *a.ctl;
    if (c.more == 0) return;
    bbb_pull_phase<TP, EXT>(a, c.L);
}

template <bool EXT>
__global__ void __launch_bounds__(THREADS, 8) k_bbb_heavy(BbArgs a)
{
    pdl_enter();
    const BbCtl c = *a.ctl;
    if (c.more == 0) return;
    bbb_heavy_phase<EXT>(a, c.L);
}

// End of backward level L (masks cleared / scattered); the last block to
// finish steps to L-1
__global__ void __launch_bounds__(THREADS) k_bbb_next(BbArgs a, cudaGraphConditionalHandle h, int use_cond)
{
    pdl_enter();
    BbCtl *cp = a.ctl;
    const BbCtl c = *cp;
    if (c.more == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0 && use_cond) cudaGraphSetConditional(h, 0u);
        return;
    }
    bbb_next_phase(a, c.L);
    if (!last_block_done(&cp->done)) return;
    const int32_t L = __ldcg(&cp->L) - 1;
    const int more = L >= 1;
    cp->L = L;
    cp->more = more;
    cp->done = 0;
    if (use_cond) cudaGraphSetConditional(h, more ? 1u : 0u);
}

// ---------------------------------------------------------------------------
// Persistent sweeps for low-degree graphs (lattices, road networks): their
// thousands of levels hold a few thousand entries each, so a level's
// launches cost more than its work.  One cooperative launch (every block
// resident) runs consecutive sparse forward levels -- mark | barrier | pull
// | barrier | heavy | barrier | compact | barrier, then every block decides
// the next level on its own copy of the loop state from the level's
// counters (the same inputs give the same decision everywhere) -- until
// the sweep ends or the direction test picks a dense level, which the
// per-level kernels above then run.  Another launch runs every backward
// level: pull | barrier | heavy | barrier | next | barrier.  The phase
// bodies are the per-level kernels' own.  A barrier timeout sets status 3.

__device__ __forceinline__ LvlCnt load_cnt_l2(const LvlCnt *k)
{
    LvlCnt r;
    r.ncand = __ldcg(&k->ncand);
    r.nnew = __ldcg(&k->nnew);
    r.nfh_build = __ldcg(&k->nfh_build);
    r.status = __ldcg(&k->status);
    r.nfe = __ldcg(&k->nfe);
    return r;
}

template <bool TP, bool EXT>
__global__ void __launch_bounds__(THREADS) k_bb_levels(BbArgs a, int heavy)
{
    __shared__ BbCtl s_c;
    __shared__ int32_t s_off[2];
    if (threadIdx.x == 0) {
        s_c = load_ctl_l2(a.ctl);
        s_off[0] = __ldcg(&a.off[s_c.d]);
        s_off[1] = __ldcg(&a.off[s_c.d + 1]);
    }
    __syncthreads();
    bool ran = false, ok = true;
    for (int32_t lv = 0;; lv++) {
        const BbCtl c = s_c;
        if (c.more == 0 || c.dense) break;
        ran = true;
        LvlCnt *k = a.pcnt + (lv & 3);
        if (blockIdx.x == 0 && threadIdx.x == 0) a.pcnt[(lv + 2) & 3] = LvlCnt{0, 0, 0, 0, 0ull};
        const int32_t b0 = s_off[0], b1 = s_off[1];
        bb_mark_phase(a, c, b0, b1, &k->ncand);
        if (!(ok = mgd::grid_sync(a.bar, a.bar_err))) break;
        const int32_t ncand = __ldcg(&k->ncand);
        bb_pull_phase<TP, EXT>(a, c, ncand);
        if (!(ok = mgd::grid_sync(a.bar, a.bar_err))) break;
        if (heavy) {
            bb_heavy_phase(a, c);
            if (!(ok = mgd::grid_sync(a.bar, a.bar_err))) break;
        }
        bb_compact_phase(a, c, b0, b1, ncand, k);
        if (!(ok = mgd::grid_sync(a.bar, a.bar_err))) break;
        if (threadIdx.x == 0) {
            BbCtl n = c;
            int32_t off_d2;
            bb_decide(n, load_cnt_l2(k), __ldcg(&a.ctl->ovf), b1, off_d2, a.m);
            if (blockIdx.x == 0) a.off[c.d + 2] = off_d2;
            s_c = n;
            s_off[0] = b1;
            s_off[1] = off_d2;
        }
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && (ran || !ok)) {
        BbCtl n = s_c;
        if (!ok || *(volatile int *)a.bar_err) {
            n.status = 3;
            n.more = 0;
        }
        n.ovf |= __ldcg(&a.ctl->ovf);
        n.k = LvlCnt{0, 0, 0, 0, 0ull};
        n.done = 0;
        *a.ctl = n;
    }
}

template <bool TP, bool EXT>
__global__ void __launch_bounds__(THREADS) k_bbb_levels(BbArgs a, int heavy)
{
    __shared__ BbCtl s_c;
    if (threadIdx.x == 0) s_c = load_ctl_l2(a.ctl);
    __syncthreads();
    if (s_c.more == 0) return;
    bool ok = true;
    int32_t L = s_c.L;
    for (; L >= 1; L--) {
        bbb_pull_phase<TP, EXT>(a, L);
        if (!(ok = mgd::grid_sync(a.bar, a.bar_err))) break;
        if (heavy) {
            bbb_heavy_phase<EXT>(a, L);
            if (!(ok = mgd::grid_sync(a.bar, a.bar_err))) break;
        }
        bbb_next_phase(a, L);
        if (!(ok = mgd::grid_sync(a.bar, a.bar_err))) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ctl->L = ok ? 0 : L;
        a.ctl->more = 0;
        a.ctl->done = 0;
        if (!ok || *(volatile int *)a.bar_err) a.ctl->status = 3;
    }
}

template <class K>
mg_status launch_coop(K kernel, int grid, cudaStream_t st, const BbArgs &a, int heavy)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(THREADS);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    MG_CUDA(cudaLaunchKernelEx(&cfg, kernel, a, heavy));
    return MG_OK;
}

__global__ void k_bb_to_float(int32_t n, const double *bc, float *out)
{
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) out[v] = (float)bc[v];
}

}  // namespace


struct BcWS {
    mgi::DevBuf vis, fm, cbm, cand, arch, amask, off, sig, q, hpart, hmask, bc, bcf, fheavy, src, ctl, bar, pcnt;
    mgi::LoopGraph fwd, bwd;
    int coop_f = 0, coop_b = 0;   // resident grids of the persistent sweeps (0: not sized yet)
};

namespace mgi {

using namespace mgbc;


void free_bc_ws(mg_graph *g)
{
    if (!g->bws) return;
    BcWS *w = g->bws;
    DevBuf *bufs[] = {&w->vis, &w->fm, &w->cbm, &w->cand, &w->arch, &w->amask, &w->off, &w->sig,
                      &w->q, &w->hpart, &w->hmask, &w->bc, &w->bcf, &w->fheavy, &w->src, &w->ctl,
                      &w->bar, &w->pcnt};
    for (DevBuf *b : bufs) dev_free(*b);
    w->fwd.destroy();
    w->bwd.destroy();
    delete w;
    g->bws = nullptr;
}

// Batched BC over engine-id sources; the float scores (engine order) are
// left in the workspace and returned through *bc_dev.
mg_status bc_batched(mg_graph *g, const int32_t *src_engine, int32_t nsrc, const mg_opts &opt, mg_run_info *info,
                     const float **bc_dev)
{
    if (!g->symmetric) return fail(MG_ERR_UNSUPPORTED, "batched BC needs a structurally symmetric graph");
    // archive positions (up to 32 entries per vertex) are int32
    if ((int64_t)g->nv * W > (int64_t)INT32_MAX - 4)
        return fail(MG_ERR_UNSUPPORTED, "batched BC takes graphs of up to %d vertices", (int)((INT32_MAX - 4) / W));
    if (!g->bws) g->bws = new BcWS();
    BcWS *w = g->bws;
    const size_t n = (size_t)std::max(g->nv, 1);
    const size_t words = (n + 31) / 32;
    const size_t cap = n * W;
    const size_t nch = (size_t)std::max(g->nhchunks, 1);
    MG_TRY(dev_alloc(w->vis, n * 4));
    MG_TRY(dev_alloc(w->fm, 3 * n * 4));
    MG_TRY(dev_alloc(w->cbm, words * 4));
    MG_TRY(dev_alloc(w->cand, n * 4));
    MG_TRY(dev_alloc(w->arch, cap * 4));
    MG_TRY(dev_alloc(w->amask, cap * 4));
    MG_TRY(dev_alloc(w->off, (n + 4) * 4));
    MG_TRY(dev_alloc(w->sig, cap * sizeof(mgops::PathCount)));
    MG_TRY(dev_alloc(w->q, cap * 8));
    MG_TRY(dev_alloc(w->hpart, nch * W * sizeof(mgops::PathCount)));
    MG_TRY(dev_alloc(w->hmask, nch * 4));
    MG_TRY(dev_alloc(w->bc, n * 8));
    MG_TRY(dev_alloc(w->bcf, n * 4));
    MG_TRY(dev_alloc(w->fheavy, n * 4));
    MG_TRY(dev_alloc(w->src, W * 4));
    MG_TRY(dev_alloc(w->ctl, sizeof(BbCtl)));
    MG_TRY(dev_alloc(w->bar, 64));
    MG_TRY(dev_alloc(w->pcnt, 4 * sizeof(LvlCnt)));

    BbArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n = g->nv;
    a.m = g->ne;
    a.row = g->row.as<int32_t>(); a.col = g->col.as<int32_t>();
    a.trow = g->trow; a.tcol = g->tcol;
    a.hchunk = g->hchunk.as<int32_t>(); a.nhchunks = g->nhchunks;
    a.hrows = g->hrows.as<int32_t>(); a.hrow_chunk = g->hrow_chunk.as<int32_t>(); a.nhrows = g->nhrows;
    a.heavy_deg = g->heavy_deg;
    a.vis = w->vis.as<uint32_t>();
    a.fm0 = w->fm.as<uint32_t>(); a.fm1 = a.fm0 + n; a.fm2 = a.fm1 + n;
    a.cbm = w->cbm.as<uint32_t>();
    a.cand = w->cand.as<int32_t>();
    a.arch = w->arch.as<int32_t>();
    a.amask = w->amask.as<uint32_t>();
    a.cap = cap;
    a.off = w->off.as<int32_t>();
    a.sig = w->sig.as<mgops::PathCount>();
    a.q = w->q.p;
    a.hpart = w->hpart.as<mgops::PathCount>();
    a.ext = g->bc_ext ? 1 : 0;
    a.hmask = w->hmask.as<uint32_t>();
    a.bc = w->bc.as<double>();
    a.fheavy = w->fheavy.as<int32_t>();
    a.src = w->src.as<int32_t>();
    a.ctl = w->ctl.as<BbCtl>();
    a.bar = w->bar.as<unsigned>();
    a.bar_err = reinterpret_cast<int *>(a.bar + 1);
    a.pcnt = w->pcnt.as<LvlCnt>();

    cudaStream_t s = g->stream;
    MG_CUDA(cudaMemsetAsync(a.bc, 0, n * 8, s));
    MG_CUDA(cudaMemsetAsync(a.cbm, 0, words * 4, s));
    const int grid = launch_grid(g, THREADS, 8);
    // Low-degree graphs (average degree <= TP_AVG_DEG, e.g. lattices: a row
    // of four or five edges, usually one source per level) take the pull
    // kernels with the thread path; their grids are what stays resident
    // (the thread path costs registers), so no CTA waits for a second wave.
    // Denser graphs keep one warp per row at eight CTAs per SM.
    const bool tp = (int64_t)g->ne <= (int64_t)TP_AVG_DEG * g->nv;
    int occ_f = 8, occ_b = 8;
    if (tp) {
        if (a.ext) MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_f, k_bb_pull<true, true>, THREADS, 0));
        else MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_f, k_bb_pull<true, false>, THREADS, 0));
        if (a.ext) MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_b, k_bbb_pull<true, true>, THREADS, 0));
        else MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_b, k_bbb_pull<true, false>, THREADS, 0));
    }
    const int grid_f = launch_grid(g, THREADS, std::max(1, std::min(8, occ_f)));
    const int grid_b = launch_grid(g, THREADS, std::max(1, std::min(8, occ_b)));
    // low-degree graphs run their sparse levels in persistent sweeps, whose
    // grids are what stays resident
    if (tp && w->coop_f == 0) {
        int of = 0, ob = 0, ofx = 0, obx = 0;
        MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&of, k_bb_levels<true, false>, THREADS, 0));
        MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ofx, k_bb_levels<true, true>, THREADS, 0));
        MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ob, k_bbb_levels<true, false>, THREADS, 0));
        MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&obx, k_bbb_levels<true, true>, THREADS, 0));
        const int pf = std::min({of, ofx, 8}), pb = std::min({ob, obx, 8});
        if (pf < 1 || pb < 1) return fail(MG_ERR_CUDA, "persistent batched BC kernels do not fit on an SM");
        w->coop_f = pf * g->num_sms;
        w->coop_b = pb * g->num_sms;
    }
    const bool persist = tp;
    const int coop_f = w->coop_f, coop_b = w->coop_b;
    const int alpha = opt.alpha > 0 ? opt.alpha : 15;
    const int max_levels = g->nv + 2;
    // heavy-row folds only on graphs that have heavy rows
    const bool heavy = g->nhrows > 0;
    Profiler &P = g->prof;
    const int s_mark = P.slot("bcb_mark"), s_pull = P.slot("bcb_pull"), s_heavy = P.slot("bcb_heavy");
    const int s_comp = P.slot("bcb_compact_decide");
    const int s_bp = P.slot("bcb_back"), s_bh = P.slot("bcb_back_heavy"), s_bn = P.slot("bcb_back_next");
    const int s_lv = persist ? P.slot("bcb_levels") : -1, s_blv = persist ? P.slot("bcb_back_levels") : -1;
    BodyFn fwd = [&](cudaStream_t st, cudaGraphConditionalHandle h, int use_cond) -> mg_status {
        if (persist) {
            MG_CUDA(cudaMemsetAsync(a.pcnt, 0, 4 * sizeof(LvlCnt), st));
            P.begin(s_lv);
            if (a.ext) MG_TRY(launch_coop(k_bb_levels<true, true>, coop_f, st, a, (int)heavy));
            else MG_TRY(launch_coop(k_bb_levels<true, false>, coop_f, st, a, (int)heavy));
            P.end();
        }
        P.begin(s_mark);
        k_bb_mark<<<grid, THREADS, 0, st>>>(a);
        P.end();
        P.begin(s_pull);
        if (a.ext) {
            if (tp) MG_TRY(launch_pdl(k_bb_pull<true, true>, grid_f, THREADS, st, a));
            else MG_TRY(launch_pdl(k_bb_pull<false, true>, grid_f, THREADS, st, a));
        } else {
            if (tp) MG_TRY(launch_pdl(k_bb_pull<true, false>, grid_f, THREADS, st, a));
            else MG_TRY(launch_pdl(k_bb_pull<false, false>, grid_f, THREADS, st, a));
        }
        P.end();
        if (heavy) {
            P.begin(s_heavy);
            MG_TRY(launch_pdl(k_bb_heavy, grid, THREADS, st, a));
            P.end();
        }
        P.begin(s_comp);
        MG_TRY(launch_pdl(k_bb_compact, grid, THREADS, st, a, h, use_cond));
        P.end();
        MG_CUDA(cudaGetLastError());
        return MG_OK;
    };
    BodyFn bwd = [&](cudaStream_t st, cudaGraphConditionalHandle h, int use_cond) -> mg_status {
        P.begin(s_bp);
        if (a.ext) {
            if (tp) k_bbb_pull<true, true><<<grid_b, THREADS, 0, st>>>(a);
            else k_bbb_pull<false, true><<<grid_b, THREADS, 0, st>>>(a);
        } else {
            if (tp) k_bbb_pull<true, false><<<grid_b, THREADS, 0, st>>>(a);
            else k_bbb_pull<false, false><<<grid_b, THREADS, 0, st>>>(a);
        }
        P.end();
        if (heavy) {
            P.begin(s_bh);
            if (a.ext) MG_TRY(launch_pdl(k_bbb_heavy<true>, grid, THREADS, st, a));
            else MG_TRY(launch_pdl(k_bbb_heavy<false>, grid, THREADS, st, a));
            P.end();
        }
        P.begin(s_bn);
        MG_TRY(launch_pdl(k_bbb_next, grid, THREADS, st, a, h, use_cond));
        P.end();
        MG_CUDA(cudaGetLastError());
        return MG_OK;
    };
    // every by-value argument of the captured kernels
    const LoopKey key = LoopKey().add(a).add(grid).add(grid_f).add(grid_b).add(heavy).add(tp).add(coop_f);
    const LoopKey key_b = LoopKey(key).add(1);
    const int mode = opt.profile ? MG_EXEC_HOST : opt.exec;
    int32_t levels = 0, dense_levels = 0;
    for (int32_t g0 = 0; g0 < nsrc; g0 += W) {
        const int32_t cnt = std::min<int32_t>(W, nsrc - g0);
        MG_CUDA(cudaMemcpyAsync(w->src.p, src_engine + g0, (size_t)cnt * 4, cudaMemcpyHostToDevice, s));
        MG_CUDA(cudaMemsetAsync(a.vis, 0, n * 4, s));
        MG_CUDA(cudaMemsetAsync(a.fm0, 0, 3 * n * 4, s));
        MG_CUDA(cudaMemsetAsync(a.bar, 0, 64, s));
        k_bb_init<<<1, 32, 0, s>>>(a, cnt, opt.direction, alpha, max_levels);
        MG_CUDA(cudaGetLastError());
        MG_TRY(run_loop(mode, opt.profile != 0, s, w->fwd, key, fwd, &a.ctl->more, g->pinned_flag, max_levels + 2));
        k_bbb_start<<<grid, THREADS, 0, s>>>(a);
        MG_CUDA(cudaGetLastError());
        if (persist) {
            // every backward level in one launch (the barrier words again
            // from zero: this grid differs from the forward one)
            MG_CUDA(cudaMemsetAsync(a.bar, 0, 64, s));
            P.begin(s_blv);
            if (a.ext) MG_TRY(launch_coop(k_bbb_levels<true, true>, coop_b, s, a, (int)heavy));
            else MG_TRY(launch_coop(k_bbb_levels<true, false>, coop_b, s, a, (int)heavy));
            P.end();
        } else {
            MG_TRY(run_loop(mode, opt.profile != 0, s, w->bwd, key_b, bwd, &a.ctl->more, g->pinned_flag,
                            max_levels + 2));
        }
        BbCtl hc;
        MG_CUDA(cudaMemcpyAsync(&hc, a.ctl, sizeof(hc), cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaStreamSynchronize(s));
        if (hc.status == 1) return fail(MG_ERR_ITER_LIMIT, "batched BC: level cap %d reached", max_levels);
        if (hc.status == 3) return fail(MG_ERR_CUDA, "batched BC: grid barrier of a persistent sweep timed out");
        if (hc.status != 0) return fail(MG_ERR_CUDA, "batched BC: level archive overflow");
        if (hc.ovf && !g->bc_ext) {
            // a path count passed FP64's comfortable range: this graph's BC
            // runs use extended path counts from now on, starting over here
            g->bc_ext = true;
            return bc_batched(g, src_engine, nsrc, opt, info, bc_dev);
        }
        levels += hc.nlevels;
        dense_levels += hc.dense_levels;
    }
    k_bb_to_float<<<grid, THREADS, 0, s>>>(g->nv, a.bc, w->bcf.as<float>());
    MG_CUDA(cudaGetLastError());
    if (info) {
        info->iterations = levels;
        info->pull_iterations = dense_levels;
    }
    *bc_dev = w->bcf.as<float>();
    return MG_OK;
}

}  // namespace mgi
