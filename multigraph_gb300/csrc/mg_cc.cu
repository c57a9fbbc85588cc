// mg_cc.cu -- connected components and multi-graph batches.
//
// Replaces MultiGraph_E_E / ee_kernel (edge hooking with parity-alternating
// min/max, process.cu:969-999,1051-1077) and MultiGraph_V_V / vv_kernel
// (pointer jumping, process.cu:940-967,1012-1049) driven by main.cu:113-119,
// which return to the host after every hooking and jumping round.
//
// Here the edges are hooked in a lock-free union-find whose links always go
// from the larger root to the smaller one (parent[x] <= x), with path halving
// in find; a final pass compresses every vertex to its root.  The root of a
// component is therefore its minimum vertex id, which is exactly the
// canonical label the reference's validator derives
// (validate.cu:234-242,263-273), whatever order the unions run in.  Union
// retries only when another thread changed the same root, so every loop is
// lock-free and bounded by the number of successful links.
//
// Symmetric graphs skip most of the edges (neighbour sampling, as in
// Sutton et al., "Optimizing Parallel Graph Connectivity Computation via
// Subgraph Sampling", IPDPS 2018): every vertex first links to its first
// SAMPLE_ROUNDS neighbours (the trees compressed after each round), the most frequent root
// among 1024 sampled vertices is taken as the giant component, and only rows
// whose vertex is outside it hook their remaining edges (in both
// directions, so an edge with one end in the giant component is hooked from
// the other end).  General graphs hook every in-edge once.
//
// Multi-graph batches: the graphs are laid out as one disjoint union (vertex
// ids offset per graph), so one multi-source BFS and one CC pass cover the
// whole batch; per-graph results are the arena results minus the offsets.

#include "mg_device.cuh"
#include "mg_ops.cuh"

#include <algorithm>
#include <cstring>
#include <memory>

namespace {

constexpr int THREADS = 256;

__device__ __forceinline__ int32_t cc_find(volatile int32_t *parent, int32_t v)
{
    int32_t p = parent[v];
    while (p != v) {
        int32_t gp = parent[p];
        if (gp != p) parent[v] = gp;  // halving; benign race, keeps parent[v] <= v
        v = p;
        p = gp;
    }
    return v;
}

__device__ __forceinline__ void cc_union(int32_t *parent, int32_t a, int32_t b)
{
    volatile int32_t *vp = parent;
    for (;;) {
        a = cc_find(vp, a);
        b = cc_find(vp, b);
        if (!mgops::Cc::update_condition(a, b)) return;
        if (a < b) { int32_t t = a; a = b; b = t; }
        int32_t old = atomicCAS(&parent[a], a, b);  // link larger root under smaller
        if (old == a) return;
        a = old;
    }
}

constexpr int SAMPLE_ROUNDS = 2;
constexpr int MODE_SAMPLES = 1024;

// link_first: the first neighbour below v starts the tree (a valid link:
// parent < v); otherwise every vertex is its own tree
__global__ void k_cc_init(int32_t n, const int32_t *row, const int32_t *col, int32_t *parent, int link_first)
{
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        int32_t p = mgops::Cc::initialize(v);
        if (link_first && row[v + 1] > row[v]) p = min(p, col[row[v]]);
        parent[v] = p;
    }
}

// link every vertex to its r-th neighbour
__global__ void k_cc_sample(int32_t n, const int32_t *row, const int32_t *col, int32_t r, int32_t *parent);

// The most frequent root among MODE_SAMPLES vertices of one graph of a
// batch (block b samples caller ids [voff[b], voff[b+1]), the whole id range
// without voff; ties: smallest id) is marked in the giant-root bitmap.
// Graphs of a batch share no edges, so skipping the rows of every marked
// component stays exact: an edge leaving a marked component is hooked from
// its unmarked end.  One block of MODE_SAMPLES threads per graph.
__global__ void __launch_bounds__(MODE_SAMPLES) k_cc_mode(int32_t n, const int32_t *voff, const int32_t *old2new,
                                                          const int32_t *parent, uint32_t *giant_bm)
{
    __shared__ int32_t s_val[MODE_SAMPLES];
    __shared__ int32_t s_best[MODE_SAMPLES / 32], s_cnt[MODE_SAMPLES / 32];
    const int t = threadIdx.x;
    const int32_t lo = voff ? voff[blockIdx.x] : 0, hi = voff ? voff[blockIdx.x + 1] : n;
    const int32_t span = hi - lo;
    if (span <= 0) return;  // block-uniform
    // spread the samples over the id range
    int32_t v = lo + (int32_t)(((int64_t)t * span) / MODE_SAMPLES +
                               (((int64_t)t * 7919) % max(span / MODE_SAMPLES, 1)));
    v = min(max(v, lo), hi - 1);
    if (old2new) v = old2new[v];
    s_val[t] = parent[v];
    __syncthreads();
    const int32_t mine = s_val[t];
    int cnt = 0;
    for (int i = 0; i < MODE_SAMPLES; i++) cnt += (s_val[i] == mine);
    // block argmax of (cnt, -value)
    int32_t bv = mine;
    int bc = cnt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const int32_t ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oc = __shfl_xor_sync(0xffffffffu, bc, o);
        if (oc > bc || (oc == bc && ov < bv)) { bv = ov; bc = oc; }
    }
    if ((t & 31) == 0) { s_best[t >> 5] = bv; s_cnt[t >> 5] = bc; }
    __syncthreads();
    if (t == 0) {
        for (int w = 1; w < MODE_SAMPLES / 32; w++)
            if (s_cnt[w] > bc || (s_cnt[w] == bc && s_best[w] < bv)) { bv = s_best[w]; bc = s_cnt[w]; }
        mgd::bm_set(giant_bm, bv);
    }
}

__global__ void k_cc_sample(int32_t n, const int32_t *row, const int32_t *col, int32_t r, int32_t *parent)
{
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int32_t b = row[v];
        if (row[v + 1] - b > r) {
            const int32_t u = col[b + r];
            if (u != v) cc_union(parent, v, u);
        }
    }
}

// per-edge union over the degree-binned rows (bins_reduce interface;
// the reduction value is unused).  With giant_bm: rows whose vertex points
// at a marked giant root are skipped and the others hook every entry;
// without: every row, each undirected edge once when symmetric.
struct HookOp {
    using T = int;
    static constexpr bool kRowAware = true;  // the union needs the row (source vertex)
    static constexpr bool kWeights = false;
    int32_t *parent;
    int symmetric;
    const uint32_t *giant_bm;
    __device__ int identity() const { return 0; }
    __device__ bool skip(int32_t v) const { return giant_bm && mgd::bm_test(giant_bm, parent[v]); }
    __device__ int edge(int32_t, int32_t src, int32_t dst, int32_t) const
    {
        if (src != dst && (giant_bm || !symmetric || dst < src)) cc_union(parent, src, dst);
        return 0;
    }
    __device__ int combine(int, int) const { return 0; }
    __device__ void flush() {}
    __device__ void finish(int32_t, int) {}
};

// one pass over the pull-side arrays; symmetric graphs take each undirected
// edge once (u > v), general graphs every entry
__global__ void __launch_bounds__(THREADS) k_cc_hook(int32_t n, const int32_t *prow, const int32_t *pcol,
                                                     const int32_t *wrows, int32_t nwrows, int32_t nwlong, const int32_t *trows,
                                                     int32_t ntrows, const int32_t *hchunk, int32_t nhchunks,
                                                     int symmetric, const uint32_t *giant_bm, int32_t *parent)
{
    HookOp op{parent, symmetric, giant_bm};
    mgd::bins_reduce(op, prow, pcol, nullptr, wrows, nwrows, nwlong, trows, ntrows);
    __shared__ int s_skip;
    for (int32_t ch = blockIdx.x; ch < nhchunks; ch += gridDim.x) {
        int32_t u = hchunk[3 * ch], b = hchunk[3 * ch + 1], e = hchunk[3 * ch + 2];
        // one thread decides for the block (parent[u] may change meanwhile)
        if (threadIdx.x == 0) s_skip = op.skip(u);
        __syncthreads();
        const bool skip = s_skip;
        __syncthreads();
        if (skip) continue;
        for (int32_t p = b + threadIdx.x; p < e; p += blockDim.x) op.edge(p, u, __ldcs(&pcol[p]), 0);
    }
}

__global__ void k_cc_compress(int32_t n, int32_t *parent)
{
    volatile int32_t *vp = parent;
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        int32_t r = cc_find(vp, v);
        parent[v] = r;
    }
}

}  // namespace

struct CcWS {
    mgi::DevBuf parent, giant, voff;
};

namespace mgi {

void free_cc_ws(mg_graph *g)
{
    if (!g->cws) return;
    dev_free(g->cws->parent);
    dev_free(g->cws->giant);
    dev_free(g->cws->voff);
    delete g->cws;
    g->cws = nullptr;
}

// CC of the graph, or of a batch arena whose graphs occupy the caller-id
// ranges voff[0..ngraphs] (one giant component per graph)
mg_status cc_run(mg_graph *g, mg_run_info *info, const std::vector<int32_t> *voff = nullptr)
{
    if (!g->cws) g->cws = new CcWS();
    const size_t words = ((size_t)std::max(g->nv, 1) + 31) / 32;
    MG_TRY(dev_alloc(g->cws->parent, (size_t)std::max(g->nv, 1) * 4));
    MG_TRY(dev_alloc(g->cws->giant, words * 4));
    int32_t *parent = g->cws->parent.as<int32_t>();
    uint32_t *giant = g->cws->giant.as<uint32_t>();
    cudaStream_t s = g->stream;
    int ngraphs = 1;
    const int32_t *voff_dev = nullptr;
    if (voff && voff->size() > 2) {
        ngraphs = (int)voff->size() - 1;
        MG_TRY(dev_alloc(g->cws->voff, voff->size() * 4));
        MG_CUDA(cudaMemcpyAsync(g->cws->voff.p, voff->data(), voff->size() * 4, cudaMemcpyHostToDevice, s));
        voff_dev = g->cws->voff.as<int32_t>();
    }
    if (g->nv == 0) return MG_OK;
    const int grid = launch_grid(g, THREADS, 8);
    Profiler &P = g->prof;
    const int si = P.slot("cc_init"), sh = P.slot("cc_hook"), sc = P.slot("cc_compress");
    const bool sample = g->symmetric;
    P.begin(si);
    k_cc_init<<<grid, THREADS, 0, s>>>(g->nv, g->trow, g->tcol, parent, sample ? 0 : 1);
    P.end();
    if (sample) {
        // singleton trees, then each sampling round links every vertex to
        // its r-th neighbour and flattens the trees again, so no find walks
        // a long chain (a lattice's first neighbours would chain rows)
        const int ss = P.slot("cc_sample"), sm = P.slot("cc_mode");
        for (int r = 0; r < SAMPLE_ROUNDS; r++) {
            P.begin(ss);
            k_cc_sample<<<grid, THREADS, 0, s>>>(g->nv, g->trow, g->tcol, r, parent);
            P.end();
            P.begin(sc);
            k_cc_compress<<<grid, THREADS, 0, s>>>(g->nv, parent);
            P.end();
        }
        MG_CUDA(cudaMemsetAsync(giant, 0, words * 4, s));
        P.begin(sm);
        k_cc_mode<<<ngraphs, MODE_SAMPLES, 0, s>>>(g->nv, voff_dev, g->relabeled ? g->old2new.as<int32_t>() : nullptr,
                                                    parent, giant);
        P.end();
    }
    P.begin(sh);
    k_cc_hook<<<grid, THREADS, 0, s>>>(g->nv, g->trow, g->tcol, g->wrows.as<int32_t>(), g->nwrows, g->nwlong,
                                       g->trows.as<int32_t>(), g->ntrows, g->hchunk.as<int32_t>(), g->nhchunks,
                                       g->symmetric ? 1 : 0, sample ? giant : nullptr, parent);
    P.end();
    P.begin(sc);
    k_cc_compress<<<grid, THREADS, 0, s>>>(g->nv, parent);
    P.end();
    MG_CUDA(cudaGetLastError());
    if (info) {
        info->iterations = 1;
        info->edges_scanned = g->ne;
    }
    return MG_OK;
}

mg_status frontier_bfs_multi(mg_graph *g, const int32_t *srcs_host, int32_t nsrc, const mg_opts &opt,
                             mg_run_info *info);
const void *frontier_label(mg_graph *g);

}  // namespace mgi

using namespace mgi;

struct mg_batch {
    mg_graph *dg = nullptr;
    std::vector<int32_t> voff;  // vertex offset of each graph (+ total)
    std::vector<int32_t> local_nv;
};

extern "C" {

mg_status mg_cc(mg_graph *g, const mg_opts *o, int32_t *label_out, mg_run_info *info)
{
    mg_opts opt;
    MG_TRY(begin_run(g, o, opt, info));
    MG_TRY(cc_run(g, info));
    MG_TRY(cc_to_caller(g, g->cws->parent.as<int32_t>(), &g->res[MG_RES_LABEL]));
    MG_TRY(end_run(g, opt, info));
    return copy_out(g, label_out, g->res[MG_RES_LABEL], (size_t)g->nv * 4);
}

mg_status mg_batch_create(const mg_host_graph *const *graphs, int32_t count, int32_t device, mg_batch **out)
{
    clear_error();
    if (!graphs || !out || count <= 0) return fail(MG_ERR_INVALID, "invalid argument");
    *out = nullptr;
    int64_t nv = 0, ne = 0;
    for (int32_t i = 0; i < count; i++) {
        if (!graphs[i]) return fail(MG_ERR_INVALID, "null graph %d", i);
        nv += graphs[i]->nv;
        ne += graphs[i]->ne;
    }
    if (nv >= INT32_MAX || ne >= INT32_MAX) return fail(MG_ERR_RANGE, "batch too large for int32 ids");
    mg_host_graph arena;
    arena.nv = (int32_t)nv;
    arena.ne = (int32_t)ne;
    arena.v.resize((size_t)nv + 1);
    arena.e.resize((size_t)ne);
    arena.ev.resize((size_t)ne);
    std::unique_ptr<mg_batch> b(new mg_batch());
    int32_t vo = 0, eo = 0;
    for (int32_t i = 0; i < count; i++) {
        const mg_host_graph *h = graphs[i];
        b->voff.push_back(vo);
        b->local_nv.push_back(h->nv);
        for (int32_t v = 0; v < h->nv; v++) arena.v[vo + v] = eo + h->v[v];
        for (int32_t p = 0; p < h->ne; p++) {
            arena.e[eo + p] = vo + h->e[p];
            arena.ev[eo + p] = h->ev[p];
        }
        vo += h->nv;
        eo += h->ne;
    }
    arena.v[nv] = (int32_t)ne;
    b->voff.push_back(vo);
    MG_TRY(mg_graph_upload(&arena, device, &b->dg));
    *out = b.release();
    return MG_OK;
}

void mg_batch_free(mg_batch *b)
{
    if (!b) return;
    mg_graph_free(b->dg);
    delete b;
}

mg_status mg_batch_bfs(mg_batch *b, const int32_t *sources, const mg_opts *o, int32_t *levels_out, mg_run_info *info)
{
    clear_error();
    if (!b || !sources) return fail(MG_ERR_INVALID, "invalid argument");
    std::vector<int32_t> srcs(b->local_nv.size());
    for (size_t i = 0; i < srcs.size(); i++) {
        if (sources[i] < 0 || sources[i] >= b->local_nv[i])
            return fail(MG_ERR_RANGE, "source %d of graph %zu out of range", sources[i], i);
        srcs[i] = to_engine(b->dg, b->voff[i] + sources[i]);
    }
    mg_graph *g = b->dg;
    mg_opts opt;
    MG_TRY(begin_run(g, o, opt, info));
    MG_TRY(frontier_bfs_multi(g, srcs.data(), (int32_t)srcs.size(), opt, info));
    MG_TRY(to_caller(g, MG_RES_LEVEL, frontier_label(g), 4, 1, &g->res[MG_RES_LEVEL]));
    MG_TRY(end_run(g, opt, info));
    return copy_out(g, levels_out, g->res[MG_RES_LEVEL], (size_t)g->nv * 4);
}

mg_status mg_batch_cc(mg_batch *b, const mg_opts *o, int32_t *labels_out, mg_run_info *info)
{
    clear_error();
    if (!b) return fail(MG_ERR_INVALID, "invalid argument");
    mg_graph *g = b->dg;
    mg_opts opt;
    MG_TRY(begin_run(g, o, opt, info));
    MG_TRY(cc_run(g, info, &b->voff));
    MG_TRY(cc_to_caller(g, g->cws->parent.as<int32_t>(), &g->res[MG_RES_LABEL]));
    MG_TRY(end_run(g, opt, info));
    if (!labels_out) return MG_OK;
    MG_TRY(copy_out(g, labels_out, g->res[MG_RES_LABEL], (size_t)g->nv * 4));
    for (size_t i = 0; i + 1 < b->voff.size(); i++)
        for (int32_t v = b->voff[i]; v < b->voff[i + 1]; v++) labels_out[v] -= b->voff[i];
    return MG_OK;
}

}  // extern "C"
