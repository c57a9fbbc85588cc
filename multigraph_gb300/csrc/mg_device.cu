// mg_device.cu -- device graph upload and the shared run machinery.
//
// mg_graph_upload replaces the reference's generate_MultiGraph
// (gen_structure.cu:2230-2947).  The reference builds a 2-D tiled layout
// (16-bit sparse-tile streams sp1/sp2, dense tiles, an intermediate buffer
// i1 written and re-read every dense iteration, ~12.5 B/edge) sized for
// Kepler's 48 KB shared memory.  On GB300 the whole pull-side gather vector
// of these graphs (n*4 B, <= 67 MB) stays in the 129 MB L2, so the layout here
// is the CSR itself, renumbered hub-first when the degrees are skewed (the
// engine-order CSR is rebuilt on the device from the caller's CSR), plus
// small index tables that balance the pull kernels:
//   wrows / trows : degree bins -- rows of tbin+1..heavy_deg in-edges (a warp
//                   each) and rows of <= tbin in-edges (a thread each);
//   hchunk        : rows with in-degree > heavy_deg split into chunk-edge
//                   pieces, processed by whole CTAs, combined in a fixed order.
// heavy_deg / chunk / tbin start at HEAVY_DEG / HCHUNK / TBIN and are
// re-chosen per graph by mg_autotune(MG_ALGO_PR).  A transposed copy is
// built only when the graph is not symmetric.

#include "mg_device.cuh"

#include <algorithm>
#include <utility>
#include <cstring>
#include <memory>

namespace mgi {

constexpr int32_t HEAVY_DEG = 512;                // pull rows above this take the CTA-chunk path
constexpr int32_t HCHUNK = 2048;                  // = 8 edges x 256 threads of a chunk CTA
constexpr int32_t TBIN = 32;                      // rows up to this in-degree take a thread each
// column / weight arrays carry this many bytes of tail padding past m
// entries (defensive: a kernel that rounds a last read up stays inside the
// allocation)
constexpr size_t COL_PAD = 16;

mg_status dev_alloc(DevBuf &b, size_t bytes)
{
    if (b.p && b.bytes >= bytes) return MG_OK;
    dev_free(b);
    if (bytes == 0) bytes = 16;
    if (inject_alloc_failure()) return fail(MG_ERR_OOM, "device allocation of %zu bytes failed (injected)", bytes);
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        b.p = nullptr;
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? MG_ERR_OOM : MG_ERR_CUDA, "cudaMalloc(%zu): %s", bytes,
                    cudaGetErrorString(e));
    }
    b.bytes = bytes;
    return MG_OK;
}

void dev_free(DevBuf &b)
{
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

// ---------------------------------------------------------------------------
void Profiler::reset(cudaStream_t s, bool enable)
{
    stream = s;
    on = enable;
    slots.clear();
    pending.clear();
    used = 0;
    open_slot = -1;
}

int Profiler::slot(const char *name)
{
    for (size_t i = 0; i < slots.size(); i++)
        if (slots[i].name == name) return (int)i;
    slots.push_back(Slot{name, 0, 0.0});
    return (int)slots.size() - 1;
}

void Profiler::begin(int slot_id)
{
    if (!on) return;
    if (used == pool.size()) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        pool.push_back({a, b});
    }
    cudaEventRecord(pool[used].first, stream);
    open_slot = slot_id;
}

void Profiler::end()
{
    if (!on || open_slot < 0) return;
    cudaEventRecord(pool[used].second, stream);
    pending.push_back({open_slot, used});
    used++;
    open_slot = -1;
}

mg_status Profiler::collect(mg_run_info *info)
{
    if (!on) return MG_OK;
    for (auto &p : pending) {
        float ms = 0.f;
        MG_CUDA(cudaEventElapsedTime(&ms, pool[p.ev].first, pool[p.ev].second));
        slots[p.slot].launches++;
        slots[p.slot].ms += ms;
    }
    pending.clear();
    used = 0;
    if (info) {
        info->nkernels = (int32_t)std::min<size_t>(slots.size(), MG_PROFILE_SLOTS);
        for (int i = 0; i < info->nkernels; i++) {
            std::snprintf(info->kernels[i].name, sizeof(info->kernels[i].name), "%s", slots[i].name.c_str());
            info->kernels[i].launches = slots[i].launches;
            info->kernels[i].total_ms = slots[i].ms;
        }
    }
    return MG_OK;
}

Profiler::~Profiler()
{
    for (auto &p : pool) { cudaEventDestroy(p.first); cudaEventDestroy(p.second); }
}

// ---------------------------------------------------------------------------
void LoopGraph::destroy()
{
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    key.clear();
}

mg_status run_loop(int exec_mode, bool profile, cudaStream_t stream, LoopGraph &lg, const LoopKey &key, const BodyFn &body,
                   const int32_t *more_dev, int32_t *more_host, int max_host_iters)
{
    if (exec_mode == MG_EXEC_GRAPH && !profile) {
        if (!lg.exec || lg.key != key.bytes) {
            lg.destroy();
            cudaGraph_t g;
            MG_CUDA(cudaGraphCreate(&g, 0));
            cudaGraphConditionalHandle h;
            cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
            if (e != cudaSuccess) { cudaGraphDestroy(g); MG_CUDA(e); }
            cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
            p.conditional.handle = h;
            p.conditional.type = cudaGraphCondTypeWhile;
            p.conditional.size = 1;
            cudaGraphNode_t node;
            e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p);
            if (e != cudaSuccess) { cudaGraphDestroy(g); MG_CUDA(e); }
            cudaGraph_t bodyg = p.conditional.phGraph_out[0];
            e = cudaStreamBeginCaptureToGraph(stream, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) { cudaGraphDestroy(g); MG_CUDA(e); }
            mg_status s = body(stream, h, 1);
            cudaGraph_t captured = nullptr;
            e = cudaStreamEndCapture(stream, &captured);
            if (s != MG_OK) { cudaGraphDestroy(g); return s; }
            if (e != cudaSuccess) { cudaGraphDestroy(g); MG_CUDA(e); }
            cudaGraphExec_t ex;
            e = cudaGraphInstantiate(&ex, g, 0);
            if (e != cudaSuccess) { cudaGraphDestroy(g); MG_CUDA(e); }
            lg.graph = g;
            lg.exec = ex;
            lg.key = key.bytes;
        }
        MG_CUDA(cudaGraphLaunch(lg.exec, stream));
        return MG_OK;
    }
    // host-driven loop: one readback of the continue flag per iteration
    for (int it = 0; it < max_host_iters; it++) {
        MG_TRY(body(stream, 0, 0));
        MG_CUDA(cudaMemcpyAsync(more_host, more_dev, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
        MG_CUDA(cudaStreamSynchronize(stream));
        if (*more_host == 0) return MG_OK;
    }
    return MG_OK;
}

int launch_grid(const mg_graph *g, int threads, int per_sm)
{
    (void)threads;
    return g->num_sms * per_sm;
}

mg_status copy_out(mg_graph *g, void *host, const void *dev, size_t bytes)
{
    if (!host || bytes == 0) return MG_OK;
    MG_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, g->stream));
    MG_CUDA(cudaStreamSynchronize(g->stream));
    return MG_OK;
}

mg_status begin_run(mg_graph *g, const mg_opts *o, mg_opts &opt, mg_run_info *info)
{
    clear_error();
    if (!g) return fail(MG_ERR_INVALID, "null graph");
    if (o) opt = *o; else mg_opts_default(&opt);
    if (info) std::memset(info, 0, sizeof(*info));
    MG_CUDA(cudaSetDevice(g->device));
    g->prof.reset(g->stream, opt.profile != 0);
    MG_CUDA(cudaEventRecord(g->ev0, g->stream));
    return MG_OK;
}

mg_status end_run(mg_graph *g, const mg_opts &opt, mg_run_info *info)
{
    (void)opt;
    MG_CUDA(cudaEventRecord(g->ev1, g->stream));
    MG_CUDA(cudaEventSynchronize(g->ev1));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(MG_ERR_CUDA, "kernel error: %s", cudaGetErrorString(e));
    if (info) {
        float ms = 0.f;
        MG_CUDA(cudaEventElapsedTime(&ms, g->ev0, g->ev1));
        info->device_ms = ms;
    }
    return g->prof.collect(info);
}

}  // namespace mgi

using namespace mgi;

// ---------------------------------------------------------------------------
// layout building (host side, O(n + m))
// ---------------------------------------------------------------------------
struct HostLayout {
    std::vector<int32_t> trow, tcol, twt;  // transpose in engine ids (empty when symmetric)
    bool symmetric = true, wsym = true;
    std::vector<int32_t> hchunk, hrows, hrow_chunk;
    std::vector<int32_t> wrows, trows;  // degree bins (engine ids)
    int32_t nwlong = 0;                  // wrows[0, nwlong): rows of SUBWARP_MAX+ edges
    std::vector<int32_t> prow;          // pull-side row offsets (engine order)
    int32_t heavy = 0, chunk = 0, tbin = 0;
    int32_t n_dangling = 0, min_weight = 0;
    // hub-first relabeling (engine id = rank by descending log2 out-degree)
    bool relabel = false;
    std::vector<int32_t> new2old, old2new, row_new;
};

// Hub-first order: vertices grouped by floor(log2(out-degree)), largest
// group first, caller order kept inside a group (counting sort, O(n)).  The
// reference reorders by degree groups when some degree reaches 128
// (read_input.cu:169 sets `tra`, gen_structure.cu:2435-2556 builds _itable);
// the same trigger is used here.  Hubs then sit at the lowest ids, so the
// gathered values of the most frequently read sources share cache lines.
static void hub_first_order(const mg_host_graph &h, std::vector<int32_t> &new2old, std::vector<int32_t> &old2new)
{
    const int32_t n = h.nv;
    auto bucket = [&](int32_t v) {
        int32_t d = h.v[v + 1] - h.v[v];
        int b = 0;
        while (d > 1) { d >>= 1; b++; }
        return 31 - b;  // descending degree -> ascending key
    };
    std::vector<int32_t> cnt(33, 0);
    for (int32_t v = 0; v < n; v++) cnt[bucket(v) + 1]++;
    for (int i = 0; i < 32; i++) cnt[i + 1] += cnt[i];
    new2old.resize(n);
    old2new.resize(n);
    for (int32_t v = 0; v < n; v++) {
        int32_t p = cnt[bucket(v)]++;
        new2old[p] = v;
        old2new[v] = p;
    }
}

// Degree bins and heavy chunks of the pull rows (row offsets prow, engine
// order): rows above `heavy` in-edges are cut into `chunk`-edge pieces,
// rows of tbin+1..heavy go to the warp bin, the rest to the thread bin.
static void build_bins(const std::vector<int32_t> &prow, int32_t n, int32_t heavy, int32_t chunk, int32_t tbin,
                       HostLayout &L)
{
    L.hchunk.clear();
    L.hrows.clear();
    L.hrow_chunk.assign(1, 0);
    L.wrows.clear();
    L.trows.clear();
    for (int32_t v = 0; v < n; v++) {
        int32_t d = prow[v + 1] - prow[v];
        if (d > heavy) {
            L.hrows.push_back(v);
            for (int32_t b = prow[v]; b < prow[v + 1]; b += chunk) {
                L.hchunk.push_back(v);
                L.hchunk.push_back(b);
                L.hchunk.push_back(std::min(prow[v + 1], b + chunk));
            }
            L.hrow_chunk.push_back((int32_t)(L.hchunk.size() / 3));
        } else if (d > tbin) {
            L.wrows.push_back(v);
        } else {
            L.trows.push_back(v);
        }
    }
    // warp-bin rows of SUBWARP_MAX or more edges first (a warp each), the
    // shorter ones after them (an 8-lane group each); order kept in each part
    std::stable_partition(L.wrows.begin(), L.wrows.end(),
                          [&](int32_t v) { return prow[v + 1] - prow[v] >= mgd::SUBWARP_MAX; });
    L.nwlong = 0;
    for (int32_t v : L.wrows)
        if (prow[v + 1] - prow[v] >= mgd::SUBWARP_MAX) L.nwlong++;
    L.heavy = heavy;
    L.chunk = chunk;
    L.tbin = tbin;
}

static void build_layout(const mg_host_graph &h, HostLayout &L, int32_t heavy = HEAVY_DEG, int32_t chunk = HCHUNK,
                         int32_t tbin = TBIN)
{
    const int32_t n = h.nv, m = h.ne;
    bool skewed = false;
    for (int32_t v = 0; v < n && !skewed; v++) skewed = (h.v[v + 1] - h.v[v] >= 128);
    L.relabel = skewed;
    if (L.relabel) {
        hub_first_order(h, L.new2old, L.old2new);
        L.row_new.assign(n + 1, 0);
        for (int32_t i = 0; i < n; i++) L.row_new[i + 1] = L.row_new[i] + (h.v[L.new2old[i] + 1] - h.v[L.new2old[i]]);
    }
    // transpose by counting sort (rows come out with ascending columns)
    std::vector<int32_t> tr(n + 1, 0), tc(m), tw(m);
    for (int32_t i = 0; i < m; i++) tr[h.e[i] + 1]++;
    for (int32_t i = 0; i < n; i++) tr[i + 1] += tr[i];
    {
        std::vector<int32_t> pos(tr.begin(), tr.end() - 1);
        for (int32_t u = 0; u < n; u++)
            for (int32_t p = h.v[u]; p < h.v[u + 1]; p++) {
                int32_t q = pos[h.e[p]]++;
                tc[q] = u;
                tw[q] = h.ev[p];
            }
    }
    L.symmetric = std::equal(tr.begin(), tr.end(), h.v.begin()) && std::equal(tc.begin(), tc.end(), h.e.begin());
    L.wsym = L.symmetric && std::equal(tw.begin(), tw.end(), h.ev.begin());
    if (!L.symmetric || !L.wsym) {
        if (L.relabel) {
            // transpose in engine ids: row i' = transpose row new2old[i'], columns mapped
            L.trow.assign(n + 1, 0);
            for (int32_t i = 0; i < n; i++) L.trow[i + 1] = L.trow[i] + (tr[L.new2old[i] + 1] - tr[L.new2old[i]]);
            L.tcol.resize(m);
            L.twt.resize(m);
            for (int32_t i = 0; i < n; i++) {
                int32_t u = L.new2old[i], o = L.trow[i];
                for (int32_t p = tr[u]; p < tr[u + 1]; p++, o++) { L.tcol[o] = L.old2new[tc[p]]; L.twt[o] = tw[p]; }
            }
        } else {
            L.trow.swap(tr); L.tcol.swap(tc); L.twt.swap(tw);
        }
    }
    const std::vector<int32_t> &prow = (!L.symmetric || !L.wsym) ? L.trow : (L.relabel ? L.row_new : h.v);
    L.n_dangling = 0;
    for (int32_t v = 0; v < n; v++) L.n_dangling += (h.v[v + 1] == h.v[v]);
    L.min_weight = m ? *std::min_element(h.ev.begin(), h.ev.end()) : 0;
    L.prow = prow;
    build_bins(prow, n, heavy, chunk, tbin, L);
}

// Engine row i of the relabeled CSR is caller row new2old[i] with the same
// entry order, so engine position p (in row r, offset p - row_new[r])
// corresponds to caller position o_row[new2old[r]] + p - row_new[r].
//
// pos_row[k] = engine row of position min(32k, m-1), built once per upload.
// A warp handles 32 consecutive positions [32c, 32c+32): their rows lie in
// [pos_row[c], pos_row[c+1]], so when that span is under 32 rows each lane
// finds its row in one coalesced load of the span's row starts and five
// shuffles; wider spans (runs of empty rows) fall back to a binary search.
// Four such 32-position steps are interleaved per warp for memory-level
// parallelism.
__device__ __forceinline__ int32_t row_of_position(const int32_t *row_new, int32_t p, int32_t lo, int32_t hi)
{
    // last r in [lo, hi] with row_new[r] <= p
    while (lo < hi) {
        const int32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(&row_new[mid]) <= p) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void k_pos_rows(int32_t n, int32_t m, const int32_t *row_new, int32_t *pos_row)
{
    const int32_t nk = m / 32 + 2;
    for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nk; k += gridDim.x * blockDim.x) {
        const int32_t p = (int32_t)min((int64_t)k * 32, (int64_t)m - 1);
        pos_row[k] = row_of_position(row_new, p, 0, n - 1);
    }
}

constexpr int RELABEL_ILP = 4;

// engine row rr and its start st of this lane's position 32c + lane, for
// RELABEL_ILP consecutive 32-position steps from c0
__device__ __forceinline__ void engine_rows(int32_t m, const int32_t *row_new, const int32_t *pos_row, int32_t c0,
                                            int32_t (&rr)[RELABEL_ILP], int32_t (&st)[RELABEL_ILP])
{
    const int lane = threadIdx.x & 31;
    int32_t ra[RELABEL_ILP], rb[RELABEL_ILP], w[RELABEL_ILP];
    const int32_t nsteps = (m + 31) / 32;
#pragma unroll
    for (int j = 0; j < RELABEL_ILP; j++) {
        const int32_t c = min(c0 + j, nsteps - 1);
        ra[j] = __ldg(&pos_row[c]);
        rb[j] = __ldg(&pos_row[c + 1]);
    }
#pragma unroll
    for (int j = 0; j < RELABEL_ILP; j++)
        w[j] = (ra[j] + lane <= rb[j]) ? __ldg(&row_new[ra[j] + lane]) : 0x7fffffff;
#pragma unroll
    for (int j = 0; j < RELABEL_ILP; j++) {
        const int32_t p = (c0 + j) * 32 + lane;
        if (rb[j] - ra[j] < 32) {
            const int o = mgd::owner_lane(w[j], p);
            rr[j] = ra[j] + o;
            st[j] = __shfl_sync(0xffffffffu, w[j], o);
        } else {
            rr[j] = row_of_position(row_new, min(p, m - 1), ra[j], rb[j]);
            st[j] = __ldg(&row_new[rr[j]]);
        }
    }
}

// Caller position of every engine position (once per layout): engine row
// r holds caller row new2old[r]'s edges in caller order, so position p of
// row r comes from o_row[new2old[r]] + (p - row_new[r]).
__global__ void k_caller_pos(int32_t m, const int32_t *new2old, const int32_t *o_row, const int32_t *row_new,
                             const int32_t *pos_row, int32_t *cpos)
{
    const int lane = threadIdx.x & 31;
    const int32_t nsteps = (m + 31) / 32;
    const int32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int32_t c0 = gwarp * RELABEL_ILP; c0 < nsteps; c0 += nwarps * RELABEL_ILP) {
        int32_t rr[RELABEL_ILP], st[RELABEL_ILP];
        engine_rows(m, row_new, pos_row, c0, rr, st);
#pragma unroll
        for (int j = 0; j < RELABEL_ILP; j++) rr[j] = __ldg(&new2old[rr[j]]);
#pragma unroll
        for (int j = 0; j < RELABEL_ILP; j++) {
            const int32_t p = (c0 + j) * 32 + lane;
            if (c0 + j < nsteps && p < m) cpos[p] = __ldg(&o_row[rr[j]]) + (p - st[j]);
        }
    }
}

// Symmetry checksum of an edge (u -> v, weight w): the hash of the
// undirected pair (min, max, w), added to sums[0] when u < v and to sums[1]
// when u > v.  A graph whose every edge has a reverse edge of the same
// weight gives equal sums; a missing reverse edge or a different weight
// makes them differ except with probability about 2^-64.
__device__ __forceinline__ unsigned long long pair_hash(uint32_t a, uint32_t b, uint32_t w)
{
    unsigned long long z = ((unsigned long long)a << 32 | b) + 0x9E3779B97F4A7C15ull * (w + 1ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ void sym_add(unsigned long long &s_lo, unsigned long long &s_hi, int32_t u, int32_t v,
                                        uint32_t w)
{
    if (u < v) s_lo += pair_hash((uint32_t)u, (uint32_t)v, w);
    else if (u > v) s_hi += pair_hash((uint32_t)v, (uint32_t)u, w);
}

__device__ __forceinline__ void sym_flush(unsigned long long *sums, unsigned long long s_lo, unsigned long long s_hi)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s_lo += __shfl_xor_sync(0xffffffffu, s_lo, o);
        s_hi += __shfl_xor_sync(0xffffffffu, s_hi, o);
    }
    if ((threadIdx.x & 31) == 0 && (s_lo | s_hi)) {
        atomicAdd(&sums[0], s_lo);
        atomicAdd(&sums[1], s_hi);
    }
}

// least edge weight of a staged input, kept in sums[3] as w + 2^31 (so an
// unsigned atomicMin orders signed weights); sums[3] starts at all ones
__device__ __forceinline__ void wmin_flush(unsigned long long *enc, int32_t w)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w = min(w, __shfl_xor_sync(0xffffffffu, w, o));
    if ((threadIdx.x & 31) == 0 && w != INT32_MAX) atomicMin(enc, (unsigned long long)((long long)w - INT32_MIN));
}

static int32_t wmin_decode(unsigned long long enc)
{
    return enc == ~0ull ? 0 : (int32_t)((long long)enc + INT32_MIN);
}

// caller CSR -> engine CSR for up to two 4-byte edge arrays through the
// caller-position table; the first is mapped through old2new when map_ids
// (column ids).  kSums: the symmetry checksum of (engine row, engine column,
// second array) is formed on the way (the relabel is a bijection, so the
// engine graph is symmetric exactly when the caller's is), the least
// second-array value (the weights) in sums[3], and sums[4] != 0 when some
// engine column id differs from the one it replaces.  A non-zero *skip
// (caller row offsets that differ from the layout's, found by
// k_rows_differ earlier on the stream) returns at once: the positions would
// not match the staged arrays.  Every load of a step is issued before its
// stores; the only dependent load is the old2new gather.
template <bool kSums>
__global__ void __launch_bounds__(256) k_relabel_edges(int32_t m, const int32_t *__restrict__ old2new,
                                                       const int32_t *__restrict__ row_new,
                                                       const int32_t *__restrict__ pos_row,
                                                       const int32_t *__restrict__ cpos,
                                                       const uint32_t *__restrict__ src0, uint32_t *__restrict__ dst0,
                                                       const uint32_t *__restrict__ src1, uint32_t *__restrict__ dst1,
                                                       int map_ids, unsigned long long *sums,
                                                       const unsigned long long *skip)
{
    if (kSums && skip && __ldcg(skip) != 0ull) return;
    const int lane = threadIdx.x & 31;
    const int32_t nsteps = (m + 31) / 32;
    const int32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    unsigned long long s_lo = 0, s_hi = 0;
    int32_t wlo = INT32_MAX;
    int changed = 0;
    for (int32_t c0 = gwarp * RELABEL_ILP; c0 < nsteps; c0 += nwarps * RELABEL_ILP) {
        int32_t q[RELABEL_ILP], rr[RELABEL_ILP], st[RELABEL_ILP];
        uint32_t x[RELABEL_ILP], y[RELABEL_ILP], old[RELABEL_ILP];
#pragma unroll
        for (int j = 0; j < RELABEL_ILP; j++) {
            const int32_t p = (c0 + j) * 32 + lane;
            q[j] = (c0 + j < nsteps && p < m) ? __ldcs(&cpos[p]) : -1;
        }
        if (kSums) engine_rows(m, row_new, pos_row, c0, rr, st);
#pragma unroll
        for (int j = 0; j < RELABEL_ILP; j++) {
            const int32_t p = (c0 + j) * 32 + lane;
            x[j] = q[j] >= 0 ? __ldcs(&src0[q[j]]) : 0u;
            y[j] = (q[j] >= 0 && dst1) ? __ldcs(&src1[q[j]]) : 0u;
            old[j] = (kSums && q[j] >= 0) ? __ldcs(&dst0[p]) : 0u;
        }
#pragma unroll
        for (int j = 0; j < RELABEL_ILP; j++)
            if (q[j] >= 0 && map_ids) x[j] = (uint32_t)__ldg(&old2new[x[j]]);
        if (kSums) {
#pragma unroll
            for (int j = 0; j < RELABEL_ILP; j++)
                if (q[j] >= 0) {
                    sym_add(s_lo, s_hi, rr[j], (int32_t)x[j], y[j]);
                    if (dst1) wlo = min(wlo, (int32_t)y[j]);
                    changed |= old[j] != x[j];
                }
        }
#pragma unroll
        for (int j = 0; j < RELABEL_ILP; j++) {
            if (q[j] < 0) continue;
            const int32_t p = (c0 + j) * 32 + lane;
            __stcs(&dst0[p], x[j]);
            if (dst1) __stcs(&dst1[p], y[j]);
        }
    }
    if (kSums) {
        sym_flush(sums, s_lo, s_hi);
        wmin_flush(&sums[3], wlo);
        if (__any_sync(0xffffffffu, changed) && lane == 0) atomicOr(&sums[4], 1ull);
    }
}

// *differ = 1 when the staged caller row offsets a differ from b (the
// offsets the current layout was built from)
__global__ void k_rows_differ(int32_t n1, const int32_t *a, const int32_t *b, unsigned long long *differ)
{
    int d = 0;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n1; i += gridDim.x * blockDim.x)
        d |= __ldcs(&a[i]) != __ldcs(&b[i]);
    if (__syncthreads_or(d) && threadIdx.x == 0) *differ = 1ull;
}

// symmetry checksum of a CSR without relabeling (rows below the hub
// threshold, so a thread per row), and its least weight in sums[3]
__global__ void k_sym_check(int32_t n, const int32_t *row, const int32_t *col, const int32_t *wt,
                            unsigned long long *sums)
{
    unsigned long long s_lo = 0, s_hi = 0;
    int32_t wlo = INT32_MAX;
    const int32_t stride = gridDim.x * blockDim.x;
    for (int32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const int32_t u = base + (threadIdx.x & 31);
        if (u < n)
            for (int32_t p = row[u]; p < row[u + 1]; p++) {
                sym_add(s_lo, s_hi, u, col[p], (uint32_t)wt[p]);
                wlo = min(wlo, wt[p]);
            }
    }
    sym_flush(sums, s_lo, s_hi);
    wmin_flush(&sums[3], wlo);
}

// inverse of k_relabel_edges for per-edge payloads (engine order -> caller order)
__global__ void k_unrelabel_edges(int32_t m, const int32_t *__restrict__ cpos, const uint32_t *__restrict__ src,
                                  uint32_t *__restrict__ dst)
{
    for (int32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < m; p += gridDim.x * blockDim.x)
        dst[__ldcs(&cpos[p])] = __ldcs(&src[p]);
}

// caller-order result: dst[r*n + v] = src[r*n + old2new[v]]
template <class T>
__global__ void k_to_caller(int32_t n, int32_t rows, const int32_t *old2new, const T *src, T *dst)
{
    const size_t total = (size_t)n * rows;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        size_t r = i / n;
        int32_t v = (int32_t)(i - r * n);
        dst[i] = src[r * n + old2new[v]];
    }
}

// CC labels: minimum caller id of every engine-space root, then per vertex.
// Most vertices share one root (the giant component), so a warp whose 32
// vertices have the same root reduces first and issues one atomic.
__global__ void k_cc_min_old(int32_t n, const int32_t *parent, const int32_t *new2old, int32_t *minold)
{
    const int lane = threadIdx.x & 31;
    for (int32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += gridDim.x * blockDim.x) {
        const int32_t v = base + lane;
        const bool ok = v < n;
        const int32_t key = ok ? parent[v] : -1 - lane;
        int32_t val = ok ? new2old[v] : 0x7fffffff;
        int same = 0;
        __match_all_sync(0xffffffffu, key, &same);
        if (same) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) val = min(val, __shfl_xor_sync(0xffffffffu, val, o));
            if (lane == 0 && val < __ldcg(&minold[key])) atomicMin(&minold[key], val);
        } else if (ok && val < __ldcg(&minold[key])) {
            atomicMin(&minold[key], val);
        }
    }
}

__global__ void k_cc_label_old(int32_t n, const int32_t *parent, const int32_t *old2new, const int32_t *minold,
                               int32_t *out)
{
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        out[v] = minold[parent[old2new[v]]];
}

// engine CSR (col, wt) from caller-order arrays with the current layout's
// positions; the optional pair checksum and skip word as k_relabel_edges.
// The first call of a layout builds the position tables from src_row (the
// layout's caller row offsets).
static mg_status relabel_device(mg_graph *g, const mgi::DevBuf &src_row, const mgi::DevBuf &src_col,
                                const mgi::DevBuf &src_wt, unsigned long long *sym_sums = nullptr,
                                const unsigned long long *skip = nullptr)
{
    if (g->ne == 0) return MG_OK;
    const int grid = g->num_sms * 8;
    if (!g->pos_valid) {  // once per layout
        MG_TRY(dev_alloc(g->pos_row, ((size_t)g->ne / 32 + 2) * 4));
        MG_TRY(dev_alloc(g->cpos, (size_t)g->ne * 4));
        k_pos_rows<<<grid, 256, 0, g->stream>>>(g->nv, g->ne, g->row.as<int32_t>(), g->pos_row.as<int32_t>());
        k_caller_pos<<<grid, 256, 0, g->stream>>>(g->ne, g->new2old.as<int32_t>(), src_row.as<int32_t>(),
                                                  g->row.as<int32_t>(), g->pos_row.as<int32_t>(),
                                                  g->cpos.as<int32_t>());
        MG_CUDA(cudaGetLastError());
        g->pos_valid = true;
    }
    if (sym_sums)
        k_relabel_edges<true><<<grid, 256, 0, g->stream>>>(
            g->ne, g->old2new.as<int32_t>(), g->row.as<int32_t>(), g->pos_row.as<int32_t>(), g->cpos.as<int32_t>(),
            src_col.as<uint32_t>(), g->col.as<uint32_t>(), src_wt.as<uint32_t>(), g->wt.as<uint32_t>(), 1, sym_sums,
            skip);
    else
        k_relabel_edges<false><<<grid, 256, 0, g->stream>>>(
            g->ne, g->old2new.as<int32_t>(), g->row.as<int32_t>(), g->pos_row.as<int32_t>(), g->cpos.as<int32_t>(),
            src_col.as<uint32_t>(), g->col.as<uint32_t>(), src_wt.as<uint32_t>(), g->wt.as<uint32_t>(), 1, nullptr,
            nullptr);
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}

static mg_status upload_bins(mg_graph *g, const HostLayout &L);

namespace mgi {

mg_status rebin(mg_graph *g, int32_t heavy, int32_t chunk, int32_t tbin)
{
    if (tbin < 1 || heavy <= tbin || chunk < 256 || chunk % 256 != 0)
        return fail(MG_ERR_INVALID, "bad bin parameters %d/%d/%d", heavy, chunk, tbin);
    if (heavy == g->heavy_deg && chunk == g->hchunk_size && tbin == g->tbin) return MG_OK;
    MG_CUDA(cudaStreamSynchronize(g->stream));
    HostLayout L;
    build_bins(g->h_prow, g->nv, heavy, chunk, tbin, L);
    MG_TRY(upload_bins(g, L));
    // captured loops and per-chunk buffers follow the old bins
    free_frontier_ws(g);
    free_pr_ws(g);
    free_cc_ws(g);
    free_bc_ws(g);
    return MG_OK;
}

int32_t to_engine(const mg_graph *g, int32_t v) { return g->relabeled ? g->h_old2new[v] : v; }

mg_status to_caller(mg_graph *g, int which, const void *src, size_t elem, int32_t rows, const void **out)
{
    if (!g->relabeled) { *out = src; return MG_OK; }
    const size_t total = (size_t)g->nv * rows;
    MG_TRY(dev_alloc(g->res_out[which], std::max<size_t>(total, 1) * elem));
    const int grid = g->num_sms * 8;
    if (elem == 8)
        k_to_caller<unsigned long long><<<grid, 256, 0, g->stream>>>(
            g->nv, rows, g->old2new.as<int32_t>(), (const unsigned long long *)src, g->res_out[which].as<unsigned long long>());
    else
        k_to_caller<uint32_t><<<grid, 256, 0, g->stream>>>(g->nv, rows, g->old2new.as<int32_t>(),
                                                           (const uint32_t *)src, g->res_out[which].as<uint32_t>());
    MG_CUDA(cudaGetLastError());
    *out = g->res_out[which].p;
    return MG_OK;
}

mg_status vertices_to_engine(mg_graph *g, const void *src_caller, void *dst_engine)
{
    if (!g->relabeled) {
        if (src_caller != dst_engine)
            MG_CUDA(cudaMemcpyAsync(dst_engine, src_caller, (size_t)g->nv * 4, cudaMemcpyDeviceToDevice, g->stream));
        return MG_OK;
    }
    k_to_caller<uint32_t><<<g->num_sms * 8, 256, 0, g->stream>>>(g->nv, 1, g->new2old.as<int32_t>(),
                                                                 (const uint32_t *)src_caller, (uint32_t *)dst_engine);
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}

mg_status cc_to_caller(mg_graph *g, const int32_t *parent, const void **out)
{
    if (!g->relabeled) { *out = parent; return MG_OK; }
    const size_t n = (size_t)std::max(g->nv, 1);
    MG_TRY(dev_alloc(g->res_out[MG_RES_LABEL], n * 4));
    MG_TRY(dev_alloc(g->res_out[7], n * 4));
    MG_CUDA(cudaMemsetAsync(g->res_out[7].p, 0x7f, n * 4, g->stream));
    const int grid = g->num_sms * 8;
    k_cc_min_old<<<grid, 256, 0, g->stream>>>(g->nv, parent, g->new2old.as<int32_t>(), g->res_out[7].as<int32_t>());
    k_cc_label_old<<<grid, 256, 0, g->stream>>>(g->nv, parent, g->old2new.as<int32_t>(), g->res_out[7].as<int32_t>(),
                                                g->res_out[MG_RES_LABEL].as<int32_t>());
    MG_CUDA(cudaGetLastError());
    *out = g->res_out[MG_RES_LABEL].p;
    return MG_OK;
}

mg_status edges_to_engine(mg_graph *g, const void *src_caller, void *dst_engine)
{
    if (!g->relabeled) {
        MG_CUDA(cudaMemcpyAsync(dst_engine, src_caller, (size_t)g->ne * 4, cudaMemcpyDeviceToDevice, g->stream));
        return MG_OK;
    }
    if (g->ne == 0) return MG_OK;
    k_relabel_edges<false><<<g->num_sms * 8, 256, 0, g->stream>>>(
        g->ne, g->old2new.as<int32_t>(), g->row.as<int32_t>(), g->pos_row.as<int32_t>(), g->cpos.as<int32_t>(),
        (const uint32_t *)src_caller, (uint32_t *)dst_engine, nullptr, nullptr, 0, nullptr, nullptr);
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}

mg_status edges_to_caller(mg_graph *g, const void *src_engine, void *dst_caller)
{
    if (!g->relabeled) {
        MG_CUDA(cudaMemcpyAsync(dst_caller, src_engine, (size_t)g->ne * 4, cudaMemcpyDeviceToDevice, g->stream));
        return MG_OK;
    }
    if (g->ne == 0) return MG_OK;
    k_unrelabel_edges<<<g->num_sms * 8, 256, 0, g->stream>>>(g->ne, g->cpos.as<int32_t>(),
                                                             (const uint32_t *)src_engine, (uint32_t *)dst_caller);
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}

}  // namespace mgi

// degree bins and heavy chunks to the device (buffers grow when needed)
static mg_status upload_bins(mg_graph *g, const HostLayout &L)
{
    cudaStream_t s = g->stream;
    MG_TRY(dev_alloc(g->hchunk, std::max<size_t>(L.hchunk.size(), 3) * 4));
    MG_TRY(dev_alloc(g->hrows, std::max<size_t>(L.hrows.size(), 1) * 4));
    MG_TRY(dev_alloc(g->hrow_chunk, L.hrow_chunk.size() * 4));
    MG_TRY(dev_alloc(g->wrows, std::max<size_t>(L.wrows.size(), 1) * 4));
    MG_TRY(dev_alloc(g->trows, std::max<size_t>(L.trows.size(), 1) * 4));
    if (!L.hchunk.empty())
        MG_CUDA(cudaMemcpyAsync(g->hchunk.p, L.hchunk.data(), L.hchunk.size() * 4, cudaMemcpyHostToDevice, s));
    if (!L.hrows.empty())
        MG_CUDA(cudaMemcpyAsync(g->hrows.p, L.hrows.data(), L.hrows.size() * 4, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(g->hrow_chunk.p, L.hrow_chunk.data(), L.hrow_chunk.size() * 4, cudaMemcpyHostToDevice, s));
    if (!L.wrows.empty())
        MG_CUDA(cudaMemcpyAsync(g->wrows.p, L.wrows.data(), L.wrows.size() * 4, cudaMemcpyHostToDevice, s));
    if (!L.trows.empty())
        MG_CUDA(cudaMemcpyAsync(g->trows.p, L.trows.data(), L.trows.size() * 4, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaStreamSynchronize(s));
    g->nwrows = (int32_t)L.wrows.size();
    g->nwlong = L.nwlong;
    g->ntrows = (int32_t)L.trows.size();
    g->nhchunks = (int32_t)(L.hchunk.size() / 3);
    g->nhrows = (int32_t)L.hrows.size();
    g->heavy_deg = L.heavy;
    g->hchunk_size = L.chunk;
    g->tbin = L.tbin;
    return MG_OK;
}

static mg_status upload_arrays(mg_graph *g, const mg_host_graph *h, const HostLayout &L, bool alloc)
{
    const size_t n = (size_t)h->nv, m = (size_t)h->ne;
    if (alloc) {
        MG_TRY(dev_alloc(g->row, (n + 1) * 4));
        MG_TRY(dev_alloc(g->col, std::max<size_t>(m, 4) * 4 + COL_PAD));
        MG_TRY(dev_alloc(g->wt, std::max<size_t>(m, 4) * 4 + COL_PAD));
        if (L.relabel) {
            MG_TRY(dev_alloc(g->o_row, (n + 1) * 4));
            MG_TRY(dev_alloc(g->o_col, std::max<size_t>(m, 4) * 4 + COL_PAD));
            MG_TRY(dev_alloc(g->o_wt, std::max<size_t>(m, 4) * 4 + COL_PAD));
            MG_TRY(dev_alloc(g->old2new, std::max<size_t>(n, 1) * 4));
            MG_TRY(dev_alloc(g->new2old, std::max<size_t>(n, 1) * 4));
        }
        if (!L.trow.empty()) {
            MG_TRY(dev_alloc(g->trow_own, (n + 1) * 4));
            MG_TRY(dev_alloc(g->tcol_own, std::max<size_t>(m, 4) * 4 + COL_PAD));
            MG_TRY(dev_alloc(g->twt_own, std::max<size_t>(m, 4) * 4 + COL_PAD));
        }
    }
    cudaStream_t s = g->stream;
    g->relabeled = L.relabel;
    if (L.relabel) {
        g->h_old2new = L.old2new;
        MG_CUDA(cudaMemcpyAsync(g->old2new.p, L.old2new.data(), n * 4, cudaMemcpyHostToDevice, s));
        MG_CUDA(cudaMemcpyAsync(g->new2old.p, L.new2old.data(), n * 4, cudaMemcpyHostToDevice, s));
        MG_CUDA(cudaMemcpyAsync(g->row.p, L.row_new.data(), (n + 1) * 4, cudaMemcpyHostToDevice, s));
        MG_CUDA(cudaMemcpyAsync(g->o_row.p, h->v.data(), (n + 1) * 4, cudaMemcpyHostToDevice, s));
        if (m) {
            MG_CUDA(cudaMemcpyAsync(g->o_col.p, h->e.data(), m * 4, cudaMemcpyHostToDevice, s));
            MG_CUDA(cudaMemcpyAsync(g->o_wt.p, h->ev.data(), m * 4, cudaMemcpyHostToDevice, s));
        }
        g->nv = h->nv;
        g->pos_valid = false;  // new engine row offsets
        MG_TRY(relabel_device(g, g->o_row, g->o_col, g->o_wt));
    } else {
        MG_CUDA(cudaMemcpyAsync(g->row.p, h->v.data(), (n + 1) * 4, cudaMemcpyHostToDevice, s));
        if (m) {
            MG_CUDA(cudaMemcpyAsync(g->col.p, h->e.data(), m * 4, cudaMemcpyHostToDevice, s));
            MG_CUDA(cudaMemcpyAsync(g->wt.p, h->ev.data(), m * 4, cudaMemcpyHostToDevice, s));
        }
    }
    if (!L.trow.empty()) {
        MG_CUDA(cudaMemcpyAsync(g->trow_own.p, L.trow.data(), (n + 1) * 4, cudaMemcpyHostToDevice, s));
        if (m) {
            MG_CUDA(cudaMemcpyAsync(g->tcol_own.p, L.tcol.data(), m * 4, cudaMemcpyHostToDevice, s));
            MG_CUDA(cudaMemcpyAsync(g->twt_own.p, L.twt.data(), m * 4, cudaMemcpyHostToDevice, s));
        }
        g->trow = g->trow_own.as<int32_t>(); g->tcol = g->tcol_own.as<int32_t>(); g->twt = g->twt_own.as<int32_t>();
    } else {
        g->trow = g->row.as<int32_t>(); g->tcol = g->col.as<int32_t>(); g->twt = g->wt.as<int32_t>();
    }
    MG_TRY(upload_bins(g, L));
    g->hub.valid = false;  // new pull columns
    g->h_prow = L.prow;
    g->symmetric = L.symmetric;
    g->weights_symmetric = L.wsym;
    g->n_dangling = L.n_dangling;
    g->min_weight = L.min_weight;
    return MG_OK;
}

static void destroy_graph(mg_graph *g)
{
    if (!g) return;
    cudaSetDevice(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    free_frontier_ws(g);
    free_pr_ws(g);
    free_cc_ws(g);
    free_bc_ws(g);
    free_ppr_ws(g);
    free_wpr_ws(g);
    hub_free(g);
    DevBuf *bufs[] = {&g->row, &g->col, &g->wt, &g->trow_own, &g->tcol_own, &g->twt_own,
                      &g->hchunk, &g->hrows, &g->hrow_chunk, &g->fw, &g->o_fw, &g->ppr_hchunk, &g->ppr_hrows,
                      &g->ppr_hrow_chunk, &g->o_row, &g->o_col, &g->o_wt, &g->old2new, &g->new2old,
                      &g->wrows, &g->trows, &g->pos_row, &g->cpos, &g->sym_sums, &g->s_row,
                      &g->s_col, &g->s_wt};
    for (DevBuf *b : bufs) dev_free(*b);
    for (DevBuf &b : g->res_out) dev_free(b);
    if (g->pinned_flag) cudaFreeHost(g->pinned_flag);
    if (g->sym_host) cudaFreeHost(g->sym_host);
    if (g->ev0) cudaEventDestroy(g->ev0);
    if (g->ev1) cudaEventDestroy(g->ev1);
    if (g->ev_staged) cudaEventDestroy(g->ev_staged);
    if (g->ev_consumed) cudaEventDestroy(g->ev_consumed);
    if (g->copy_stream) {
        cudaStreamSynchronize(g->copy_stream);
        cudaStreamDestroy(g->copy_stream);
    }
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

extern "C" {

void mg_opts_default(mg_opts *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->exec = MG_EXEC_GRAPH;
    o->direction = MG_DIR_AUTO;
    o->max_iter = 0;
    o->alpha = 15;
    o->beta = 18;
    o->damping = 0.85f;
    o->tol = 1e-6f;
    o->profile = 0;
    o->pr_layout = MG_PR_LAYOUT_AUTO;
}

mg_status mg_graph_upload(const mg_host_graph *h, int32_t device, mg_graph **out)
{
    clear_error();
    if (!h || !out) return fail(MG_ERR_INVALID, "null argument");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(MG_ERR_CUDA, "no CUDA device available (%s)", cudaGetErrorString(e));
    }
    if (device < 0 || device >= ndev) return fail(MG_ERR_RANGE, "device %d out of range [0,%d)", device, ndev);
    MG_CUDA(cudaSetDevice(device));
    std::unique_ptr<mg_graph, void (*)(mg_graph *)> g(new mg_graph(), destroy_graph);
    g->device = device;
    g->nv = h->nv;
    g->ne = h->ne;
    MG_CUDA(cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, device));
    MG_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    MG_CUDA(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
    MG_CUDA(cudaEventCreate(&g->ev0));
    MG_CUDA(cudaEventCreate(&g->ev1));
    MG_CUDA(cudaEventCreateWithFlags(&g->ev_staged, cudaEventDisableTiming));
    MG_CUDA(cudaEventCreateWithFlags(&g->ev_consumed, cudaEventDisableTiming));
    MG_CUDA(cudaMallocHost(&g->pinned_flag, 64));
    MG_CUDA(cudaMallocHost(&g->sym_host, 64));
    HostLayout L;
    build_layout(*h, L);
    MG_TRY(upload_arrays(g.get(), h, L, true));
    MG_CUDA(cudaEventRecord(g->ev_consumed, g->stream));
    *out = g.release();
    return MG_OK;
}

mg_status mg_graph_stage(mg_graph *g, const mg_host_graph *h)
{
    clear_error();
    if (!g || !h) return fail(MG_ERR_INVALID, "null argument");
    if (h->nv != g->nv || h->ne != g->ne) return fail(MG_ERR_INVALID, "staging needs the same nv/ne");
    MG_CUDA(cudaSetDevice(g->device));
    const size_t n = (size_t)h->nv, m = (size_t)h->ne;
    // staging buffers, separate from the current graph's caller-order
    // arrays (o_*), which runs before the commit still read
    MG_TRY(dev_alloc(g->s_row, (n + 1) * 4));
    MG_TRY(dev_alloc(g->s_col, std::max<size_t>(m, 4) * 4 + COL_PAD));
    MG_TRY(dev_alloc(g->s_wt, std::max<size_t>(m, 4) * 4 + COL_PAD));
    cudaStream_t cs = g->copy_stream;
    MG_CUDA(cudaStreamWaitEvent(cs, g->ev_consumed, 0));  // the last commit has read them
    const int32_t *hv = h->pin_v ? h->pin_v : h->v.data();
    const int32_t *he = h->pin_e ? h->pin_e : h->e.data();
    const int32_t *hev = h->pin_ev ? h->pin_ev : h->ev.data();
    MG_CUDA(cudaMemcpyAsync(g->s_row.p, hv, (n + 1) * 4, cudaMemcpyHostToDevice, cs));
    if (m) {
        MG_CUDA(cudaMemcpyAsync(g->s_col.p, he, m * 4, cudaMemcpyHostToDevice, cs));
        MG_CUDA(cudaMemcpyAsync(g->s_wt.p, hev, m * 4, cudaMemcpyHostToDevice, cs));
    }
    MG_CUDA(cudaEventRecord(g->ev_staged, cs));
    g->staged_h = h;
    return MG_OK;
}

// A commit that laid the graph out again may have changed the bins, the
// chunk lists and the least weight that captured loops carry by value:
// drop the workspaces (and with them the captured loops) so the next runs
// rebuild them.
static void drop_workspaces(mg_graph *g)
{
    free_frontier_ws(g);
    free_pr_ws(g);
    free_cc_ws(g);
    free_bc_ws(g);
    free_ppr_ws(g);
    free_wpr_ws(g);
    // the personalised-PageRank heavy-row table follows the pull offsets of
    // the old layout: rebuild it on the next mg_ppr_batch
    g->ppr_nhchunks = -1;
    g->ppr_nhrows = 0;
    // a new layout has not been timed by mg_autotune
    g->pr_prefer_gather = false;
}

mg_status mg_graph_commit(mg_graph *g)
{
    clear_error();
    if (!g) return fail(MG_ERR_INVALID, "null argument");
    if (!g->staged_h) return fail(MG_ERR_INVALID, "nothing staged (mg_graph_stage)");
    MG_CUDA(cudaSetDevice(g->device));
    const mg_host_graph *h = g->staged_h;
    g->staged_h = nullptr;
    cudaStream_t s = g->stream;
    MG_CUDA(cudaStreamWaitEvent(s, g->ev_staged, 0));
    const size_t n = (size_t)h->nv, m = (size_t)h->ne;
    if (!(g->symmetric && g->weights_symmetric)) {
        // a transposed copy to rebuild: lay the graph out again (with the
        // graph's current, possibly tuned, bin parameters)
        HostLayout L;
        build_layout(*h, L, g->heavy_deg, g->hchunk_size, g->tbin);
        MG_CUDA(cudaStreamSynchronize(s));
        drop_workspaces(g);
        MG_TRY(upload_arrays(g, h, L, true));
    } else {
        // the layout assumes the caller row offsets it was built from and
        // symmetric edges and weights: compare the offsets on the device,
        // check the staged input with the pair checksum (formed during the
        // relabel pass), read both back in one copy and lay the graph out
        // again from the host when either fails
        MG_TRY(dev_alloc(g->sym_sums, 64));
        unsigned long long *sums = g->sym_sums.as<unsigned long long>();
        MG_CUDA(cudaMemsetAsync(sums, 0, 24, s));
        MG_CUDA(cudaMemsetAsync(sums + 3, 0xff, 8, s));
        // column change word: set by the relabel pass; the copy path below
        // rewrites the columns without comparing, so it counts as changed
        MG_CUDA(cudaMemsetAsync(sums + 4, g->relabeled ? 0 : 0xff, 8, s));
        const int32_t *ref_row = g->relabeled ? g->o_row.as<int32_t>() : g->row.as<int32_t>();
        k_rows_differ<<<g->num_sms * 4, 256, 0, s>>>((int32_t)n + 1, g->s_row.as<int32_t>(), ref_row, sums + 2);
        MG_CUDA(cudaGetLastError());
        if (g->relabeled) {
            // engine CSR from the staged caller-order arrays
            MG_TRY(relabel_device(g, g->s_row, g->s_col, g->s_wt, sums, sums + 2));
        } else {
            MG_CUDA(cudaMemcpyAsync(g->row.p, g->s_row.p, (n + 1) * 4, cudaMemcpyDeviceToDevice, s));
            if (m) {
                MG_CUDA(cudaMemcpyAsync(g->col.p, g->s_col.p, m * 4, cudaMemcpyDeviceToDevice, s));
                MG_CUDA(cudaMemcpyAsync(g->wt.p, g->s_wt.p, m * 4, cudaMemcpyDeviceToDevice, s));
            }
            k_sym_check<<<g->num_sms * 8, 256, 0, s>>>(g->nv, g->row.as<int32_t>(), g->col.as<int32_t>(),
                                                       g->wt.as<int32_t>(), sums);
            MG_CUDA(cudaGetLastError());
        }
        MG_CUDA(cudaMemcpyAsync(g->sym_host, sums, 40, cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaStreamSynchronize(s));
        if (g->sym_host[2] != 0 || g->sym_host[0] != g->sym_host[1]) {
            HostLayout L;
            build_layout(*h, L, g->heavy_deg, g->hchunk_size, g->tbin);
            drop_workspaces(g);
            MG_TRY(upload_arrays(g, h, L, true));
        } else {
            // same layout, new weights: their least value bounds the SSSP
            // pull's settled-row skip and gates SSSP on negative weights
            g->min_weight = wmin_decode(g->sym_host[3]);
            // PageRank's hub split follows the columns: rebuilt only when
            // some column id changed
            if (g->sym_host[4] != 0) g->hub.valid = false;
            if (g->relabeled) {
                // the staged arrays are now the current graph's caller-order CSR
                std::swap(g->o_row, g->s_row);
                std::swap(g->o_col, g->s_col);
                std::swap(g->o_wt, g->s_wt);
            }
        }
    }
    MG_CUDA(cudaEventRecord(g->ev_consumed, s));
    g->fw_version += 1;  // quantities derived from the float weights are stale
    return MG_OK;
}

mg_status mg_graph_reload(mg_graph *g, const mg_host_graph *h)
{
    MG_TRY(mg_graph_stage(g, h));
    return mg_graph_commit(g);
}

void mg_graph_free(mg_graph *g) { destroy_graph(g); }

mg_status mg_graph_info(const mg_graph *g, int32_t *nv, int32_t *ne)
{
    if (!g) return fail(MG_ERR_INVALID, "null graph");
    if (nv) *nv = g->nv;
    if (ne) *ne = g->ne;
    return MG_OK;
}

void *mg_graph_stream(mg_graph *g) { return g ? (void *)g->stream : nullptr; }

mg_status mg_graph_set_float_weights(mg_graph *g, const float *w)
{
    clear_error();
    if (!g || (!w && g->ne > 0)) return fail(MG_ERR_INVALID, "null argument");
    MG_CUDA(cudaSetDevice(g->device));
    MG_TRY(dev_alloc(g->fw, std::max<size_t>((size_t)g->ne, 4) * 4 + COL_PAD));
    if (g->relabeled) {
        // keep the caller-order copy (the transposed weights are found there,
        // where rows have ascending columns) and relabel into engine order
        MG_TRY(dev_alloc(g->o_fw, std::max<size_t>((size_t)g->ne, 4) * 4 + COL_PAD));
        if (g->ne) MG_CUDA(cudaMemcpyAsync(g->o_fw.p, w, (size_t)g->ne * 4, cudaMemcpyHostToDevice, g->stream));
        MG_TRY(edges_to_engine(g, g->o_fw.p, g->fw.p));
    } else if (g->ne) {
        MG_CUDA(cudaMemcpyAsync(g->fw.p, w, (size_t)g->ne * 4, cudaMemcpyHostToDevice, g->stream));
    }
    MG_CUDA(cudaStreamSynchronize(g->stream));
    g->has_fw = true;
    g->fw_version += 1;
    return MG_OK;
}

const void *mg_result_device(mg_graph *g, int32_t which)
{
    if (!g || which < 0 || which >= 8) return nullptr;
    return g->res[which];
}

void mg_host_graph_free(mg_host_graph *h)
{
    if (!h) return;
    if (h->pinned) {
        if (h->pin_v) cudaFreeHost(h->pin_v);
        if (h->pin_e) cudaFreeHost(h->pin_e);
        if (h->pin_ev) cudaFreeHost(h->pin_ev);
    }
    delete h;
}

mg_status mg_host_graph_pin(mg_host_graph *h)
{
    clear_error();
    if (!h) return fail(MG_ERR_INVALID, "null argument");
    if (h->pinned) return MG_OK;
    // driver-allocated page-locked copies (registered malloc pages were
    // measured slower for uploads that overlap running kernels)
    auto copy = [](const std::vector<int32_t> &src, int32_t **dst) -> mg_status {
        if (src.empty()) return MG_OK;
        MG_CUDA(cudaHostAlloc((void **)dst, src.size() * 4, cudaHostAllocDefault));
        std::memcpy(*dst, src.data(), src.size() * 4);
        return MG_OK;
    };
    mg_status st = copy(h->v, &h->pin_v);
    if (st == MG_OK) st = copy(h->e, &h->pin_e);
    if (st == MG_OK) st = copy(h->ev, &h->pin_ev);
    if (st != MG_OK) {
        if (h->pin_v) cudaFreeHost(h->pin_v);
        if (h->pin_e) cudaFreeHost(h->pin_e);
        if (h->pin_ev) cudaFreeHost(h->pin_ev);
        h->pin_v = h->pin_e = h->pin_ev = nullptr;
        return st;
    }
    h->pinned = true;
    return MG_OK;
}

int64_t mg_host_graph_stage_bytes(const mg_host_graph *h)
{
    if (!h) return 0;
    const int64_t n = h->nv, m = h->ne;
    return 4 * (n + 1) + 8 * m;
}

}  // extern "C"
