// mg_hub.cu -- shared-memory hub split of the pull rows for PageRank sweeps.
//
// The reference turns the random gathers of its dense PageRank phases into
// partition-local work: edges are regrouped into 16-bit tile streams by
// source partition (gen_structure.cu:1534-1947, sp1/sp2/mapper) and each
// partition's values are summed in shared memory (processi.cu:682-894,
// _phase1/_phase2).  Re-derived for GB300 and the hub-first vertex order:
// with hubs at the lowest ids, the first HUB_MAX vertices (the most a CTA's
// 227 KB of shared memory holds as FP32) are the sources of most edges
// (R-MAT 22: 59.6 % of 128 M), so each pull row is split once per layout
// into
//   hub part  : in-edges from ids < H, as 16-bit ids in one stream
//               (hub_col16, row offsets hub_off), gathered from a shared-
//               memory copy of the contributions c[0, H) that every CTA
//               stages with one bulk copy (cp.async.bulk) per sweep;
//   tail part : the other in-edges, int32 ids (hub_tcol, offsets
//               hub_toff), gathered through L2 by the degree-binned sweep.
// The hub stream is cut into 256-edge chunks, a warp each: every lane takes
// 8 consecutive edges with one 128-bit load, a bitmap marks the first hub
// edge of every row, and a segmented sum (per lane, then a shuffle tree
// across lanes) gives every row that ends inside the chunk its total; a row
// that runs past the chunk is finished by k_hub_fix, which adds the chunk
// heads that follow in order.  Sums are formed in a fixed order, so sweeps
// are reproducible.  Rows with no hub edge keep hub_sum = 0.
//
// Per sweep the hub part moves 2 B per hub edge (plus 1 bit of row starts)
// instead of 4 B of ids and a 32-byte L2 sector per gather.

#include "mg_device.cuh"

#include <algorithm>
#include <atomic>
#include <cstring>

namespace {

constexpr int32_t HUB_MAX = 57344;  // hub vertices staged per CTA: 224 KB of FP32 contributions
constexpr int HUB_CHUNK = 256;      // edges per warp chunk: 8 per lane
constexpr int HUB_THREADS = 1024;   // one CTA per SM (shared memory bound)
constexpr int HUB_ILP = 2;          // chunks in flight per warp
constexpr int SCAN_T = 1024, SCAN_IPT = 4, SCAN_TILE = SCAN_T * SCAN_IPT;
constexpr long long HUB_WAIT_LIMIT = 20000000ll;  // clock64 cycles (~10 ms) for the bulk copy
constexpr int32_t FIX_SHORT = 8;    // carry spans up to this many chunks: a thread each

// ---------------------------------------------------------------------------
// exclusive scan of int32 (out[n] = total): tiles of 4096, tile totals
// scanned by one block, offsets added back
// ---------------------------------------------------------------------------
__device__ __forceinline__ int32_t block_excl_scan(int32_t v, int32_t *s_warp, int32_t *total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int32_t t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    if (w == 0) {
        int32_t y = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t t = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= o) y += t;
        }
        s_warp[lane] = y;  // inclusive warp totals
    }
    __syncthreads();
    const int32_t before = w ? s_warp[w - 1] : 0;
    *total = s_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(SCAN_T) k_scan_tiles(const int32_t *in, int32_t n, int32_t *out, int32_t *tile_sum)
{
    __shared__ int32_t s_warp[32];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_IPT;
    int32_t v[SCAN_IPT], s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_IPT; i++) {
        v[i] = base + i < n ? in[base + i] : 0;
        s += v[i];
    }
    int32_t tot;
    int32_t e = block_excl_scan(s, s_warp, &tot);
#pragma unroll
    for (int i = 0; i < SCAN_IPT; i++) {
        if (base + i < n) out[base + i] = e;
        e += v[i];
    }
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

// one block: exclusive scan of the tile totals in place; total -> *grand
__global__ void __launch_bounds__(SCAN_T) k_scan_part(int32_t *tile_sum, int32_t ntiles, int32_t *grand)
{
    __shared__ int32_t s_warp[32];
    int32_t carry = 0;
    for (int32_t b0 = 0; b0 < ntiles; b0 += SCAN_T) {
        const int32_t i = b0 + threadIdx.x;
        const int32_t v = i < ntiles ? tile_sum[i] : 0;
        int32_t tot;
        const int32_t e = block_excl_scan(v, s_warp, &tot);
        if (i < ntiles) tile_sum[i] = carry + e;
        carry += tot;
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void k_scan_add(int32_t *out, int32_t n, const int32_t *tile_sum)
{
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    const int32_t add = tile_sum[blockIdx.x];
    for (int i = threadIdx.x; i < SCAN_TILE; i += blockDim.x)
        if (base + i < n) out[base + i] += add;
}

// ---------------------------------------------------------------------------
// layout build
// ---------------------------------------------------------------------------
// hub edges per row (warp per row) and the has-hub-edges flag
__global__ void k_hub_count(int32_t n, const int32_t *prow, const int32_t *pcol, int32_t H, int32_t *hcnt,
                            int32_t *hflag)
{
    const int lane = threadIdx.x & 31;
    const int32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (int32_t v = gw; v < n; v += nw) {
        const int32_t b = prow[v], e = prow[v + 1];
        int32_t c = 0;
        for (int32_t p = b + lane; p < e; p += 32) c += __ldg(&pcol[p]) < H;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0) {
            hcnt[v] = c;
            hflag[v] = c > 0;
        }
    }
}

// stable split of every row (warp per row, ballot-ordered writes), tail
// offsets, the hub-row list and the row-start bits of the hub stream
__global__ void k_hub_scatter(int32_t n, const int32_t *prow, const int32_t *pcol, int32_t H, const int32_t *hoff,
                              const int32_t *hidx, uint16_t *hcol, int32_t *tcol, int32_t *toff, int32_t *hrows,
                              uint32_t *rstart)
{
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (int32_t v = gw; v < n; v += nw) {
        const int32_t b = prow[v], e = prow[v + 1];
        const int32_t hb = hoff[v], tb = b - hb;
        int32_t nh = 0, nt = 0;
        for (int32_t p0 = b; p0 < e; p0 += 32) {
            const int32_t p = p0 + lane;
            const int32_t c = p < e ? __ldg(&pcol[p]) : -1;
            const bool hub = p < e && c < H, tl = p < e && c >= H;
            const unsigned mh = __ballot_sync(0xffffffffu, hub), mt = __ballot_sync(0xffffffffu, tl);
            if (hub) hcol[hb + nh + __popc(mh & lt)] = (uint16_t)c;
            if (tl) tcol[tb + nt + __popc(mt & lt)] = c;
            nh += __popc(mh);
            nt += __popc(mt);
        }
        if (lane == 0) {
            toff[v] = tb;
            if (v == n - 1) toff[n] = prow[n] - hoff[n];
            if (nh > 0) {
                hrows[hidx[v]] = v;
                atomicOr(&rstart[hb >> 5], 1u << (hb & 31));
            }
        }
    }
}

// padding of the hub stream up to whole chunks: id H (a zero in shared memory)
__global__ void k_hub_pad(uint16_t *hcol, int64_t from, int64_t to, int32_t H)
{
    for (int64_t i = from + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < to; i += (int64_t)gridDim.x * blockDim.x)
        hcol[i] = (uint16_t)H;
}

// row starts per chunk (8 bitmap words each)
__global__ void k_chunk_starts(const uint32_t *rstart, int32_t nchunks, int32_t *cnt)
{
    for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nchunks; c += gridDim.x * blockDim.x) {
        int32_t s = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) s += __popc(rstart[8 * c + k]);
        cnt[c] = s;
    }
}

// ---------------------------------------------------------------------------
// sweep
// ---------------------------------------------------------------------------
struct HubArgs {
    const uint16_t *hcol;     // hub stream (padded to whole chunks)
    const uint32_t *rstart;   // row-start bits of the hub stream
    const int32_t *crow;      // hub-row index of each chunk's first row start
    const int32_t *hrows;     // rows that have hub edges, ascending
    const float *c[2];        // contributions (ping-pong, ctl selects)
    const int32_t *cur;       // current iterate index (loop control block)
    const int32_t *more;      // loop continue flag
    const int32_t *off;       // non-zero: sweeps run elsewhere (queue sweeps)
    float *hsum;              // per-row hub sums
    float *chead, *ctail;     // per chunk: sum before its first row start / of its open last row
    int32_t *cstart;          // per chunk: has a row start
    const int32_t *cnext;     // per chunk with a start: the next chunk with one (nchunks: none)
    const int32_t *clong;     // chunks whose last row spans more than FIX_SHORT chunks
    int32_t nlong;
    int32_t *err;             // bulk copy wait ran out
    int32_t H, nchunks;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Stage c[0, H) into shared memory with bulk copies on an mbarrier; the
// wait is bounded (HUB_WAIT_LIMIT cycles), after which *err is set and the
// CTA returns false (it still waits, bounded, for its copies to land).
__device__ __forceinline__ bool stage_hub(float *s_c, const float *c, int32_t H, uint64_t *mbar, int32_t *err)
{
    const uint32_t bar = smem_u32(mbar);
    const uint32_t bytes = (uint32_t)H * 4u;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
        constexpr uint32_t PIECE = 32768;
        for (uint32_t off = 0; off < bytes; off += PIECE) {
            const uint32_t sz = min(PIECE, bytes - off);
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(reinterpret_cast<char *>(s_c) + off)),
                "l"(reinterpret_cast<const char *>(c) + off), "r"(sz), "r"(bar)
                : "memory");
        }
    }
    if (threadIdx.x < 4) s_c[H + threadIdx.x] = 0.0f;  // the padding id's slot
    __syncthreads();
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        uint32_t done = 0;
        const long long t0 = clock64();
        bool ok = true;
        while (!done) {
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(done)
                : "r"(bar)
                : "memory");
            if (!done && clock64() - t0 > HUB_WAIT_LIMIT) {
                ok = false;
                break;
            }
        }
        if (!ok) {
            atomicExch(err, 1);
            // the copies may still land: wait for them (bounded again)
            // before the CTA's shared memory is released
            const long long t1 = clock64();
            while (!done && clock64() - t1 < HUB_WAIT_LIMIT) {
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
                    "selp.u32 %0, 1, 0, p;\n\t}"
                    : "=r"(done)
                    : "r"(bar)
                    : "memory");
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

__global__ void __launch_bounds__(HUB_THREADS, 1) k_hub_sweep(HubArgs a)
{
    extern __shared__ __align__(128) float s_c[];   // [H + 4]
    __shared__ __align__(8) uint64_t mbar;
    if (__ldg(a.more) == 0 || __ldg(a.off) != 0) return;
    const float *c = __ldg(a.cur) ? a.c[1] : a.c[0];
    if (!stage_hub(s_c, c, a.H, &mbar, a.err)) return;
    const int lane = threadIdx.x & 31;
    const int32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (int32_t c0 = gw * HUB_ILP; c0 < a.nchunks; c0 += nw * HUB_ILP) {
        uint4 cols[HUB_ILP];
        uint32_t word[HUB_ILP];
        int32_t crow[HUB_ILP];
#pragma unroll
        for (int j = 0; j < HUB_ILP; j++) {
            const int32_t ch = c0 + j;
            if (ch < a.nchunks) {
                cols[j] = __ldcs(reinterpret_cast<const uint4 *>(a.hcol + (int64_t)ch * HUB_CHUNK) + lane);
                word[j] = __ldcs(&a.rstart[(int64_t)ch * 8 + (lane >> 2)]);
                crow[j] = __ldg(&a.crow[ch]);
            }
        }
#pragma unroll
        for (int j = 0; j < HUB_ILP; j++) {
            const int32_t ch = c0 + j;
            if (ch >= a.nchunks) break;   // warp-uniform
            const uint32_t fl = (word[j] >> ((lane & 3) * 8)) & 0xffu;
            const uint32_t w32[4] = {cols[j].x, cols[j].y, cols[j].z, cols[j].w};
            float v[8];
#pragma unroll
            for (int i = 0; i < 8; i++) v[i] = s_c[(w32[i >> 1] >> ((i & 1) * 16)) & 0xffffu];
            // hub-row index of this lane's first row start
            const int nst = __popc(fl);
            int32_t before = nst;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t t = __shfl_up_sync(0xffffffffu, before, o);
                if (lane >= o) before += t;
            }
            before -= nst;
            // per-lane segmented sums, branch-free: outv[i] is the total of
            // the row that ends just before edge i (outf[i]: it started in
            // this lane too); the row indices are loaded together afterwards
            const int32_t rbase = crow[j] + before;   // hub-row index of this lane's first start
            float head = 0.0f, run = 0.0f;
            bool started = false;
            float outv[8];
            bool outf[8];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const bool st = (fl >> i) & 1u;
                outf[i] = st && started;
                outv[i] = run;
                head = (st && !started) ? run : head;
                run = st ? 0.0f : run;
                started = started || st;
                run += v[i];
            }
            if (!started) head = run;
            int32_t rrow[8];
#pragma unroll
            for (int i = 0; i < 8; i++)
                if (outf[i]) rrow[i] = __ldg(&a.hrows[rbase + __popc(fl & ((1u << i) - 1u)) - 1]);
#pragma unroll
            for (int i = 0; i < 8; i++)
                if (outf[i]) a.hsum[rrow[i]] = outv[i];
            const int32_t ridx = rbase + nst - 1;   // the lane's last start (when started)
            // T = sum of heads from this lane up to and including the first
            // lane (>= this one) that has a row start
            float T = head;
            int F = started;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float T2 = __shfl_down_sync(0xffffffffu, T, o);
                const int F2 = __shfl_down_sync(0xffffffffu, F, o);
                if (lane + o < 32 && !F) {
                    T += T2;
                    F |= F2;
                }
            }
            const float Tn = __shfl_down_sync(0xffffffffu, T, 1);
            const int Fn = __shfl_down_sync(0xffffffffu, F, 1);
            const unsigned any = __ballot_sync(0xffffffffu, started);
            if (started) {
                const bool closed = lane < 31 && Fn;
                const float total = run + (lane < 31 ? Tn : 0.0f);
                if (closed) a.hsum[__ldg(&a.hrows[ridx])] = total;
                else a.ctail[ch] = total;   // the chunk's last row runs on
            }
            if (lane == 0) {
                a.chead[ch] = T;
                a.cstart[ch] = any != 0u;
            }
        }
    }
}

// rows that run past their chunk: the open tail plus the heads of the
// following chunks up to and including the next chunk with a row start
// (cnext, fixed by the layout), summed in FP64 and rounded once: a hub row
// can span hundreds of chunks, and an FP32 running sum of their heads would
// carry rounding of a few 1e-6 that moves from sweep to sweep.  Spans of up
// to FIX_SHORT chunks take a thread each; longer ones (clong) a warp each,
// lane-strided then a fixed shuffle tree.  crow[ch + 1] - 1 is the hub-row
// index of chunk ch's last row start.
__global__ void k_hub_fix(HubArgs a)
{
    if (__ldg(a.more) == 0 || __ldg(a.off) != 0) return;
    const int32_t tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    for (int32_t ch = tid; ch < a.nchunks; ch += nth) {
        if (!__ldg(&a.cstart[ch])) continue;
        const int32_t last = min(__ldg(&a.cnext[ch]), a.nchunks - 1);
        if (last - ch > FIX_SHORT) continue;
        double total = a.ctail[ch];
        for (int32_t k = ch + 1; k <= last; k++) total += a.chead[k];
        a.hsum[__ldg(&a.hrows[__ldg(&a.crow[ch + 1]) - 1])] = (float)total;
    }
    const int lane = threadIdx.x & 31;
    for (int32_t i = tid >> 5; i < a.nlong; i += nth >> 5) {
        const int32_t ch = __ldg(&a.clong[i]);
        const int32_t last = min(__ldg(&a.cnext[ch]), a.nchunks - 1);
        double t = 0.0;
        for (int32_t k = ch + 1 + lane; k <= last; k += 32) t += a.chead[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) a.hsum[__ldg(&a.hrows[__ldg(&a.crow[ch + 1]) - 1])] = (float)(t + (double)a.ctail[ch]);
    }
}

// layout: for every chunk with a row start, the next chunk with one (its
// last row ends there), and the list of chunks whose span is long
__global__ void k_hub_spans(const int32_t *cnt, int32_t nchunks, int32_t *cnext, int32_t *clong, int32_t *nlong)
{
    for (int32_t ch = blockIdx.x * blockDim.x + threadIdx.x; ch < nchunks; ch += gridDim.x * blockDim.x) {
        if (!cnt[ch]) continue;
        int32_t k = ch + 1;
        while (k < nchunks && cnt[k] == 0) k++;
        cnext[ch] = k;
        if (min(k, nchunks - 1) - ch > FIX_SHORT) clong[atomicAdd(nlong, 1)] = ch;
    }
}

}  // namespace

namespace mgi {

// exclusive scan of in[0, n) into out[0, n], out[n] = total (on the stream)
static mg_status scan_excl(const int32_t *in, int32_t n, int32_t *out, DevBuf &tiles, cudaStream_t s)
{
    const int32_t ntiles = std::max(1, (n + SCAN_TILE - 1) / SCAN_TILE);
    MG_TRY(dev_alloc(tiles, (size_t)(ntiles + 1) * 4));
    int32_t *t = tiles.as<int32_t>();
    if (n > 0) k_scan_tiles<<<ntiles, SCAN_T, 0, s>>>(in, n, out, t);
    else MG_CUDA(cudaMemsetAsync(t, 0, 4, s));
    k_scan_part<<<1, SCAN_T, 0, s>>>(t, n > 0 ? ntiles : 1, out + n);
    if (n > 0) k_scan_add<<<ntiles, 256, 0, s>>>(out, n, t);
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}

void hub_free(mg_graph *g)
{
    HubSplit &h = g->hub;
    DevBuf *bufs[] = {&h.hoff, &h.toff, &h.hrows, &h.hcol, &h.tcol, &h.rstart, &h.crow, &h.chead,
                      &h.ctail, &h.cstart, &h.cnext, &h.clong, &h.hsum, &h.tmp0, &h.tmp1, &h.tiles, &h.err};
    for (DevBuf *b : bufs) dev_free(*b);
    h = HubSplit();
}

static std::atomic<uint64_t> g_hub_builds{0};

mg_status hub_prepare(mg_graph *g)
{
    HubSplit &h = g->hub;
    if (h.valid) return MG_OK;
    h.gen = ++g_hub_builds;
    cudaStream_t s = g->stream;
    const int32_t n = g->nv;
    const int64_t m = g->ne;
    h.use = false;
    h.H = std::min<int32_t>(HUB_MAX, n & ~3);
    if (n == 0 || m == 0 || h.H < 4) {
        h.valid = true;
        return MG_OK;
    }
    const int32_t *prow = g->trow, *pcol = g->tcol;
    MG_TRY(dev_alloc(h.tmp0, (size_t)(n + 1) * 4));   // hub edges per row, later starts per chunk
    MG_TRY(dev_alloc(h.tmp1, (size_t)(n + 1) * 4));   // has-hub-edges flags
    MG_TRY(dev_alloc(h.hoff, (size_t)(n + 1) * 4));
    MG_TRY(dev_alloc(h.toff, (size_t)(n + 1) * 4));
    const int grid = g->num_sms * 8;
    k_hub_count<<<grid, 256, 0, s>>>(n, prow, pcol, h.H, h.tmp0.as<int32_t>(), h.tmp1.as<int32_t>());
    MG_CUDA(cudaGetLastError());
    MG_TRY(scan_excl(h.tmp0.as<int32_t>(), n, h.hoff.as<int32_t>(), h.tiles, s));
    // hub-row indices go into toff for now (rewritten by the scatter)
    MG_TRY(scan_excl(h.tmp1.as<int32_t>(), n, h.toff.as<int32_t>(), h.tiles, s));
    int32_t tot[2] = {0, 0};
    MG_CUDA(cudaMemcpyAsync(&tot[0], h.hoff.as<int32_t>() + n, 4, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(&tot[1], h.toff.as<int32_t>() + n, 4, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    h.mh = tot[0];
    h.nrows = tot[1];
    // the split pays when a quarter of the edges or more come from the hubs
    if (h.mh * 4 < m) {
        dev_free(h.tmp0);
        dev_free(h.tmp1);
        h.valid = true;
        return MG_OK;
    }
    h.nchunks = (int32_t)((h.mh + HUB_CHUNK - 1) / HUB_CHUNK);
    const int64_t padded = (int64_t)h.nchunks * HUB_CHUNK;
    MG_TRY(dev_alloc(h.hcol, (size_t)padded * 2 + 16));
    MG_TRY(dev_alloc(h.tcol, (size_t)std::max<int64_t>(m - h.mh, 1) * 4 + 16));
    MG_TRY(dev_alloc(h.hrows, (size_t)std::max(h.nrows, 1) * 4));
    MG_TRY(dev_alloc(h.rstart, (size_t)h.nchunks * 32 + 16));
    MG_TRY(dev_alloc(h.crow, (size_t)(h.nchunks + 1) * 4));
    MG_TRY(dev_alloc(h.chead, (size_t)h.nchunks * 4));
    MG_TRY(dev_alloc(h.ctail, (size_t)h.nchunks * 4));
    MG_TRY(dev_alloc(h.cstart, (size_t)h.nchunks * 4));
    MG_TRY(dev_alloc(h.hsum, (size_t)n * 4));
    MG_TRY(dev_alloc(h.err, 16));
    MG_TRY(dev_alloc(h.tmp0, (size_t)(std::max(n, h.nchunks) + 1) * 4));   // starts per chunk
    // hub-row indices: copy out of toff before the scatter rewrites it
    MG_TRY(dev_alloc(h.tmp1, (size_t)(n + 1) * 4));
    MG_CUDA(cudaMemcpyAsync(h.tmp1.p, h.toff.p, (size_t)(n + 1) * 4, cudaMemcpyDeviceToDevice, s));
    MG_CUDA(cudaMemsetAsync(h.rstart.p, 0, (size_t)h.nchunks * 32, s));
    MG_CUDA(cudaMemsetAsync(h.hsum.p, 0, (size_t)n * 4, s));
    MG_CUDA(cudaMemsetAsync(h.err.p, 0, 16, s));
    k_hub_scatter<<<grid, 256, 0, s>>>(n, prow, pcol, h.H, h.hoff.as<int32_t>(), h.tmp1.as<int32_t>(),
                                       h.hcol.as<uint16_t>(), h.tcol.as<int32_t>(), h.toff.as<int32_t>(),
                                       h.hrows.as<int32_t>(), h.rstart.as<uint32_t>());
    if (padded > h.mh) k_hub_pad<<<1, 256, 0, s>>>(h.hcol.as<uint16_t>(), h.mh, padded, h.H);
    k_chunk_starts<<<grid, 256, 0, s>>>(h.rstart.as<uint32_t>(), h.nchunks, h.tmp0.as<int32_t>());
    MG_CUDA(cudaGetLastError());
    MG_TRY(scan_excl(h.tmp0.as<int32_t>(), h.nchunks, h.crow.as<int32_t>(), h.tiles, s));
    MG_TRY(dev_alloc(h.cnext, (size_t)h.nchunks * 4));
    MG_TRY(dev_alloc(h.clong, (size_t)h.nchunks * 4 + 4));   // [0]: count, then the chunk ids
    MG_CUDA(cudaMemsetAsync(h.clong.p, 0, 4, s));
    k_hub_spans<<<grid, 256, 0, s>>>(h.tmp0.as<int32_t>(), h.nchunks, h.cnext.as<int32_t>(),
                                     h.clong.as<int32_t>() + 1, h.clong.as<int32_t>());
    MG_CUDA(cudaGetLastError());
    MG_CUDA(cudaMemcpyAsync(&h.nlong, h.clong.p, 4, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    dev_free(h.tmp0);
    dev_free(h.tmp1);
    h.use = true;
    h.valid = true;
    return MG_OK;
}

size_t hub_smem_bytes(const mg_graph *g) { return (size_t)(g->hub.H + 4) * 4; }

mg_status hub_launch(mg_graph *g, const float *c0, const float *c1, const int32_t *cur, const int32_t *more,
                     const int32_t *off, cudaStream_t st, int slot_sweep, int slot_fix)
{
    HubSplit &h = g->hub;
    HubArgs a;
    std::memset(&a, 0, sizeof(a));
    a.hcol = h.hcol.as<uint16_t>();
    a.rstart = h.rstart.as<uint32_t>();
    a.crow = h.crow.as<int32_t>();
    a.hrows = h.hrows.as<int32_t>();
    a.c[0] = c0;
    a.c[1] = c1;
    a.cur = cur;
    a.more = more;
    a.off = off;
    a.hsum = h.hsum.as<float>();
    a.chead = h.chead.as<float>();
    a.ctail = h.ctail.as<float>();
    a.cstart = h.cstart.as<int32_t>();
    a.cnext = h.cnext.as<int32_t>();
    a.clong = h.clong.as<int32_t>() + 1;
    a.nlong = h.nlong;
    a.err = h.err.as<int32_t>();
    a.H = h.H;
    a.nchunks = h.nchunks;
    const size_t smem = hub_smem_bytes(g);
    MG_CUDA(cudaFuncSetAttribute(k_hub_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    Profiler &P = g->prof;
    P.begin(slot_sweep);
    k_hub_sweep<<<g->num_sms, HUB_THREADS, smem, st>>>(a);
    P.end();
    P.begin(slot_fix);
    k_hub_fix<<<std::max(1, std::min(g->num_sms * 4, (h.nchunks + 255) / 256)), 256, 0, st>>>(a);
    P.end();
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}

// the bulk-copy wait of some sweep ran out (read after the run)
mg_status hub_check(mg_graph *g)
{
    if (!g->hub.use) return MG_OK;
    int32_t e = 0;
    MG_CUDA(cudaMemcpyAsync(&e, g->hub.err.p, 4, cudaMemcpyDeviceToHost, g->stream));
    MG_CUDA(cudaStreamSynchronize(g->stream));
    if (e) {
        MG_CUDA(cudaMemsetAsync(g->hub.err.p, 0, 4, g->stream));
        return fail(MG_ERR_CUDA, "PageRank hub sweep: shared-memory staging did not complete");
    }
    return MG_OK;
}

}  // namespace mgi
