// mg_hub.cu -- shared-memory segmented pull for PageRank sweeps.
//
// The reference turns the random gathers of its dense PageRank phases into
// partition-local work: edges are regrouped into 16-bit tile streams by
// source partition (gen_structure.cu:1534-1947, sp1/sp2/mapper) and each
// partition's values are summed in shared memory (processi.cu:682-894,
// _phase1/_phase2).  Re-derived for GB300: the source ids are cut into
// segments of H = SEG_H vertices (the most a CTA's 227 KB of shared memory
// holds as FP32 contributions, 224 KB), and each pull row's in-edges are
// grouped by segment once per layout:
//   segment streams : for segment s, the rows that have in-edges from it
//                     (ascending), each row's edges from s as 16-bit local
//                     ids (id - s*H), padded to whole 1024-edge chunks; a
//                     bitmap marks the first edge of every (row, segment)
//                     pair; slot[] gives each pair its place in P;
//   P, pair_off     : the pairs' partial sums in row-major order (row v's
//                     pairs at P[pair_off[v] .. pair_off[v+1]), segments
//                     ascending), summed by the row's finish;
//   tail            : in-edges from ids beyond the last segment (graphs
//                     with more than SEG_MAX segments' worth of vertices),
//                     int32 ids gathered through L2 by the degree-binned
//                     sweep.
// One sweep: k_hub_sweep streams the chunks -- each CTA a contiguous,
// edge-balanced range, staging the contributions c[s*H, (s+1)*H) of every
// segment its range enters with bulk copies (cp.async.bulk on an mbarrier),
// each warp a 1024-edge chunk at a time: every lane takes 32 consecutive
// edges with four 128-bit loads and gathers from shared memory, a segmented
// sum (per lane, then a shuffle tree across lanes) gives every pair that
// ends inside the chunk its total; k_hub_fix finishes the pairs that run
// past their chunk (FP64, fixed order).  (With 8 edges per lane the chunk's
// fixed work -- the cross-lane scans and carries -- made the kernel
// issue-bound: ~350 warp instructions per 256 edges.)  Sums are formed in
// a fixed order, so sweeps are reproducible.
//
// Per sweep the streams move 2 B per edge plus 1 bit per edge and 4 B per
// pair, instead of 4 B of ids and a 32-byte L2 sector per gather.

#include "mg_device.cuh"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <functional>
#include <thread>

namespace {

constexpr int32_t SEG_H = 57344;    // vertices per segment: 224 KB of FP32 contributions
constexpr int32_t SEG_MAX = 64;     // segments at most; ids beyond stay in the L2 tail
constexpr int HUB_CHUNK = 1024;     // edges per warp chunk: 32 per lane
constexpr int HUB_THREADS = 1024;   // one CTA per SM (shared memory bound)
constexpr long long HUB_WAIT_LIMIT = 20000000ll;  // clock64 cycles (~10 ms) for a bulk copy
constexpr int32_t FIX_SHORT = 8;    // carry spans up to this many chunks: a thread each
constexpr int64_t START_COST = 32;  // a pair start's cost in edges, for balancing CTA ranges

struct HubArgs {
    const uint16_t *hcol;     // segment streams (each padded to whole chunks), segment-major
    const uint32_t *rstart;   // bits: first edge of each (row, segment) pair
    const int32_t *crow;      // [nchunks+1] pair index (segment-major) of each chunk's first start
    const int32_t *slot;      // per pair (segment-major): its place in P
    const int32_t *segchunk;  // [nseg+1] first chunk of each segment
    const int32_t *cta_lo;    // [grid+1] each CTA's chunk range, balanced by edges + starts
    const float *c[2];        // contributions (ping-pong, ctl selects)
    const int32_t *cur;       // current iterate index (loop control block)
    const int32_t *more;      // loop continue flag
    const int32_t *off;       // non-zero: sweeps run elsewhere (queue sweeps)
    float *P;                 // pair partial sums, row-major
    float *chead, *ctail;     // per chunk: sum before its first start / of its open last pair
    int32_t *cstart;          // per chunk: has a start
    const int32_t *cnext;     // per chunk with a start: the next chunk with one (nchunks: none)
    const int32_t *clong;     // chunks whose last pair spans more than FIX_SHORT chunks
    int32_t nlong;
    int32_t *err;             // a bulk copy wait ran out
    int32_t n, H, nseg, nchunks;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}

// Stage `bytes` (a multiple of 16) from src into s_c with bulk copies
// completing on the mbarrier (phase `parity`).  Thread 0 waits, bounded by
// HUB_WAIT_LIMIT cycles; on timeout it sets *err, waits again (bounded)
// for the copies to land, and the CTA returns false.
__device__ __forceinline__ bool stage_segment(float *s_c, const float *src, uint32_t bytes, uint32_t bar,
                                              uint32_t parity, int32_t *err)
{
    __shared__ int s_ok;
    __syncthreads();   // every warp is done with the previous segment
    if (threadIdx.x == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
        constexpr uint32_t PIECE = 32768;
        for (uint32_t off = 0; off < bytes; off += PIECE) {
            const uint32_t sz = min(PIECE, bytes - off);
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(reinterpret_cast<char *>(s_c) + off)),
                "l"(reinterpret_cast<const char *>(src) + off), "r"(sz), "r"(bar)
                : "memory");
        }
        bool ok = true;
        const long long t0 = clock64();
        while (!mbar_try(bar, parity)) {
            if (clock64() - t0 > HUB_WAIT_LIMIT) {
                ok = false;
                break;
            }
        }
        if (!ok) {
            atomicExch(err, 1);
            const long long t1 = clock64();
            while (!mbar_try(bar, parity) && clock64() - t1 < HUB_WAIT_LIMIT) {
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// One chunk of HUB_CHUNK = 1024 edges: every lane takes 32 consecutive
// edges (four 128-bit loads of 16-bit ids) and their 32 start bits (one
// word), gathers from shared memory and forms segmented sums; the pair
// totals that end inside the lane go straight to P, the open ends are joined
// across lanes by a shuffle tree, and the chunk's carries go to
// chead / ctail / cstart.
__device__ __forceinline__ void sweep_chunk(const HubArgs &a, const float *s_c, int32_t ch, const uint4 (&cols)[4],
                                            uint32_t bits, int32_t crow)
{
    const int lane = threadIdx.x & 31;
    // pair index of this lane's first start
    const int nst = __popc(bits);
    int32_t before = nst;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, before, o);
        if (lane >= o) before += t;
    }
    before -= nst;
    int32_t k = crow + before - 1;   // pair index of the open pair (after its start)
    float head = 0.0f, run = 0.0f;
    bool started = false;
    if (bits == 0) {
        // no pair starts in this lane: its 32 edges all continue the open
        // pair; summed as a pairwise tree (the same adds, a rounding error of
        // five steps instead of 32: long hub sums stay steady from sweep to
        // sweep, which the FP32 fixed-point iteration needs to settle)
        float t[16];
#pragma unroll
        for (int g = 0; g < 4; g++) {
            const uint32_t w32[4] = {cols[g].x, cols[g].y, cols[g].z, cols[g].w};
#pragma unroll
            for (int i = 0; i < 4; i++)
                t[4 * g + i] = s_c[w32[i] & 0xffffu] + s_c[w32[i] >> 16];
        }
#pragma unroll
        for (int w = 8; w > 0; w >>= 1)
#pragma unroll
            for (int i = 0; i < w; i++) t[i] = t[i] + t[i + w];
        run = t[0];   // head = run below: the lane's whole sum continues the open pair
    } else {
#pragma unroll
        for (int g = 0; g < 4; g++) {
            const uint32_t w32[4] = {cols[g].x, cols[g].y, cols[g].z, cols[g].w};
            float v[8];
#pragma unroll
            for (int i = 0; i < 8; i++) v[i] = s_c[(w32[i >> 1] >> ((i & 1) * 16)) & 0xffffu];
            // branch-free segmented sums: outv[i] is the total of the pair
            // that ends just before edge 8g+i (outf[i]: it started in this
            // lane); the slots of the group are loaded together, then stored to
            float outv[8];
            bool outf[8];
            int32_t oidx[8];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const bool st = (bits >> (8 * g + i)) & 1u;
                outf[i] = st && started;
                outv[i] = run;
                oidx[i] = k;
                head = (st && !started) ? run : head;
                run = st ? 0.0f : run;
                started = started || st;
                k += st ? 1 : 0;
                run += v[i];
            }
            int32_t sl[8];
#pragma unroll
            for (int i = 0; i < 8; i++)
                if (outf[i]) sl[i] = __ldg(&a.slot[oidx[i]]);
#pragma unroll
            for (int i = 0; i < 8; i++)
                if (outf[i]) a.P[sl[i]] = outv[i];
        }
    }
    if (!started) head = run;
    // T = sum of heads from this lane up to and including the first lane
    // (>= this one) that has a start
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
        if (closed) a.P[__ldg(&a.slot[k])] = total;
        else a.ctail[ch] = total;   // the chunk's last pair runs on
    }
    if (lane == 0) {
        a.chead[ch] = T;
        a.cstart[ch] = any != 0u;
    }
}

__global__ void __launch_bounds__(HUB_THREADS, 1) k_hub_sweep(HubArgs a)
{
    extern __shared__ __align__(128) float s_c[];   // [H + 4]
    __shared__ __align__(8) uint64_t mbar;
    if (__ldg(a.more) == 0 || __ldg(a.off) != 0) return;
    const float *c = __ldg(a.cur) ? a.c[1] : a.c[0];
    const uint32_t bar = smem_u32(&mbar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < 4) s_c[a.H + threadIdx.x] = 0.0f;   // the padding id's slot
    // this CTA's chunk range (balanced by edges and pair starts), cut at
    // segment boundaries
    const int32_t c_lo = __ldg(&a.cta_lo[blockIdx.x]), c_hi = __ldg(&a.cta_lo[blockIdx.x + 1]);
    const int32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int32_t NW = HUB_THREADS / 32;
    uint32_t phase = 0;
    int32_t s = 0;
    while (s < a.nseg && __ldg(&a.segchunk[s + 1]) <= c_lo) s++;
    for (int32_t lo = c_lo; lo < c_hi && s < a.nseg; s++) {
        const int32_t hi = min(c_hi, __ldg(&a.segchunk[s + 1]));
        if (hi <= lo) continue;
        const int32_t base = s * a.H;
        const int32_t len = min(a.H, a.n - base);
        if (!stage_segment(s_c, c + base, (uint32_t)((len + 3) & ~3) * 4u, bar, phase, a.err)) return;
        phase ^= 1u;
        for (int32_t ch = lo + warp; ch < hi; ch += NW) {
            const uint4 *src = reinterpret_cast<const uint4 *>(a.hcol + (int64_t)ch * HUB_CHUNK) + lane * 4;
            uint4 cols[4];
#pragma unroll
            for (int g = 0; g < 4; g++) cols[g] = __ldcs(src + g);
            const uint32_t bits = __ldcs(&a.rstart[(int64_t)ch * 32 + lane]);
            sweep_chunk(a, s_c, ch, cols, bits, __ldg(&a.crow[ch]));
        }
        lo = hi;
    }
}

// pairs that run past their chunk: the open tail plus the heads of the
// following chunks up to and including the next chunk with a start
// (cnext, fixed by the layout), summed in FP64 and rounded once: a hub row
// can span hundreds of chunks, and an FP32 running sum of their heads would
// carry rounding of a few 1e-6 that moves from sweep to sweep.  Spans of up
// to FIX_SHORT chunks take a thread each; longer ones (clong) a warp each,
// lane-strided then a fixed shuffle tree.  crow[ch + 1] - 1 is the pair
// index of chunk ch's last start.
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
        a.P[__ldg(&a.slot[__ldg(&a.crow[ch + 1]) - 1])] = (float)total;
    }
    const int lane = threadIdx.x & 31;
    for (int32_t i = tid >> 5; i < a.nlong; i += nth >> 5) {
        const int32_t ch = __ldg(&a.clong[i]);
        const int32_t last = min(__ldg(&a.cnext[ch]), a.nchunks - 1);
        double t = 0.0;
        for (int32_t k = ch + 1 + lane; k <= last; k += 32) t += a.chead[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) a.P[__ldg(&a.slot[__ldg(&a.crow[ch + 1]) - 1])] = (float)(t + (double)a.ctail[ch]);
    }
}

}  // namespace

namespace mgi {

void hub_free(mg_graph *g)
{
    HubSplit &h = g->hub;
    DevBuf *bufs[] = {&h.hcol, &h.rstart, &h.crow, &h.slot, &h.segchunk, &h.cta_lo, &h.pair_off, &h.P, &h.toff,
                      &h.tcol, &h.chead, &h.ctail, &h.cstart, &h.cnext, &h.clong, &h.err};
    for (DevBuf *b : bufs) dev_free(*b);
    h = HubSplit();
}

static std::atomic<uint64_t> g_hub_builds{0};

// Build the segmented layout from the pull CSR (copied back from the
// device): row-parallel host passes over the edges (count, then write),
// each thread a contiguous row range whose share of every segment's stream
// is contiguous too, so the streams come out segment-major with rows
// ascending.
mg_status hub_prepare(mg_graph *g)
{
    HubSplit &h = g->hub;
    if (h.valid) return MG_OK;
    h.gen = ++g_hub_builds;
    h.use = false;
    cudaStream_t s = g->stream;
    const int32_t n = g->nv;
    const int64_t m = g->ne;
    if (n < 4 || m == 0) {
        h.valid = true;
        return MG_OK;
    }
    const int32_t H = SEG_H;
    const int32_t nseg = std::min<int32_t>(SEG_MAX, (n + H - 1) / H);
    const int64_t cover = std::min<int64_t>(n, (int64_t)nseg * H);
    std::vector<int32_t> prow((size_t)n + 1), pcol((size_t)m);
    MG_CUDA(cudaMemcpyAsync(prow.data(), g->trow, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(pcol.data(), g->tcol, (size_t)m * 4, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    const int nt = std::max(1, std::min(host_threads(0), 32));
    // row ranges of equal edge counts
    std::vector<int32_t> rlo((size_t)nt + 1, n);
    rlo[0] = 0;
    for (int t = 1; t < nt; t++) {
        const int64_t goal = m * t / nt;
        rlo[t] = (int32_t)(std::lower_bound(prow.begin(), prow.end(), (int32_t)goal) - prow.begin());
        rlo[t] = std::min(std::max(rlo[t], rlo[t - 1]), n);
    }
    auto run = [&](const std::function<void(int)> &fn) {
        std::vector<std::thread> th;
        for (int t = 1; t < nt; t++) th.emplace_back(fn, t);
        fn(0);
        for (auto &x : th) x.join();
    };
    // pass 1: per thread and segment the edges and pairs; per row its pairs
    // and tail edges
    std::vector<int64_t> tedge((size_t)nt * nseg, 0), tpair((size_t)nt * nseg, 0);
    std::vector<int32_t> npair((size_t)n + 1, 0), ntail((size_t)n + 1, 0);
    run([&](int t) {
        int64_t *te = &tedge[(size_t)t * nseg], *tp = &tpair[(size_t)t * nseg];
        for (int32_t v = rlo[t]; v < rlo[t + 1]; v++) {
            uint64_t mask = 0;
            int32_t nt_ = 0;
            for (int32_t p = prow[v]; p < prow[v + 1]; p++) {
                const int32_t c = pcol[p];
                if (c < cover) {
                    const int sg = c / H;
                    te[sg]++;
                    mask |= 1ull << sg;
                } else {
                    nt_++;
                }
            }
            npair[v] = __builtin_popcountll(mask);
            ntail[v] = nt_;
            for (uint64_t mm = mask; mm; mm &= mm - 1) tp[__builtin_ctzll(mm)]++;
        }
    });
    int64_t covered = 0;
    for (int64_t x : tedge) covered += x;
    // the segmented pull pays when a quarter of the edges or more are covered
    if (covered * 4 < m) {
        h.valid = true;
        return MG_OK;
    }
    // offsets: segments' chunks, per-thread shares, row-major pair slots, tail rows
    std::vector<int32_t> segchunk((size_t)nseg + 1, 0);
    std::vector<int64_t> segpair((size_t)nseg + 1, 0);
    std::vector<int64_t> toffE((size_t)nt * nseg), toffP((size_t)nt * nseg);
    for (int sg = 0; sg < nseg; sg++) {
        int64_t e = 0, pp = 0;
        for (int t = 0; t < nt; t++) {
            toffE[(size_t)t * nseg + sg] = e;
            toffP[(size_t)t * nseg + sg] = segpair[sg] + pp;
            e += tedge[(size_t)t * nseg + sg];
            pp += tpair[(size_t)t * nseg + sg];
        }
        segchunk[sg + 1] = segchunk[sg] + (int32_t)((e + HUB_CHUNK - 1) / HUB_CHUNK);
        segpair[sg + 1] = segpair[sg] + pp;
    }
    const int32_t nchunks = segchunk[nseg];
    const int64_t npairs = segpair[nseg];
    if (npairs > INT32_MAX || (int64_t)nchunks * HUB_CHUNK > INT32_MAX)
        return fail(MG_ERR_RANGE, "segmented PageRank layout too large");
    std::vector<int32_t> pair_off((size_t)n + 1, 0), toff((size_t)n + 1, 0);
    for (int32_t v = 0; v < n; v++) {
        pair_off[v + 1] = pair_off[v] + npair[v];
        toff[v + 1] = toff[v] + ntail[v];
    }
    std::vector<uint16_t> hcol((size_t)nchunks * HUB_CHUNK, (uint16_t)H);
    std::vector<uint32_t> rstart((size_t)nchunks * (HUB_CHUNK / 32), 0u);
    std::vector<int32_t> slot((size_t)std::max<int64_t>(npairs, 1)), tcol((size_t)std::max<int32_t>(toff[n], 1));
    // pass 2: every row's edges into its segments' streams.  A thread's
    // share of a segment's stream starts on a chunk of its own only by
    // chance, so the row-start bits are set with atomic ORs.
    std::vector<std::atomic<uint32_t>> rbits((size_t)nchunks * (HUB_CHUNK / 32));
    for (auto &b : rbits) b.store(0u, std::memory_order_relaxed);
    run([&](int t) {
        std::vector<int64_t> ep((size_t)nseg), pp((size_t)nseg);
        for (int sg = 0; sg < nseg; sg++) {
            ep[sg] = (int64_t)segchunk[sg] * HUB_CHUNK + toffE[(size_t)t * nseg + sg];
            pp[sg] = toffP[(size_t)t * nseg + sg];
        }
        int32_t cnt[SEG_MAX];
        int64_t start[SEG_MAX];
        for (int32_t v = rlo[t]; v < rlo[t + 1]; v++) {
            std::memset(cnt, 0, sizeof(int32_t) * nseg);
            int32_t tp = toff[v];
            for (int32_t p = prow[v]; p < prow[v + 1]; p++) {
                const int32_t c = pcol[p];
                if (c < cover) cnt[c / H]++;
                else tcol[tp++] = c;
            }
            int32_t rank = 0;
            for (int sg = 0; sg < nseg; sg++) {
                if (!cnt[sg]) continue;
                const int64_t e0 = ep[sg];
                start[sg] = e0;
                rbits[(size_t)(e0 >> 5)].fetch_or(1u << (e0 & 31), std::memory_order_relaxed);
                slot[pp[sg]++] = pair_off[v] + rank++;
                ep[sg] += cnt[sg];
            }
            for (int32_t p = prow[v]; p < prow[v + 1]; p++) {
                const int32_t c = pcol[p];
                if (c < cover) {
                    const int sg = c / H;
                    hcol[start[sg]++] = (uint16_t)(c - sg * H);
                }
            }
        }
    });
    for (size_t i = 0; i < rstart.size(); i++) rstart[i] = rbits[i].load(std::memory_order_relaxed);
    // pair index of every chunk's first start; span of every chunk's last pair
    std::vector<int32_t> crow((size_t)nchunks + 1, 0), cnext((size_t)std::max(nchunks, 1), 0), clong;
    for (int32_t ch = 0; ch < nchunks; ch++) {
        int32_t k = 0;
        for (int w = 0; w < HUB_CHUNK / 32; w++) k += __builtin_popcount(rstart[(size_t)ch * (HUB_CHUNK / 32) + w]);
        crow[ch + 1] = crow[ch] + k;
    }
    {
        int32_t next = nchunks;
        for (int32_t ch = nchunks - 1; ch >= 0; ch--) {
            cnext[ch] = next;
            if (crow[ch + 1] > crow[ch]) {
                if (std::min(next, nchunks - 1) - ch > FIX_SHORT) clong.push_back(ch);
                next = ch;
            }
        }
    }
    // CTA ranges: a chunk costs its 1024 edges plus START_COST per pair start
    // (the slot load and scattered store of a short pair's total); chunk
    // counts alone left one SM four times as busy as the average
    const int G = g->num_sms;
    std::vector<int32_t> cta_lo((size_t)G + 1, nchunks);
    {
        const int64_t total = (int64_t)nchunks * HUB_CHUNK + START_COST * (int64_t)crow[nchunks];
        int64_t acc = 0;
        int b = 0;
        cta_lo[0] = 0;
        for (int32_t ch = 0; ch < nchunks && b + 1 < G; ch++) {
            acc += HUB_CHUNK + START_COST * (int64_t)(crow[ch + 1] - crow[ch]);
            while (b + 1 < G && acc * G >= total * (b + 1)) cta_lo[++b] = ch + 1;
        }
        while (b + 1 <= G) cta_lo[++b] = nchunks;
    }
    auto up = [&](DevBuf &b, const void *src, size_t bytes) -> mg_status {
        MG_TRY(dev_alloc(b, std::max<size_t>(bytes, 16) + 16));
        if (bytes) MG_CUDA(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, s));
        return MG_OK;
    };
    MG_TRY(up(h.hcol, hcol.data(), hcol.size() * 2));
    MG_TRY(up(h.rstart, rstart.data(), rstart.size() * 4));
    MG_TRY(up(h.crow, crow.data(), crow.size() * 4));
    MG_TRY(up(h.slot, slot.data(), (size_t)npairs * 4));
    MG_TRY(up(h.segchunk, segchunk.data(), segchunk.size() * 4));
    MG_TRY(up(h.cta_lo, cta_lo.data(), cta_lo.size() * 4));
    MG_TRY(up(h.pair_off, pair_off.data(), pair_off.size() * 4));
    MG_TRY(up(h.toff, toff.data(), toff.size() * 4));
    MG_TRY(up(h.tcol, tcol.data(), (size_t)toff[n] * 4));
    MG_TRY(up(h.cnext, cnext.data(), (size_t)nchunks * 4));
    MG_TRY(up(h.clong, clong.data(), clong.size() * 4));
    MG_TRY(dev_alloc(h.P, (size_t)std::max<int64_t>(npairs, 1) * 4));
    MG_TRY(dev_alloc(h.chead, (size_t)std::max(nchunks, 1) * 4));
    MG_TRY(dev_alloc(h.ctail, (size_t)std::max(nchunks, 1) * 4));
    MG_TRY(dev_alloc(h.cstart, (size_t)std::max(nchunks, 1) * 4));
    MG_TRY(dev_alloc(h.err, 16));
    MG_CUDA(cudaMemsetAsync(h.err.p, 0, 16, s));
    MG_CUDA(cudaStreamSynchronize(s));
    h.H = H;
    h.nseg = nseg;
    h.nchunks = nchunks;
    h.npairs = npairs;
    h.nlong = (int32_t)clong.size();
    h.covered = covered;
    h.ntail = toff[n];
    h.grid = G;
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
    a.slot = h.slot.as<int32_t>();
    a.segchunk = h.segchunk.as<int32_t>();
    a.cta_lo = h.cta_lo.as<int32_t>();
    a.c[0] = c0;
    a.c[1] = c1;
    a.cur = cur;
    a.more = more;
    a.off = off;
    a.P = h.P.as<float>();
    a.chead = h.chead.as<float>();
    a.ctail = h.ctail.as<float>();
    a.cstart = h.cstart.as<int32_t>();
    a.cnext = h.cnext.as<int32_t>();
    a.clong = h.clong.as<int32_t>();
    a.nlong = h.nlong;
    a.err = h.err.as<int32_t>();
    a.n = g->nv;
    a.H = h.H;
    a.nseg = h.nseg;
    a.nchunks = h.nchunks;
    const size_t smem = hub_smem_bytes(g);
    MG_CUDA(cudaFuncSetAttribute(k_hub_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    Profiler &P = g->prof;
    P.begin(slot_sweep);
    k_hub_sweep<<<h.grid, HUB_THREADS, smem, st>>>(a);
    P.end();
    P.begin(slot_fix);
    k_hub_fix<<<std::max(1, std::min(g->num_sms * 4, (h.nchunks + 255) / 256)), 256, 0, st>>>(a);
    P.end();
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}

// a bulk-copy wait of some sweep ran out (read after the run)
mg_status hub_check(mg_graph *g)
{
    if (!g->hub.use) return MG_OK;
    int32_t e = 0;
    MG_CUDA(cudaMemcpyAsync(&e, g->hub.err.p, 4, cudaMemcpyDeviceToHost, g->stream));
    MG_CUDA(cudaStreamSynchronize(g->stream));
    if (e) {
        MG_CUDA(cudaMemsetAsync(g->hub.err.p, 0, 4, g->stream));
        return fail(MG_ERR_CUDA, "PageRank segmented sweep: shared-memory staging did not complete");
    }
    return MG_OK;
}

}  // namespace mgi
