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
//   pairs, pieces   : a (row, segment) pair is the row's in-edges from the
//                     segment; it is cut into pieces of at most PIECE_MAX
//                     edges (the row's order kept);
//   warp groups     : per segment, pieces of equal length lambda are bucketed
//                     (rows ascending) and packed GROUP at a time, padded;
//                     a group stores its ids as 16-bit local ids (id - s*H)
//                     step-major, [lambda][GROUP], so each step is one
//                     coalesced 256-byte warp load (four pieces per lane);
//   P, pair_off     : the pieces' sums in row-major order (row v's pieces at
//                     P[pair_off[v] .. pair_off[v+1]), segments ascending),
//                     summed by the row's finish; pslot gives each packed
//                     piece its place in P;
//   tail            : in-edges from ids beyond the last segment (graphs
//                     with more than SEG_MAX segments' worth of vertices),
//                     int32 ids gathered through L2 by the degree-binned
//                     sweep.
// One sweep: k_hub_sweep gives each CTA a contiguous range of groups (an
// even share of the groups' cost weights: steps plus a fixed cost per group
// at first, re-weighted by mg_autotune from measured per-CTA times), stages
// the contributions c[s*H, (s+1)*H) of every segment its range enters, and
// its warps claim chunks of consecutive groups from a shared-memory counter
// and stream them: a lane adds its four pieces' edges in order from shared
// memory and stores the four totals to P.  Pieces never cross a group, so
// there are no carries between lanes, warps or CTAs; every sum is formed in
// a fixed order, whichever warp runs it, so sweeps are reproducible.
//
// Per sweep the streams move 2 B per edge (plus padding, ~2.4 % on R-MAT),
// a 4-byte slot and a 4-byte store per piece (about one piece per ten
// edges), instead of 4 B of ids and a 32-byte L2 sector per gather.  The
// row finish (k_pr_seg in mg_pr.cu) reads each row's piece sums.

#include "mg_device.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <thread>

namespace {

constexpr int32_t SEG_H = 57344;    // vertices per segment: 224 KB of FP32 contributions
constexpr int32_t SEG_MAX = 64;     // segments at most; ids beyond stay in the L2 tail
constexpr int32_t PIECE_MAX = 64;   // edges per piece at most
constexpr int32_t GROUP = 128;      // pieces per warp group: four per lane
constexpr int HUB_THREADS = 1024;   // one CTA per SM (shared memory bound)
constexpr int HUB_UNROLL = 4;       // steps (256-byte warp loads) in flight per warp
constexpr int STAGE_BATCH = 4;      // 16-byte loads in flight per thread while staging a segment
constexpr int64_t GROUP_COST = 16;  // a group's fixed cost in steps, for balancing CTA ranges
constexpr int64_t CHUNK_COST = 64;  // a chunk's cost (steps + GROUP_COST per group): the unit warps claim
                                    // (R-MAT 22 sweep: 128 -> 129-140 us, 64 -> 122 us, 32 -> 124-127, 16 -> 129-131)
// the row finish sums rows with more than FIN_WARP pieces a warp each, the
// rest a thread each (8-lane groups for rows of 5-64 pieces walked their
// rows one after another and were slower)
constexpr int32_t FIN_WARP = 32;

struct HubArgs {
    const uint2 *hdat;        // groups' ids, four 16-bit ids per lane per step
    const int32_t *goff;      // [ngroups+1] each group's first step
    const int4 *pslot;        // [ngroups*GROUP/4] the four P slots of each lane's pieces
    const int32_t *cpart;     // [grid+1] each CTA's parts
    const int32_t *pseg;      // [nparts] each part's segment
    const int32_t *pch;       // [nparts+1] each part's chunks
    const int32_t *cb;        // [nchunks+1] chunk k = groups [cb[k], cb[k+1])
    const float *c[2];        // contributions (ping-pong, ctl selects)
    const int32_t *cur;       // current iterate index (loop control block)
    const int32_t *more;      // loop continue flag
    const int32_t *off;       // non-zero: sweeps run elsewhere (queue sweeps)
    float *P;                 // piece sums, row-major
    long long *ctime;         // [grid] each CTA's clock cycles (read back to re-split the work)
    int32_t n, H, nseg;
};

// One warp streams groups [ga, gb) (contiguous in hdat): the next
// HUB_UNROLL steps are loaded while the current ones are summed, across
// group ends, so the loads run back to back instead of one latency chain per
// group.  Every edge gets one compensated add, in edge order, so a piece's
// sum does not depend on where a warp's range starts (the work split is
// re-cut from measurements; a faster pairwise add of four steps at a time,
// applied where a batch of loads fell inside one group, made the rounding
// follow the split).  The groups' first steps come from goff 32 at a time
// (one load, then shuffles); each group's slots are loaded when it starts.
__device__ __forceinline__ void stream_groups(const HubArgs &a, const float *s_c, int32_t ga, int32_t gb, int lane)
{
    constexpr unsigned FULL = 0xffffffffu;
    const uint2 *D = a.hdat + lane;
    int32_t cbase = ga;
    int32_t cg = __ldg(&a.goff[min(cbase + lane, gb)]);
    int32_t t = __shfl_sync(FULL, cg, 0);
    const int32_t tend = __ldg(&a.goff[gb]);
    int32_t g = ga;
    int32_t gend = __shfl_sync(FULL, cg, 1);
    // slots and ids are streamed once per sweep: evict-first loads keep L2
    // for the piece sums the row finish reads next
    int4 sl = __ldcs(&a.pslot[(int64_t)g * 32 + lane]);
    // compensated sums (Kahan): a piece of up to PIECE_MAX edges is exact to
    // about one rounding, so a hub row's total does not drift by a few 1e-6
    // from sweep to sweep as its inputs settle
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f, r0 = 0.0f, r1 = 0.0f, r2 = 0.0f, r3 = 0.0f;
    uint2 wc[HUB_UNROLL], wn[HUB_UNROLL];
#pragma unroll
    for (int j = 0; j < HUB_UNROLL; j++) wc[j] = t + j < tend ? __ldcs(D + (int64_t)(t + j) * 32) : make_uint2(0u, 0u);
    while (t < tend) {
#pragma unroll
        for (int j = 0; j < HUB_UNROLL; j++) {
            const int32_t q = t + HUB_UNROLL + j;
            wn[j] = q < tend ? __ldcs(D + (int64_t)q * 32) : make_uint2(0u, 0u);
        }
#pragma unroll
        for (int j = 0; j < HUB_UNROLL; j++) {
            if (t < tend) {
                mgd::kahan_add(s0, r0, s_c[wc[j].x & 0xffffu]);
                mgd::kahan_add(s1, r1, s_c[wc[j].x >> 16]);
                mgd::kahan_add(s2, r2, s_c[wc[j].y & 0xffffu]);
                mgd::kahan_add(s3, r3, s_c[wc[j].y >> 16]);
                t++;
                if (t == gend) {   // group g is complete (warp-uniform)
                    a.P[sl.x] = s0 - r0;
                    a.P[sl.y] = s1 - r1;
                    a.P[sl.z] = s2 - r2;
                    a.P[sl.w] = s3 - r3;
                    s0 = s1 = s2 = s3 = r0 = r1 = r2 = r3 = 0.0f;
                    g++;
                    if (g < gb) {
                        if (g + 1 - cbase >= 32) {
                            cbase = g + 1;
                            cg = __ldg(&a.goff[min(cbase + lane, gb)]);
                        }
                        gend = __shfl_sync(FULL, cg, g + 1 - cbase);
                        sl = __ldcs(&a.pslot[(int64_t)g * 32 + lane]);
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < HUB_UNROLL; j++) wc[j] = wn[j];
    }
}

// One sweep over every piece: each CTA walks its parts (one segment each),
// stages the segment's contributions in shared memory, and its warps claim
// the part's chunks from a shared-memory counter; the CTA's clock cycles go
// to ctime for the next re-split.
__global__ void __launch_bounds__(HUB_THREADS, 1) k_hub_sweep(HubArgs a)
{
    extern __shared__ __align__(16) float s_c[];   // [H + 4]
    if (__ldg(a.more) == 0 || __ldg(a.off) != 0) return;
    const float *c = __ldg(a.cur) ? a.c[1] : a.c[0];
    if (threadIdx.x < 4) s_c[a.H + threadIdx.x] = 0.0f;   // the padding id's slot
    __shared__ int32_t s_next;   // the part's next unclaimed chunk
    const long long t_start = clock64();
    const int32_t lane = threadIdx.x & 31;
    const int32_t p0 = __ldg(&a.cpart[blockIdx.x]), p1 = __ldg(&a.cpart[blockIdx.x + 1]);
    for (int32_t pi = p0; pi < p1; pi++) {
        const int32_t s = __ldg(&a.pseg[pi]);
        // stage c[s*H, s*H + len) (16-byte units; the arrays carry 16 bytes
        // of slack past the last vertex)
        const int32_t base = s * a.H;
        const int32_t n4 = (min(a.H, a.n - base) + 3) >> 2;
        __syncthreads();   // every warp is done with the previous segment
        const int32_t k1 = __ldg(&a.pch[pi + 1]);
        if (threadIdx.x == 0) s_next = __ldg(&a.pch[pi]);
        const float4 *src = reinterpret_cast<const float4 *>(c + base);
        float4 *dst = reinterpret_cast<float4 *>(s_c);
        // all of a thread's loads in flight at once, in batches of STAGE_BATCH
        for (int32_t i0 = threadIdx.x; i0 < n4; i0 += STAGE_BATCH * HUB_THREADS) {
            float4 v[STAGE_BATCH];
#pragma unroll
            for (int k = 0; k < STAGE_BATCH; k++) {
                const int32_t i = i0 + k * HUB_THREADS;
                if (i < n4) v[k] = __ldcg(&src[i]);
            }
#pragma unroll
            for (int k = 0; k < STAGE_BATCH; k++) {
                const int32_t i = i0 + k * HUB_THREADS;
                if (i < n4) dst[i] = v[k];
            }
        }
        __syncthreads();
        // the warps claim the part's chunks in order until none is left
        while (true) {
            int32_t k = 0;
            if (lane == 0) k = atomicAdd(&s_next, 1);
            k = __shfl_sync(0xffffffffu, k, 0);
            if (k >= k1) break;
            stream_groups(a, s_c, __ldg(&a.cb[k]), __ldg(&a.cb[k + 1]), lane);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) a.ctime[blockIdx.x] = clock64() - t_start;
}

}  // namespace

namespace mgi {

static std::atomic<uint64_t> g_hub_builds{0};

void hub_free(mg_graph *g)
{
    HubSplit &h = g->hub;
    DevBuf *bufs[] = {&h.hdat, &h.goff, &h.pslot, &h.cpart, &h.pseg, &h.pch, &h.cb, &h.ctime, &h.pair_off, &h.P, &h.toff,
                      &h.tcol, &h.fin};
    for (DevBuf *b : bufs) dev_free(*b);
    h = HubSplit();
}

// Split the groups among the CTAs by the groups' cost weights h.w: each
// CTA an even share of the total weight (contiguous groups), cut at
// segment boundaries into parts and each part into chunks of about
// CHUNK_COST that the CTA's warps claim one at a time.  The captured loops
// that launch the sweep take the new split (the build number changes).
static mg_status hub_split(mg_graph *g)
{
    HubSplit &h = g->hub;
    cudaStream_t s = g->stream;
    const int G = h.grid;
    const int32_t ngroups = (int32_t)h.hglam.size();
    const std::vector<int32_t> &segg = h.hsegg;
    std::vector<double> gcum((size_t)ngroups + 1, 0.0);
    for (int32_t q = 0; q < ngroups; q++) gcum[q + 1] = gcum[q] + h.w[q];
    auto cut = [&](int32_t lo, int32_t hi, int parts, int32_t *out) {
        // out[0..parts]: boundaries in [lo, hi] of equal weight
        out[0] = lo;
        for (int k = 1; k < parts; k++) {
            const double goal = gcum[lo] + (gcum[hi] - gcum[lo]) * k / parts;
            int32_t b = (int32_t)(std::lower_bound(gcum.begin() + lo, gcum.begin() + hi, goal) - gcum.begin());
            out[k] = std::min(std::max(b, out[k - 1]), hi);
        }
        out[parts] = hi;
    };
    // the weight of an average group, for sizing chunks: CHUNK_COST is in
    // units of the initial weights (steps)
    double w0 = 0.0, wn = 0.0;
    for (int32_t q = 0; q < ngroups; q++) {
        w0 += (double)h.hglam[q] + (double)GROUP_COST;
        wn += h.w[q];
    }
    const double chunk_w = (double)CHUNK_COST * (w0 > 0.0 ? wn / w0 : 1.0);
    std::vector<int32_t> cta_lo((size_t)G + 1);
    cut(0, ngroups, G, cta_lo.data());
    std::vector<int32_t> cpart((size_t)G + 1, 0), pseg, pch, cb;
    for (int b = 0; b < G; b++) {
        cpart[b] = (int32_t)pseg.size();
        int32_t lo = cta_lo[b];
        const int32_t hi = cta_lo[b + 1];
        while (lo < hi) {
            const int32_t sg = (int32_t)(std::upper_bound(segg.begin(), segg.end(), lo) - segg.begin()) - 1;
            const int32_t e = std::min(hi, segg[sg + 1]);
            pseg.push_back(sg);
            pch.push_back((int32_t)cb.size());
            const double cost = gcum[e] - gcum[lo];
            const int nch = (int)std::max<int64_t>(1, std::min<int64_t>(e - lo, (int64_t)std::ceil(cost / chunk_w)));
            std::vector<int32_t> bnd((size_t)nch + 1);
            cut(lo, e, nch, bnd.data());
            for (int k = 0; k < nch; k++)
                if (bnd[k] < bnd[k + 1]) cb.push_back(bnd[k]);
            lo = e;
        }
    }
    cpart[G] = (int32_t)pseg.size();
    pch.push_back((int32_t)cb.size());
    cb.push_back(ngroups);
    auto up = [&](DevBuf &b, const void *src, size_t bytes) -> mg_status {
        MG_TRY(dev_alloc(b, std::max<size_t>(bytes, 16) + 16));
        if (bytes) MG_CUDA(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, s));
        return MG_OK;
    };
    MG_TRY(up(h.cpart, cpart.data(), cpart.size() * 4));
    MG_TRY(up(h.pseg, pseg.data(), pseg.size() * 4));
    MG_TRY(up(h.pch, pch.data(), pch.size() * 4));
    MG_TRY(up(h.cb, cb.data(), cb.size() * 4));
    MG_CUDA(cudaStreamSynchronize(s));   // the host vectors go out of scope
    h.gen = ++g_hub_builds;
    return MG_OK;
}

// Build the segmented layout from a pull CSR on the host (prow [n+1], pcol
// [m], engine ids): row-parallel passes over the edges (count, then write)
// on nt threads, each a contiguous row range whose pieces take consecutive
// places in every (segment, length) bucket, so buckets come out rows
// ascending and the layout does not depend on nt.  o.use stays false when a
// quarter of the edges or fewer fall in the segments.
struct HubHost {
    bool use = false;
    int32_t H = 0, nseg = 0, nfw = 0;
    int64_t covered = 0, npieces = 0;
    std::vector<uint16_t> hdat;
    std::vector<int32_t> goff, pslot, glam, segg, pair_off, toff, tcol, fin;
};

static mg_status build_hub(const std::vector<int32_t> &prow, const std::vector<int32_t> &pcol, int32_t n, int64_t m,
                           int nt, HubHost &o)
{
    const int32_t H = SEG_H;
    const int32_t nseg = std::min<int32_t>(SEG_MAX, (n + H - 1) / H);
    const int64_t cover = std::min<int64_t>(n, (int64_t)nseg * H);
    constexpr int32_t L = PIECE_MAX;
    o = HubHost();
    o.H = H;
    o.nseg = nseg;
    nt = std::max(1, std::min(nt, 32));
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
    // bucket (segment sg, piece length lam) of thread t: bc[(t * nseg + sg) * (L + 1) + lam]
    const size_t NB = (size_t)nseg * (L + 1);
    std::vector<int64_t> bc((size_t)nt * NB, 0), tcov((size_t)nt, 0);
    std::vector<int32_t> npc((size_t)n, 0), ntl((size_t)n, 0);
    // pass 1: per row its pieces and tail edges; per thread its bucket counts
    run([&](int t) {
        int64_t *b = &bc[(size_t)t * NB];
        int32_t cnt[SEG_MAX];
        int64_t cov = 0;
        for (int32_t v = rlo[t]; v < rlo[t + 1]; v++) {
            std::memset(cnt, 0, sizeof(int32_t) * nseg);
            int32_t tl = 0;
            for (int32_t p = prow[v]; p < prow[v + 1]; p++) {
                const int32_t c = pcol[p];
                if (c < cover) cnt[c / H]++;
                else tl++;
            }
            int32_t pieces = 0;
            for (int sg = 0; sg < nseg; sg++) {
                if (!cnt[sg]) continue;
                cov += cnt[sg];
                const int32_t full = cnt[sg] / L, rem = cnt[sg] % L;
                b[(size_t)sg * (L + 1) + L] += full;
                if (rem) b[(size_t)sg * (L + 1) + rem]++;
                pieces += full + (rem ? 1 : 0);
            }
            npc[v] = pieces;
            ntl[v] = tl;
        }
        tcov[t] = cov;
    });
    int64_t covered = 0;
    for (int64_t x : tcov) covered += x;
    o.covered = covered;
    // the segmented pull pays when a quarter of the edges or more are covered
    if (covered * 4 < m) return MG_OK;
    // buckets in order: segments ascending, lengths descending; each padded
    // to whole groups.  tb: thread t's first place in its bucket.
    std::vector<int64_t> tb((size_t)nt * NB, 0);
    std::vector<int32_t> segg((size_t)nseg + 1, 0);
    std::vector<int32_t> glam;      // steps of every group
    int64_t place = 0;              // padded place of the next bucket's first piece
    for (int sg = 0; sg < nseg; sg++) {
        segg[sg] = (int32_t)glam.size();
        for (int32_t lam = L; lam >= 1; lam--) {
            const size_t k = (size_t)sg * (L + 1) + lam;
            int64_t size = 0;
            for (int t = 0; t < nt; t++) {
                tb[(size_t)t * NB + k] = place + size;
                size += bc[(size_t)t * NB + k];
            }
            const int64_t groups = (size + GROUP - 1) / GROUP;
            for (int64_t q = 0; q < groups; q++) glam.push_back(lam);
            place += groups * GROUP;
        }
    }
    const int32_t ngroups = (int32_t)glam.size();
    segg[nseg] = ngroups;
    std::vector<int64_t> goff64((size_t)ngroups + 1, 0);
    for (int32_t q = 0; q < ngroups; q++) goff64[q + 1] = goff64[q] + glam[q];
    std::vector<int32_t> pair_off((size_t)n + 1, 0), toff((size_t)n + 1, 0);
    for (int32_t v = 0; v < n; v++) {
        pair_off[v + 1] = pair_off[v] + npc[v];
        toff[v + 1] = toff[v] + ntl[v];
    }
    const int64_t npieces = pair_off[n];
    if (npieces >= INT32_MAX || goff64[ngroups] >= INT32_MAX)
        return fail(MG_ERR_RANGE, "segmented PageRank layout too large");
    std::vector<int32_t> goff(goff64.begin(), goff64.end());
    std::vector<uint16_t> hdat((size_t)goff64[ngroups] * GROUP, (uint16_t)H);
    std::vector<int32_t> pslot((size_t)ngroups * GROUP, (int32_t)npieces);
    std::vector<int32_t> tcol((size_t)toff[n]);
    // pass 2: every row's pieces into their buckets, every edge into its
    // piece's step and lane
    run([&](int t) {
        std::vector<int64_t> next(tb.begin() + (size_t)t * NB, tb.begin() + (size_t)(t + 1) * NB);
        int32_t cnt[SEG_MAX], full[SEG_MAX], e[SEG_MAX];
        int64_t qfull[SEG_MAX], qrem[SEG_MAX];
        for (int32_t v = rlo[t]; v < rlo[t + 1]; v++) {
            std::memset(cnt, 0, sizeof(int32_t) * nseg);
            int32_t tp = toff[v];
            for (int32_t p = prow[v]; p < prow[v + 1]; p++) {
                const int32_t c = pcol[p];
                if (c < cover) cnt[c / H]++;
                else tcol[tp++] = c;
            }
            int32_t slot = pair_off[v];   // the row's pieces: segments ascending, pieces in order
            for (int sg = 0; sg < nseg; sg++) {
                e[sg] = 0;
                if (!cnt[sg]) continue;
                full[sg] = cnt[sg] / L;
                const int32_t rem = cnt[sg] % L;
                int64_t &nf = next[(size_t)sg * (L + 1) + L];
                qfull[sg] = nf;
                for (int32_t i = 0; i < full[sg]; i++) pslot[(size_t)(nf++)] = slot++;
                if (rem) {
                    int64_t &nr = next[(size_t)sg * (L + 1) + rem];
                    qrem[sg] = nr;
                    pslot[(size_t)(nr++)] = slot++;
                }
            }
            for (int32_t p = prow[v]; p < prow[v + 1]; p++) {
                const int32_t c = pcol[p];
                if (c >= cover) continue;
                const int sg = c / H;
                const int32_t i = e[sg] / L, k = e[sg] % L;
                e[sg]++;
                const int64_t q = i < full[sg] ? qfull[sg] + i : qrem[sg];
                const int64_t grp = q / GROUP;
                hdat[(size_t)(goff64[grp] * GROUP + (int64_t)k * GROUP + q % GROUP)] = (uint16_t)(c - sg * H);
            }
        }
    });
    o.hdat.swap(hdat);
    o.goff.swap(goff);
    o.pslot.swap(pslot);
    o.glam.swap(glam);
    o.segg.swap(segg);
    o.pair_off.swap(pair_off);
    o.toff.swap(toff);
    o.tcol.swap(tcol);
    o.npieces = npieces;
    o.use = true;
    // rows of more than FIN_WARP pieces, which k_pr_seg sums a warp each
    // (graphs without a tail finish every row there)
    for (int32_t v = 0; v < n; v++)
        if (npc[v] > FIN_WARP) o.fin.push_back(v);
    o.nfw = (int32_t)o.fin.size();
    return MG_OK;
}

// Build the segmented layout from the pull CSR (copied back from the
// device), upload it and split the sweep's work among the CTAs.
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
    std::vector<int32_t> prow((size_t)n + 1), pcol((size_t)m);
    MG_CUDA(cudaMemcpyAsync(prow.data(), g->trow, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(pcol.data(), g->tcol, (size_t)m * 4, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    HubHost o;
    MG_TRY(build_hub(prow, pcol, n, m, host_threads(0), o));
    h.covered = o.covered;
    if (!o.use) {
        h.valid = true;
        return MG_OK;
    }
    const int32_t ngroups = (int32_t)o.glam.size();
    h.hglam = o.glam;
    h.hsegg = o.segg;
    h.w.assign((size_t)ngroups, 0.0);
    for (int32_t q = 0; q < ngroups; q++) h.w[q] = (double)o.glam[q] + (double)GROUP_COST;
    h.grid = g->num_sms;
    MG_TRY(dev_alloc(h.ctime, (size_t)h.grid * 8));
    MG_TRY(hub_split(g));
    auto up = [&](DevBuf &b, const void *src, size_t bytes) -> mg_status {
        MG_TRY(dev_alloc(b, std::max<size_t>(bytes, 16) + 16));
        if (bytes) MG_CUDA(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, s));
        return MG_OK;
    };
    MG_TRY(up(h.hdat, o.hdat.data(), o.hdat.size() * 2));
    MG_TRY(up(h.goff, o.goff.data(), o.goff.size() * 4));
    MG_TRY(up(h.pslot, o.pslot.data(), o.pslot.size() * 4));
    MG_TRY(up(h.pair_off, o.pair_off.data(), o.pair_off.size() * 4));
    MG_TRY(up(h.toff, o.toff.data(), o.toff.size() * 4));
    MG_TRY(up(h.tcol, o.tcol.data(), o.tcol.size() * 4));
    MG_TRY(up(h.fin, o.fin.data(), o.fin.size() * 4));   // at least 16 bytes even when empty
    MG_TRY(dev_alloc(h.P, (size_t)(o.npieces + 1) * 4));
    MG_CUDA(cudaStreamSynchronize(s));
    h.H = o.H;
    h.nseg = o.nseg;
    h.ngroups = ngroups;
    h.npieces = o.npieces;
    h.ntail = o.toff[n];
    h.nfw = o.nfw;
    h.fin_warp = FIN_WARP;
    h.use = true;
    h.valid = true;
    return MG_OK;
}

bool hub_covers_all(const mg_graph *g) { return (int64_t)g->nv <= (int64_t)SEG_MAX * SEG_H; }

// Re-split the sweep's work from the last sweep's per-CTA clock counts:
// every group's weight is scaled by its CTA's measured time over the
// CTA's share of the weight (normalised to the mean), so groups whose real
// cost the initial model (steps + GROUP_COST) misjudges move to other CTAs.
mg_status hub_rebalance(mg_graph *g)
{
    HubSplit &h = g->hub;
    if (!h.use) return MG_OK;
    const int G = h.grid;
    std::vector<long long> t((size_t)G);
    std::vector<int32_t> cpart((size_t)G + 1), pch, cb;
    MG_CUDA(cudaMemcpyAsync(t.data(), h.ctime.p, (size_t)G * 8, cudaMemcpyDeviceToHost, g->stream));
    MG_CUDA(cudaMemcpyAsync(cpart.data(), h.cpart.p, cpart.size() * 4, cudaMemcpyDeviceToHost, g->stream));
    MG_CUDA(cudaStreamSynchronize(g->stream));
    // each CTA's first and last group: from its parts' chunks
    const size_t nparts = (size_t)cpart[G];
    pch.resize(nparts + 1);
    MG_CUDA(cudaMemcpy(pch.data(), h.pch.p, pch.size() * 4, cudaMemcpyDeviceToHost));
    cb.resize((size_t)pch[nparts] + 1);
    MG_CUDA(cudaMemcpy(cb.data(), h.cb.p, cb.size() * 4, cudaMemcpyDeviceToHost));
    std::vector<double> ratio((size_t)G, 0.0);
    double tt = 0.0, tw = 0.0;
    for (int b = 0; b < G; b++) {
        if (cpart[b] == cpart[b + 1]) continue;
        const int32_t lo = cb[(size_t)pch[(size_t)cpart[b]]], hi = cb[(size_t)pch[(size_t)cpart[b + 1]]];
        double wb = 0.0;
        for (int32_t q = lo; q < hi; q++) wb += h.w[q];
        if (wb <= 0.0 || t[b] <= 0) continue;
        ratio[b] = (double)t[b] / wb;
        tt += (double)t[b];
        tw += wb;
    }
    if (tt <= 0.0 || tw <= 0.0) return MG_OK;
    const double mean = tt / tw;
    for (int b = 0; b < G; b++) {
        if (ratio[b] <= 0.0) continue;
        const int32_t lo = cb[(size_t)pch[(size_t)cpart[b]]], hi = cb[(size_t)pch[(size_t)cpart[b + 1]]];
        for (int32_t q = lo; q < hi; q++) h.w[q] *= ratio[b] / mean;
    }
    return hub_split(g);
}

// Read (get) or replace (set) the groups' cost weights; false when the
// segmented layout is not in use or set has the wrong length.
bool hub_weights(mg_graph *g, std::vector<double> *get, const std::vector<double> *set)
{
    HubSplit &h = g->hub;
    if (!h.use) return false;
    if (get) *get = h.w;
    if (set) {
        if (set->size() != h.w.size()) return false;
        h.w = *set;
        if (hub_split(g) != MG_OK) return false;
    }
    return true;
}

size_t hub_smem_bytes(const mg_graph *g) { return (size_t)(g->hub.H + 4) * 4; }

mg_status hub_launch(mg_graph *g, const float *c0, const float *c1, const int32_t *cur, const int32_t *more,
                     const int32_t *off, cudaStream_t st, int slot_sweep)
{
    HubSplit &h = g->hub;
    HubArgs a;
    std::memset(&a, 0, sizeof(a));
    a.hdat = h.hdat.as<uint2>();
    a.goff = h.goff.as<int32_t>();
    a.pslot = h.pslot.as<int4>();
    a.cpart = h.cpart.as<int32_t>();
    a.pseg = h.pseg.as<int32_t>();
    a.pch = h.pch.as<int32_t>();
    a.cb = h.cb.as<int32_t>();
    a.c[0] = c0;
    a.c[1] = c1;
    a.cur = cur;
    a.more = more;
    a.off = off;
    a.P = h.P.as<float>();
    a.ctime = h.ctime.as<long long>();
    a.n = g->nv;
    a.H = h.H;
    a.nseg = h.nseg;
    const size_t smem = hub_smem_bytes(g);
    MG_CUDA(cudaFuncSetAttribute(k_hub_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    Profiler &P = g->prof;
    P.begin(slot_sweep);
    k_hub_sweep<<<h.grid, HUB_THREADS, smem, st>>>(a);
    P.end();
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}

// The sweep has no waits of its own (plain loads stage the segments), so
// there is nothing to report after a run.
mg_status hub_check(mg_graph *) { return MG_OK; }

}  // namespace mgi

// ---------------------------------------------------------------------------
// Host-only check of the segmented layout (no GPU): builds it from a host
// pull CSR on `threads` threads and on one, requires the two to be equal,
// and verifies every invariant the sweep and the row finish rely on, with
// exact integer sums (each edge's id + 1 in place of its contribution).
// ---------------------------------------------------------------------------
extern "C" mg_status mg_selftest_segmented_layout(int32_t nv, int64_t ne, const int32_t *row, const int32_t *col,
                                                  int32_t threads, int64_t *pieces_out)
{
    using namespace mgi;
    clear_error();
    if (!row || (ne > 0 && !col) || !pieces_out || nv < 0 || ne < 0 || ne > INT32_MAX)
        return fail(MG_ERR_INVALID, "bad argument");
    if (row[0] != 0 || row[nv] != ne) return fail(MG_ERR_INVALID, "row offsets must run from 0 to ne");
    for (int32_t v = 0; v < nv; v++)
        if (row[v + 1] < row[v]) return fail(MG_ERR_INVALID, "row offsets decrease at row %d", v);
    for (int64_t p = 0; p < ne; p++)
        if (col[p] < 0 || col[p] >= nv) return fail(MG_ERR_INVALID, "column id out of range at %lld", (long long)p);
    *pieces_out = 0;
    if (nv < 4 || ne == 0) return MG_OK;
    const std::vector<int32_t> prow(row, row + nv + 1), pcol(col, col + ne);
    HubHost a, b;
    MG_TRY(build_hub(prow, pcol, nv, ne, threads, a));
    MG_TRY(build_hub(prow, pcol, nv, ne, 1, b));
    if (a.use != b.use || a.covered != b.covered || a.npieces != b.npieces || a.hdat != b.hdat || a.goff != b.goff ||
        a.pslot != b.pslot || a.glam != b.glam || a.segg != b.segg || a.pair_off != b.pair_off || a.toff != b.toff ||
        a.tcol != b.tcol || a.fin != b.fin)
        return fail(MG_ERR_INTERNAL, "segmented layout differs between %d threads and one", threads);
    if (!a.use) return MG_OK;
    const int32_t H = a.H, nseg = a.nseg;
    const int64_t cover = std::min<int64_t>(nv, (int64_t)nseg * H);
    const int64_t np = a.npieces;
    const int32_t ngroups = (int32_t)a.glam.size();
    if ((int32_t)a.goff.size() != ngroups + 1 || (int64_t)a.hdat.size() != (int64_t)a.goff[ngroups] * GROUP ||
        (int64_t)a.pslot.size() != (int64_t)ngroups * GROUP || (int32_t)a.segg.size() != nseg + 1 ||
        a.segg[0] != 0 || a.segg[nseg] != ngroups || (int32_t)a.pair_off.size() != nv + 1 || a.pair_off[0] != 0 ||
        a.pair_off[nv] != np || (int32_t)a.toff.size() != nv + 1)
        return fail(MG_ERR_INTERNAL, "segmented layout: array sizes");
    // every packed piece: its slot (once), segment, length and id sum
    std::vector<int32_t> seen((size_t)np, 0), pseg((size_t)np, -1), plen((size_t)np, 0);
    std::vector<int64_t> psum((size_t)np, 0);
    for (int32_t sg = 0; sg < nseg; sg++) {
        for (int32_t q = a.segg[sg]; q < a.segg[sg + 1]; q++) {
            const int32_t lam = a.goff[q + 1] - a.goff[q];
            if (lam != a.glam[q] || lam < 1 || lam > PIECE_MAX || (q > a.segg[sg] && lam > a.glam[q - 1]))
                return fail(MG_ERR_INTERNAL, "segmented layout: group %d length", q);
            for (int32_t j = 0; j < GROUP; j++) {
                const int32_t slot = a.pslot[(size_t)q * GROUP + j];
                int64_t sum = 0;
                bool pad = true, real = true;
                for (int32_t k = 0; k < lam; k++) {
                    const int32_t id = a.hdat[((size_t)a.goff[q] + k) * GROUP + j];
                    pad = pad && id == H;
                    real = real && id < H && (int64_t)sg * H + id < nv;
                    sum += (int64_t)sg * H + id + 1;
                }
                if (slot == np) {
                    if (!pad) return fail(MG_ERR_INTERNAL, "segmented layout: padding of group %d", q);
                    continue;
                }
                if (slot < 0 || slot > np || !real || seen[slot]++)
                    return fail(MG_ERR_INTERNAL, "segmented layout: piece %d of group %d", j, q);
                pseg[slot] = sg;
                plen[slot] = lam;
                psum[slot] = sum;
            }
        }
    }
    for (int64_t p = 0; p < np; p++)
        if (seen[p] != 1) return fail(MG_ERR_INTERNAL, "segmented layout: slot %lld unused", (long long)p);
    // every row: its pieces (segments ascending, full pieces first) hold
    // exactly its covered in-edges; its tail holds the rest in row order
    std::vector<int32_t> fin;
    for (int32_t v = 0; v < nv; v++) {
        int64_t cnt[SEG_MAX] = {0}, sum[SEG_MAX] = {0};
        std::vector<int32_t> tail;
        for (int32_t p = row[v]; p < row[v + 1]; p++) {
            if (col[p] < cover) {
                cnt[col[p] / H]++;
                sum[col[p] / H] += (int64_t)col[p] + 1;
            } else {
                tail.push_back(col[p]);
            }
        }
        int64_t pcnt[SEG_MAX] = {0}, pss[SEG_MAX] = {0};
        for (int32_t p = a.pair_off[v]; p < a.pair_off[v + 1]; p++) {
            const int32_t sg = pseg[p];
            if (p > a.pair_off[v] && sg < pseg[p - 1]) return fail(MG_ERR_INTERNAL, "row %d: segments out of order", v);
            if (p > a.pair_off[v] && sg == pseg[p - 1] && plen[p - 1] != PIECE_MAX)
                return fail(MG_ERR_INTERNAL, "row %d: a short piece before another of its segment", v);
            pcnt[sg] += plen[p];
            pss[sg] += psum[p];
        }
        for (int32_t sg = 0; sg < nseg; sg++)
            if (pcnt[sg] != cnt[sg] || pss[sg] != sum[sg])
                return fail(MG_ERR_INTERNAL, "row %d: segment %d holds other edges", v, sg);
        if (a.toff[v + 1] - a.toff[v] != (int32_t)tail.size() ||
            !std::equal(tail.begin(), tail.end(), a.tcol.begin() + a.toff[v]))
            return fail(MG_ERR_INTERNAL, "row %d: tail", v);
        if (a.pair_off[v + 1] - a.pair_off[v] > FIN_WARP) fin.push_back(v);
    }
    if (fin != a.fin) return fail(MG_ERR_INTERNAL, "segmented layout: warp-row list");
    *pieces_out = np;
    return MG_OK;
}
