// mg_bins.cuh -- degree-binned row reduction shared by the pull kernels
// (PageRank sweeps, SSSP / BC pull, CC hooking).
//
// The pull-side rows are split at upload into three bins by in-degree:
//   warp bin   : 32 < deg <= heavy   rows of SUBWARP_MAX+ edges one warp per
//                row, lanes stride the row (one 128-byte line of column ids
//                per step); shorter rows one 8-lane group each (four rows
//                per warp in flight); an xor shuffle tree sums the lanes;
//   thread bin : deg <= 32           one thread per row, sequential walk;
//   heavy rows : deg > heavy         CTA-sized chunks (handled by the caller).
// With the hub-first vertex order rows of one bin are sorted by log2 degree,
// so the rows of a warp have similar lengths.  Every row's total is formed
// in a fixed order, so floating-point results are reproducible.
#pragma once

#include <cstdint>

namespace mgd {

// lane exchange of a row value (built-in types; composite value types
// provide their own shfl_xor_val, found by argument-dependent lookup)
template <class T>
__device__ __forceinline__ T shfl_xor_val(T v, int o)
{
    return __shfl_xor_sync(0xffffffffu, v, o);
}

// loads in flight per lane in the warp-row and 8-lane-row loops
constexpr int WARP_ILP = 2;
constexpr int G8_ILP = 2;

// One group of G lanes (G = 32: a warp; G = 8: a quarter warp), one row v
// with edges [b, e): lanes stride the row by G with ILP loads in flight;
// the group's total (xor steps within the group, fixed order) on every lane
// of the group.  All 32 lanes call it (groups without a row pass b == e).
template <int G, int ILP, class Op>
__device__ __forceinline__ typename Op::T group_row(Op &op, const int32_t *__restrict__ pcol,
                                                    const int32_t *__restrict__ pwt, int32_t v, int32_t b, int32_t e)
{
    using T = typename Op::T;
    T acc[ILP];
#pragma unroll
    for (int k = 0; k < ILP; k++) acc[k] = op.identity();
    int32_t p = b + (threadIdx.x & (G - 1));
    // the column / weight stream is read once per sweep: evict-first loads
    // (__ldcs) keep L1 and L2 for the gathered vertex values
    for (; p + G * (ILP - 1) < e; p += G * ILP) {
        int32_t u[ILP], w[ILP];
#pragma unroll
        for (int k = 0; k < ILP; k++) {
            u[k] = __ldcs(&pcol[p + G * k]);
            w[k] = Op::kWeights ? __ldcs(&pwt[p + G * k]) : 0;
        }
#pragma unroll
        for (int k = 0; k < ILP; k++) acc[k] = op.combine(acc[k], op.edge(p + G * k, v, u[k], w[k]));
    }
#pragma unroll
    for (int k = 0; k < ILP - 1; k++, p += G)
        if (p < e) acc[k] = op.combine(acc[k], op.edge(p, v, __ldcs(&pcol[p]), Op::kWeights ? __ldcs(&pwt[p]) : 0));
    T t = acc[0];
#pragma unroll
    for (int k = 1; k < ILP; k++) t = op.combine(t, acc[k]);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) t = op.combine(t, shfl_xor_val(t, o));
    return t;
}

// One warp, one row v (warp-uniform call).  Returns the total on every lane.
template <class Op>
__device__ __forceinline__ typename Op::T warp_row(Op &op, const int32_t *__restrict__ prow,
                                                   const int32_t *__restrict__ pcol, const int32_t *__restrict__ pwt,
                                                   int32_t v)
{
    return group_row<32, WARP_ILP>(op, pcol, pwt, v, prow[v], prow[v + 1]);
}

// One thread, one row v.
template <class Op>
__device__ __forceinline__ typename Op::T thread_row(Op &op, const int32_t *__restrict__ prow,
                                                     const int32_t *__restrict__ pcol, const int32_t *__restrict__ pwt,
                                                     int32_t v)
{
    using T = typename Op::T;
    const int32_t b = prow[v], e = prow[v + 1];
    T acc = op.identity();
    int32_t p = b;
    for (; p + 4 <= e; p += 4) {
        int32_t u0 = __ldg(&pcol[p]), u1 = __ldg(&pcol[p + 1]), u2 = __ldg(&pcol[p + 2]), u3 = __ldg(&pcol[p + 3]);
        int32_t w0 = 0, w1 = 0, w2 = 0, w3 = 0;
        if (Op::kWeights) { w0 = __ldg(&pwt[p]); w1 = __ldg(&pwt[p + 1]); w2 = __ldg(&pwt[p + 2]); w3 = __ldg(&pwt[p + 3]); }
        T t0 = op.edge(p, v, u0, w0), t1 = op.edge(p + 1, v, u1, w1), t2 = op.edge(p + 2, v, u2, w2),
          t3 = op.edge(p + 3, v, u3, w3);
        acc = op.combine(op.combine(acc, t0), t1);
        acc = op.combine(op.combine(acc, t2), t3);
    }
    for (; p < e; p++) acc = op.combine(acc, op.edge(p, v, __ldg(&pcol[p]), Op::kWeights ? __ldg(&pwt[p]) : 0));
    return acc;
}

// All rows of the warp and thread bins, grid-stride.  op.finish(v, total) is
// called once per row (by lane 0 for warp rows, by the group's first lane
// for 8-lane rows); op.flush() is called by every lane at warp-uniform points
// after each warp row, each round of four 8-lane rows and each round of
// thread rows (at most 32 finishes per warp in between).  Rows with
// op.skip(v) are finished with the identity without reading their edges.
// wrows[0, nwlong) hold the warp bin's rows of SUBWARP_MAX+ edges.
template <class Op>
__device__ __forceinline__ void bins_reduce(Op &op, const int32_t *__restrict__ prow, const int32_t *__restrict__ pcol,
                                            const int32_t *__restrict__ pwt, const int32_t *__restrict__ wrows,
                                            int32_t nw, int32_t nwlong, const int32_t *__restrict__ trows, int32_t nt)
{
    const int ln = threadIdx.x & 31;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int32_t i = gwarp; i < nwlong; i += nwarps) {
        const int32_t v = wrows[i];
        if (Op::kRowAware && op.skip(v)) {
            if (ln == 0) op.finish(v, op.identity());
        } else {
            auto t = warp_row(op, prow, pcol, pwt, v);
            if (ln == 0) op.finish(v, t);
        }
        op.flush();
    }
    // short warp-bin rows: four per warp, an 8-lane group each
    const int grp = ln >> 3;
    for (int32_t base = nwlong + gwarp * 4; base < nw; base += nwarps * 4) {
        const int32_t i = base + grp;
        int32_t v = -1, b = 0, e = 0;
        bool skipped = false;
        if (i < nw) {
            v = wrows[i];
            if (Op::kRowAware && op.skip(v)) {
                skipped = true;
            } else {
                b = prow[v];
                e = prow[v + 1];
            }
        }
        const auto t = group_row<8, G8_ILP>(op, pcol, pwt, v, b, e);
        if ((ln & 7) == 0 && v >= 0) op.finish(v, skipped ? op.identity() : t);
        op.flush();
    }
    const int32_t nthreads = gridDim.x * blockDim.x;
    const int32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t rounds = (nt + nthreads - 1) / nthreads;
    for (int32_t r = 0; r < rounds; r++) {
        const int32_t i = r * nthreads + gt;
        if (i < nt) {
            const int32_t v = trows[i];
            if (Op::kRowAware && op.skip(v)) op.finish(v, op.identity());
            else op.finish(v, thread_row(op, prow, pcol, pwt, v));
        }
        op.flush();
    }
}

}  // namespace mgd
