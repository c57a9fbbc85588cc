// mg_bins.cuh -- degree-binned row reduction shared by the pull kernels
// (PageRank sweeps, SSSP / BC pull, CC hooking).
//
// The pull-side rows are split at upload into three bins by in-degree:
//   warp bin   : 32 < deg <= heavy   one warp per row, lanes stride the row
//                (one 128-byte line of column ids per step), a fixed xor
//                shuffle tree sums the lanes;
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

// warp-wide xor reduction tree (fixed order)
template <class Op>
__device__ __forceinline__ typename Op::T warp_combine(const Op &op, typename Op::T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = op.combine(v, shfl_xor_val(v, o));
    return v;
}

// One warp, one row v (warp-uniform call).  Returns the total on every lane.
template <class Op>
__device__ __forceinline__ typename Op::T warp_row(Op &op, const int32_t *__restrict__ prow,
                                                   const int32_t *__restrict__ pcol, const int32_t *__restrict__ pwt,
                                                   int32_t v)
{
    using T = typename Op::T;
    const int ln = threadIdx.x & 31;
    const int32_t b = prow[v], e = prow[v + 1];
    T acc0 = op.identity(), acc1 = op.identity();
    int32_t p = b + ln;
    // the column / weight stream is read once per sweep: evict-first loads
    // (__ldcs) keep L1 and L2 for the gathered vertex values
    for (; p + 32 < e; p += 64) {  // two independent loads in flight per lane
        int32_t u0 = __ldcs(&pcol[p]), u1 = __ldcs(&pcol[p + 32]);
        int32_t w0 = Op::kWeights ? __ldcs(&pwt[p]) : 0, w1 = Op::kWeights ? __ldcs(&pwt[p + 32]) : 0;
        acc0 = op.combine(acc0, op.edge(p, v, u0, w0));
        acc1 = op.combine(acc1, op.edge(p + 32, v, u1, w1));
    }
    if (p < e) acc0 = op.combine(acc0, op.edge(p, v, __ldcs(&pcol[p]), Op::kWeights ? __ldcs(&pwt[p]) : 0));
    return warp_combine(op, op.combine(acc0, acc1));
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
// called once per row (by lane 0 for warp rows); op.flush() is called by
// every lane at warp-uniform points after each warp row and after each round
// of thread rows (at most 32 finishes per warp in between).  Rows with
// op.skip(v) are finished with the identity without reading their edges.
template <class Op>
__device__ __forceinline__ void bins_reduce(Op &op, const int32_t *__restrict__ prow, const int32_t *__restrict__ pcol,
                                            const int32_t *__restrict__ pwt, const int32_t *__restrict__ wrows,
                                            int32_t nw, const int32_t *__restrict__ trows, int32_t nt)
{
    const int ln = threadIdx.x & 31;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int32_t i = gwarp; i < nw; i += nwarps) {
        const int32_t v = wrows[i];
        if (Op::kRowAware && op.skip(v)) {
            if (ln == 0) op.finish(v, op.identity());
        } else {
            auto t = warp_row(op, prow, pcol, pwt, v);
            if (ln == 0) op.finish(v, t);
        }
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
