// mg_group.cuh -- the edge-balanced row reduction shared by the pull kernels
// (PageRank sweeps, SSSP / BC pull, CC hooking).
#pragma once

#include <cstdint>

namespace mgd {

// rows per pull group and edges per pull group (groups built at upload)
constexpr int GROUP_ROWS = 128;
constexpr int GROUP_EDGES = 512;
// shared staging per warp: GROUP_EDGES column ids plus vector alignment slack
constexpr int GROUP_STAGE = GROUP_EDGES + 8;
// edges whose loads a lane keeps in flight together
constexpr int GROUP_BATCH = 8;

// Per-warp shared scratch of group_reduce: off (GROUP_ROWS + 1 ints), col
// (GROUP_STAGE ints, 16-byte aligned) and, for Op::kWeights, wt (same).
struct GroupSmem {
    int32_t *off;
    int32_t *col;
    int32_t *wt;
};

// Row reduction of one edge-balanced group [r0, r1) by one warp.
//
// The group's in-edges [off[r0], off[r1]) (<= GROUP_EDGES of them) are first
// copied to shared memory with 16-byte loads (column ids, and the integer
// weights when Op::kWeights), then cut into 32 contiguous slices of odd
// length (so the lanes' shared reads fall in distinct banks), one per lane.
// Each lane walks its slice in batches of GROUP_BATCH edges -- all column
// reads and gathers of a batch are issued before they are folded -- calling
// op.finish(row, total) for every row that starts and ends in its slice.
// Rows crossing slice boundaries are summed with one segmented scan over the
// lanes (earlier lanes first) and finished by the lane holding their last
// edge; zero-length rows are finished by the lane whose slice ends at their
// offset (lane 0 for those at the group start).  Every row is finished
// exactly once and the combine order depends only on the layout, so floating
// point results are reproducible run to run.  The column arrays must have at
// least 3 ints of readable padding past their end.  All 32 lanes must call.
//
// Op: static constexpr bool kRowAware (edge values depend on the row or rows
//     may be skipped), kWeights (pass the edge's integer weight);
//     typedef T; T identity(); bool skip(int row) (row's edges are not read,
//     its total is the identity); T edge(int e, int row, int u, int w);
//     T combine(T a, T b); void finish(int row, T total).
template <class Op>
__device__ __forceinline__ void group_reduce(Op &op, const int32_t *__restrict__ prow,
                                             const int32_t *__restrict__ pcol, const int32_t *__restrict__ pwt,
                                             int32_t r0, int32_t r1, GroupSmem sm)
{
    using T = typename Op::T;
    const int ln = threadIdx.x & 31;
    const int nr = r1 - r0;
    for (int i = ln; i <= nr; i += 32) sm.off[i] = prow[r0 + i];
    __syncwarp();
    const int32_t E0 = sm.off[0], E1 = sm.off[nr];
    const int32_t tot = E1 - E0;
    // stage [a0, a1) with int4 loads; a0, a1 multiples of 4
    const int32_t a0 = E0 & ~3;
    const int32_t n4 = (((E1 + 3) & ~3) - a0) >> 2;
    {
        const int4 *src = reinterpret_cast<const int4 *>(pcol + a0);
        int4 *dst = reinterpret_cast<int4 *>(sm.col);
        for (int i = ln; i < n4; i += 32) dst[i] = __ldg(src + i);
        if (Op::kWeights) {
            const int4 *ws = reinterpret_cast<const int4 *>(pwt + a0);
            int4 *wd = reinterpret_cast<int4 *>(sm.wt);
            for (int i = ln; i < n4; i += 32) wd[i] = __ldg(ws + i);
        }
    }
    __syncwarp();
    const int32_t *scol = sm.col - a0;  // scol[e] for e in [E0, E1)
    const int32_t *swt = sm.wt - a0;
    int32_t k = (tot + 31) >> 5;
    k |= 1;  // odd stride: lane slices start in distinct banks
    const int32_t ls = E0 + min(ln * k, tot), le = E0 + min(ln * k + k, tot);
    int key = -1;           // row continuing past le
    T val = op.identity();  // its sum over this slice
    int head_row = -1;      // row started before ls and ending in (ls, le]
    T head_acc = op.identity();
    if (ls < le) {
        int lo = 0, hi = nr - 1;  // largest r with off[r] <= ls
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (sm.off[mid] <= ls) lo = mid; else hi = mid - 1;
        }
        int r = lo;
        if (ln == 0)
            for (int z = 0; z < r; z++) op.finish(r0 + z, op.identity());
        int32_t rs = sm.off[r], re = sm.off[r + 1];
        T acc = op.identity();
        int rt = r;
        int32_t ret = re;
        bool skt = Op::kRowAware ? op.skip(r0 + r) : false;
        for (int32_t base = ls; base < le; base += GROUP_BATCH) {
            T vj[GROUP_BATCH];
            if (Op::kRowAware) {
                int rowj[GROUP_BATCH];
                bool live[GROUP_BATCH];
#pragma unroll
                for (int j = 0; j < GROUP_BATCH; j++) {
                    const int32_t e = base + j;
                    live[j] = false;
                    rowj[j] = rt;
                    if (e < le) {
                        while (e >= ret) { rt++; ret = sm.off[rt + 1]; skt = op.skip(r0 + rt); }
                        rowj[j] = rt;
                        live[j] = !skt;
                    }
                }
#pragma unroll
                for (int j = 0; j < GROUP_BATCH; j++)
                    vj[j] = live[j] ? op.edge(base + j, r0 + rowj[j], scol[base + j], Op::kWeights ? swt[base + j] : 0)
                                    : op.identity();
            } else {
#pragma unroll
                for (int j = 0; j < GROUP_BATCH; j++)
                    vj[j] = (base + j < le) ? op.edge(base + j, 0, scol[base + j], Op::kWeights ? swt[base + j] : 0)
                                            : op.identity();
            }
#pragma unroll
            for (int j = 0; j < GROUP_BATCH; j++) {
                const int32_t e = base + j;
                if (e < le) {
                    while (e >= re) {  // row r ended before edge e
                        if (rs >= ls) op.finish(r0 + r, acc);
                        else { head_row = r; head_acc = acc; }
                        r++;
                        rs = sm.off[r];
                        re = sm.off[r + 1];
                        acc = op.identity();
                    }
                    acc = op.combine(acc, vj[j]);
                }
            }
        }
        // rows ending at or before le (incl. zero-length rows at le), then the
        // row continuing into the next slice
        for (;;) {
            if (re <= le) {
                if (rs >= ls) op.finish(r0 + r, acc);
                else { head_row = r; head_acc = acc; }
                r++;
                if (r >= nr) break;
                rs = sm.off[r];
                re = sm.off[r + 1];
                acc = op.identity();
                if (rs >= le && re > le) break;  // starts the next slice
            } else {
                key = r;
                val = acc;
                break;
            }
        }
    } else if (tot == 0 && ln == 0) {
        for (int z = 0; z < nr; z++) op.finish(r0 + z, op.identity());
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int pk = __shfl_up_sync(0xffffffffu, key, o);
        T pv = __shfl_up_sync(0xffffffffu, val, o);
        if (ln >= o && key >= 0 && pk == key) val = op.combine(pv, val);
    }
    int pk = __shfl_up_sync(0xffffffffu, key, 1);
    T pv = __shfl_up_sync(0xffffffffu, val, 1);
    if (head_row >= 0) {
        T carry = (ln > 0 && pk == head_row) ? pv : op.identity();
        op.finish(r0 + head_row, op.combine(carry, head_acc));
    }
    __syncwarp();
}

}  // namespace mgd
