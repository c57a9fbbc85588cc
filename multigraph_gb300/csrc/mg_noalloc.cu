// mg_noalloc.cu -- PageRank that allocates nothing.
//
// Some callers cannot call cudaMalloc: code that runs inside a custom device
// allocator or a memory-pool callback, applications that pre-reserve all
// device memory at start-up and forbid later allocations, and real-time
// loops where an allocation (which can synchronise the device) would break a
// latency budget.  mg_pagerank_noalloc serves them: the caller passes its own
// device buffers for the graph and the result, and every intermediate lives
// in the fixed file-scope array g_noalloc_scratch below (MG_NOALLOC_MAX_VERTICES
// vertices' worth, held by every GPU that loads the library until the
// process exits).  The computation is the normalised, topology-driven
// PageRank of mg_pagerank(MG_PR_TOPOLOGY): x = (1-d)/n + d*(sum + dangling/n)
// from x = 1/n until the L1 change is <= tol, pulled over the rows of a
// symmetric CSR (the loader's MG_LOAD_SYM output), a warp per row with a
// fixed reduction order.
//
// Host code cannot use the array's name as a device address: it is a
// host-side stand-in.  The first call on a device (that device current) asks
// the runtime for the array's device address with cudaGetSymbolAddress and
// caches it.  No call may be made on a stream that is being captured: each
// call waits for its stream: it enqueues sweeps in batches of NA_BATCH and reads
// the control word back after each batch (sweeps after convergence are
// no-ops, so the batching changes neither the result nor the sweep count).
// All calls share the array and it keeps the last call's contents; every
// call re-initialises what it reads.  Calls that overlap on the GPU (two
// streams, or a call enqueued before the previous one finished) race on the
// array.

#include "mg_device.cuh"

#include <algorithm>
#include <mutex>

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_MAX_BLOCKS = 1024;
constexpr int NA_BATCH = 8;  // sweep + finish pairs enqueued per readback

struct NaCtl {
    int32_t more, iter, cur, pad;
    double resid;
    double dangling;
};

// layout of the scratch: x_alt | c0 | c1 | block partials | control word
constexpr size_t NA_VEC = (size_t)MG_NOALLOC_MAX_VERTICES * sizeof(float);
constexpr size_t NA_PART = (size_t)NA_MAX_BLOCKS * 2 * sizeof(double);
constexpr size_t NA_BYTES = 3 * NA_VEC + NA_PART + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

struct NaArgs {
    int32_t n;
    const int32_t *row, *col;
    float *x[2];   // x[0] = caller's output buffer, x[1] = scratch
    float *c[2];
    double *part;  // [nblocks][2] residual, dangling
    NaCtl *ctl;
    float damping, tol;
    int32_t max_iter;
};

__global__ void k_na_init(NaArgs a)
{
    const float x0 = 1.0f / (float)a.n;
    double dang = 0.0;
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.n; v += gridDim.x * blockDim.x) {
        int32_t deg = a.row[v + 1] - a.row[v];
        a.x[0][v] = x0;
        a.c[0][v] = deg > 0 ? x0 / (float)deg : 0.0f;
        if (deg == 0) dang += x0;
    }
    __shared__ double s[NA_THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dang += __shfl_xor_sync(0xffffffffu, dang, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = dang;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < NA_THREADS / 32; w++) t += s[w];
        a.part[2 * blockIdx.x] = 0.0;
        a.part[2 * blockIdx.x + 1] = t;
    }
}

__global__ void k_na_init_ctl(NaArgs a, int nblocks)
{
    if (threadIdx.x != 0) return;
    double dang = 0.0;
    for (int b = 0; b < nblocks; b++) dang += a.part[2 * b + 1];
    a.ctl->more = 1;
    a.ctl->iter = 0;
    a.ctl->cur = 0;
    a.ctl->resid = 0.0;
    a.ctl->dangling = dang;
}

// one sweep: warp per row, lane-strided partial sums + fixed xor tree
__global__ void __launch_bounds__(NA_THREADS) k_na_sweep(NaArgs a)
{
    const NaCtl c = *a.ctl;
    if (!c.more) return;
    const int cur = c.cur, nxt = cur ^ 1;
    const float d = a.damping;
    const float base = (float)((1.0 - (double)d) / a.n + (double)d * c.dangling / a.n);
    const int lane = threadIdx.x & 31;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    float resid = 0.0f, dang = 0.0f;
    for (int32_t v = gwarp; v < a.n; v += nwarps) {
        const int32_t b = a.row[v], e = a.row[v + 1];
        float s = 0.0f;
        for (int32_t p = b + lane; p < e; p += 32) s += a.c[cur][__ldg(&a.col[p])];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            const float xn = base + d * s;
            const float xo = a.x[cur][v];
            a.x[nxt][v] = xn;
            const int32_t deg = e - b;
            a.c[nxt][v] = deg > 0 ? xn / (float)deg : 0.0f;
            if (deg == 0) dang += xn;
            resid += fabsf(xn - xo);
        }
    }
    __shared__ double sr[NA_THREADS / 32], sd[NA_THREADS / 32];
    if (lane == 0) { sr[threadIdx.x >> 5] = resid; sd[threadIdx.x >> 5] = dang; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double R = 0.0, D = 0.0;
        for (int w = 0; w < NA_THREADS / 32; w++) { R += sr[w]; D += sd[w]; }
        a.part[2 * blockIdx.x] = R;
        a.part[2 * blockIdx.x + 1] = D;
    }
}

__global__ void k_na_finish(NaArgs a, int nblocks)
{
    if (threadIdx.x != 0) return;
    NaCtl *c = a.ctl;
    if (!c->more) return;
    double R = 0.0, D = 0.0;
    for (int b = 0; b < nblocks; b++) { R += a.part[2 * b]; D += a.part[2 * b + 1]; }
    c->resid = R;
    c->dangling = D;
    c->iter += 1;
    c->cur ^= 1;
    c->more = (R > (double)a.tol && c->iter < a.max_iter) ? 1 : 0;
}

std::mutex g_na_mu;
void *g_na_ptr[64] = {nullptr};

// device address of g_noalloc_scratch on the current device (cached per device)
mg_status scratch_address(int dev, unsigned char **out)
{
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (dev < 0 || dev >= 64) return mgi::fail(MG_ERR_RANGE, "device %d out of range", dev);
    if (!g_na_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return mgi::fail(MG_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch): %s", cudaGetErrorString(e));
        }
        g_na_ptr[dev] = p;
    }
    *out = (unsigned char *)g_na_ptr[dev];
    return MG_OK;
}

}  // namespace

extern "C" mg_status mg_pagerank_noalloc(const int32_t *d_row, const int32_t *d_col, int32_t nv, int32_t ne,
                                         float damping, float tol, int32_t max_iter, float *d_rank, void *stream,
                                         int32_t *iterations_out, double *residual_out)
{
    mgi::clear_error();
    if (!d_row || (!d_col && ne > 0) || !d_rank || nv <= 0 || ne < 0)
        return mgi::fail(MG_ERR_INVALID, "invalid argument");
    if (nv > MG_NOALLOC_MAX_VERTICES)
        return mgi::fail(MG_ERR_RANGE, "mg_pagerank_noalloc handles at most %d vertices (got %d)",
                         MG_NOALLOC_MAX_VERTICES, nv);
    // 0 selects the default; anything else must be a damping in (0, 1) and a
    // positive tolerance (NaN fails both tests)
    if (damping != 0.0f && !(damping > 0.0f && damping < 1.0f))
        return mgi::fail(MG_ERR_INVALID, "damping %g outside (0, 1)", (double)damping);
    if (tol != 0.0f && !(tol > 0.0f))
        return mgi::fail(MG_ERR_INVALID, "tolerance %g is not positive", (double)tol);
    cudaStream_t s = (cudaStream_t)stream;
    {
        // the row offsets must span exactly the ne column ids
        int32_t ends[2] = {-1, -1};
        MG_CUDA(cudaMemcpyAsync(&ends[0], d_row, 4, cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaMemcpyAsync(&ends[1], d_row + nv, 4, cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaStreamSynchronize(s));
        if (ends[0] != 0 || ends[1] != ne)
            return mgi::fail(MG_ERR_INVALID, "row offsets run from %d to %d, expected 0 to ne = %d", ends[0], ends[1],
                             ne);
    }
    int dev = 0;
    MG_CUDA(cudaGetDevice(&dev));
    unsigned char *base = nullptr;
    MG_TRY(scratch_address(dev, &base));
    int nsm = 0;
    MG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int nblocks = std::max(1, std::min(NA_MAX_BLOCKS, nsm * 4));
    NaArgs a;
    a.n = nv;
    a.row = d_row;
    a.col = d_col;
    a.x[0] = d_rank;
    a.x[1] = (float *)(base);
    a.c[0] = (float *)(base + NA_VEC);
    a.c[1] = (float *)(base + 2 * NA_VEC);
    a.part = (double *)(base + 3 * NA_VEC);
    a.ctl = (NaCtl *)(base + 3 * NA_VEC + NA_PART);
    a.damping = damping != 0.0f ? damping : 0.85f;
    a.tol = tol != 0.0f ? tol : 1e-6f;
    a.max_iter = max_iter > 0 ? max_iter : 10000;
    k_na_init<<<nblocks, NA_THREADS, 0, s>>>(a);
    k_na_init_ctl<<<1, 32, 0, s>>>(a, nblocks);
    MG_CUDA(cudaGetLastError());
    NaCtl h;
    for (int it = 0; it < a.max_iter; it += NA_BATCH) {
        // once the control word says stop, the remaining pairs of the batch
        // return at once; k_na_finish stops at max_iter by itself
        const int k = std::min(NA_BATCH, a.max_iter - it);
        for (int j = 0; j < k; j++) {
            k_na_sweep<<<nblocks, NA_THREADS, 0, s>>>(a);
            k_na_finish<<<1, 32, 0, s>>>(a, nblocks);
        }
        MG_CUDA(cudaGetLastError());
        MG_CUDA(cudaMemcpyAsync(&h, a.ctl, sizeof(NaCtl), cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaStreamSynchronize(s));
        if (!h.more) break;
    }
    // the last iterate is x[cur]; bring it into the caller's buffer
    if (h.cur == 1) {
        MG_CUDA(cudaMemcpyAsync(d_rank, a.x[1], (size_t)nv * sizeof(float), cudaMemcpyDeviceToDevice, s));
        MG_CUDA(cudaStreamSynchronize(s));
    }
    if (iterations_out) *iterations_out = h.iter;
    if (residual_out) *residual_out = h.resid;
    if (h.resid > (double)a.tol)
        return mgi::fail(MG_ERR_ITER_LIMIT, "PageRank did not converge in %d sweeps (residual %g)", a.max_iter, h.resid);
    return MG_OK;
}
