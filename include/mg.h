/*
 * mg.h -- C ABI of the GB300 frontier-processing engine (libmg.so).
 *
 * Plain C types only: pointers, sizes, status codes and opaque handles.  No
 * C++ or torch type crosses this boundary.  Every entry point returns an
 * mg_status; a failing call also leaves a message for mg_last_error() on the
 * calling thread.  No entry point exits the process.
 *
 * Each declaration names the reference interface it replaces
 * (hochawa/multigraph, paths relative to the project root).
 */
#ifndef MG_H
#define MG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* status                                                                   */
/* ------------------------------------------------------------------------ */
/* The reference has no error reporting (errors are printed and ignored,
 * read_input.cu:73-76 calls exit(0) on a bad id); these codes replace that. */
typedef int32_t mg_status;
enum {
    MG_OK = 0,
    MG_ERR_IO = 1,          /* file cannot be opened / written               */
    MG_ERR_PARSE = 2,       /* malformed or truncated MTX                    */
    MG_ERR_RANGE = 3,       /* vertex id or source out of range              */
    MG_ERR_OOM = 4,         /* host or device allocation failed              */
    MG_ERR_CUDA = 5,        /* CUDA runtime error (incl. no device)          */
    MG_ERR_ITER_LIMIT = 6,  /* iteration cap reached before convergence     */
    MG_ERR_INVALID = 7,     /* invalid argument                              */
    MG_ERR_UNSUPPORTED = 8, /* graph lacks what the call needs (e.g. weights)*/
    MG_ERR_INTERNAL = 9     /* a self-check found an inconsistency           */
};

const char *mg_status_string(mg_status s);
/* Message of the last failing call on this thread ("" if none). */
const char *mg_last_error(void);
/* Library version string. */
const char *mg_version(void);

/* ------------------------------------------------------------------------ */
/* host graph  (replaces struct csc_package + generate_CSC)                 */
/* ------------------------------------------------------------------------ */
typedef struct mg_host_graph mg_host_graph;

/* Loader flags: the compile-time -DSYM / -DNSYM / -DCC switches of
 * read_input.cu:39-44,111-113 as runtime bits. */
#define MG_LOAD_SYM  1u   /* treat the file as symmetric (install.sh builds) */
#define MG_LOAD_NSYM 2u   /* treat the file as general                       */
#define MG_LOAD_CC   4u   /* keep only src < dst edges (CC build)            */

/* View of a host CSR; pointers stay valid until the graph is freed.
 * Mirrors struct csc_package (common.h:170-182). */
typedef struct mg_csr_view {
    int32_t nv, ne;           /* vertices / directed edges after the loader */
    int32_t start_p;          /* source vertex after renumbering            */
    int32_t tra;              /* 1 if some degree >= 128                    */
    const int32_t *csc_v;     /* [nv+1] row offsets                          */
    const int32_t *csc_e;     /* [ne]   column ids                           */
    const int32_t *csc_ev;    /* [ne]   integer edge weights                 */
} mg_csr_view;

/* Replaces generate_CSC (read_input.cu:11-254): MTX -> deduplicated,
 * compacted CSR with the source renumbered.  Pattern files get weights
 * 1 + splitmix64(weight_seed, entry) % 64 instead of the reference's
 * rand()%64+1 under srand(time(NULL)) (read_input.cu:21,77), so runs are
 * reproducible.  Parsing and sorting use nthreads host threads (0 = all). */
mg_status mg_load_mtx(const char *path, int32_t source, uint32_t flags, uint64_t weight_seed,
                      int32_t nthreads, mg_host_graph **out);

/* Same pipeline from an in-memory entry list (0-based ids, the order a file
 * would list them; val may be NULL for pattern entries).  nv_decl is the
 * declared vertex count of the size line. */
mg_status mg_host_graph_from_entries(int32_t nv_decl, int64_t nentries, const int32_t *src,
                                     const int32_t *dst, const int32_t *val, int32_t source,
                                     uint32_t flags, uint64_t weight_seed, int32_t nthreads,
                                     mg_host_graph **out);

/* Wrap an existing CSR (copied).  wt may be NULL (all weights 1). */
mg_status mg_host_graph_from_csr(int32_t nv, int32_t ne, const int32_t *csc_v, const int32_t *csc_e,
                                 const int32_t *csc_ev, int32_t start_p, mg_host_graph **out);

mg_status mg_host_graph_view(const mg_host_graph *g, mg_csr_view *view);
/* Make page-locked copies of the host arrays (driver allocations) from which
 * mg_graph_stage uploads at full link speed (optional; doubles the graph's
 * host memory until mg_host_graph_free). */
mg_status mg_host_graph_pin(mg_host_graph *g);
/* Bytes mg_graph_stage copies to the device for this graph (row offsets,
 * column ids and weights, all int32). */
int64_t mg_host_graph_stage_bytes(const mg_host_graph *g);
void mg_host_graph_free(mg_host_graph *g);
/* Write as MatrixMarket "coordinate integer general" (1-based, every CSR
 * entry) or "pattern" when with_weights == 0. */
mg_status mg_write_mtx(const mg_host_graph *g, const char *path, int32_t with_weights);

/* Binary CSR cache: the loader's output (row offsets, column ids, weights,
 * start_p, tra) in one file, so a graph parsed once from MTX reloads at
 * disk speed.  Layout: a 40-byte header (magic "MGCSR001", nv, ne,
 * start_p, tra, flags, FNV-1a 64 checksum of the arrays, little-endian),
 * then csc_v[nv+1], csc_e[ne], csc_ev[ne] as int32.  mg_load_csr checks
 * the header, the file size, the checksum and the CSR invariants
 * (MG_ERR_PARSE on any mismatch).  No reference counterpart (the reference
 * re-parses the MTX text on every run, read_input.cu:24-97). */
mg_status mg_save_csr(const mg_host_graph *g, const char *path);
mg_status mg_load_csr(const char *path, mg_host_graph **out);

/* Synthetic inputs (no reference counterpart; the reference reads files).
 * R-MAT (Chakrabarti, Zhan, Faloutsos 2004): edge_factor * 2^scale draws,
 * quadrant probabilities a, b, c, 1-a-b-c; symmetrised, self-loops and
 * duplicates removed, then compacted as the loader does.  Integer weights
 * uniform in [wmin, wmax] per undirected edge. */
mg_status mg_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed,
                      int32_t wmin, int32_t wmax, int32_t nthreads, mg_host_graph **out);
/* rows x cols 4-neighbour lattice plus, for a fraction of vertices, one
 * diagonal shortcut (to (r+1, c+1)); symmetrised; weights 1. */
mg_status mg_gen_lattice(int32_t rows, int32_t cols, double shortcut_frac, uint64_t seed,
                         mg_host_graph **out);

/* ------------------------------------------------------------------------ */
/* device graph  (replaces struct HYB / MULTI_SPARSE, generate_MultiGraph,   */
/* generate_MultiGraphS, release_MultiGraph)                                */
/* ------------------------------------------------------------------------ */
typedef struct mg_graph mg_graph;

/* Replaces generate_MultiGraph (gen_structure.cu:2230) and
 * generate_MultiGraphS (gen_structure.cu:99): uploads the CSR and builds the
 * device layouts (edge-balanced row partitions, degree classes, the
 * src<dst edge list for CC) on `device`. */
mg_status mg_graph_upload(const mg_host_graph *g, int32_t device, mg_graph **out);
/* Re-copy a host CSR of the same nv/ne into an existing device graph (the
 * allocation is reused when the degrees are unchanged; a graph whose row
 * offsets differ is laid out again).  Equivalent to mg_graph_stage followed
 * by mg_graph_commit. */
mg_status mg_graph_reload(mg_graph *dg, const mg_host_graph *g);
/* Double-buffered input: mg_graph_stage starts copying g (same nv/ne) into
 * the device graph's staging buffers on the graph's copy stream and returns
 * at once, so the copy overlaps runs still working on the current graph;
 * g must stay alive and unchanged until mg_graph_commit.  Runs (and
 * mg_graph_set_float_weights) between the two calls use the current graph;
 * the staged copy has buffers of its own.  mg_graph_commit makes later runs
 * wait for the copy and rebuilds the device CSR from it on the graph's
 * stream (row offsets compared on the device; a relabel pass when they
 * match the layout's, which also takes the new weights' least value for
 * SSSP; otherwise the graph is laid out again and captured loops are
 * rebuilt on their next run).  No reference counterpart. */
mg_status mg_graph_stage(mg_graph *dg, const mg_host_graph *g);
mg_status mg_graph_commit(mg_graph *dg);
/* Replaces release_MultiGraph (release_structure.cu:4). */
void mg_graph_free(mg_graph *dg);
mg_status mg_graph_info(const mg_graph *dg, int32_t *nv, int32_t *ne);
/* cudaStream_t (as void*) on which every run of this graph is enqueued. */
void *mg_graph_stream(mg_graph *dg);
/* Float edge weights (one per CSR entry) for weighted PageRank; host array. */
mg_status mg_graph_set_float_weights(mg_graph *dg, const float *w);

/* ------------------------------------------------------------------------ */
/* run options / info                                                        */
/* ------------------------------------------------------------------------ */
enum { MG_EXEC_GRAPH = 0,     /* iteration loop in a CUDA graph (device-side while) */
       MG_EXEC_HOST = 1 };    /* host-driven loop, one readback per iteration      */

enum { MG_DIR_AUTO = 0, MG_DIR_PUSH = 1, MG_DIR_PULL = 2 };  /* SPARSE_MODE / DENSE_MODE */

typedef struct mg_opts {
    int32_t exec;          /* MG_EXEC_*                                        */
    int32_t direction;     /* MG_DIR_*: AUTO = hybrid switch                   */
    int32_t max_iter;      /* 0 = default cap                                  */
    int32_t alpha;         /* push->pull when frontier edges > unvisited/alpha */
    int32_t beta;          /* pull->push when frontier vertices < nv/beta      */
    float damping;         /* PageRank d (0.85)                                */
    float tol;             /* PageRank tolerance                               */
    int32_t profile;       /* 1: host loop with cudaEvents around each kernel  */
    int32_t pr_layout;     /* PageRank pull sweep over unweighted graphs:      */
                           /* MG_PR_LAYOUT_AUTO (default: segmented where it   */
                           /* applies, unless mg_autotune measured the gather  */
                           /* layout faster on this graph),                    */
                           /* MG_PR_LAYOUT_GATHER (L2 gathers over degree      */
                           /* bins) or MG_PR_LAYOUT_SEGMENTED (shared-memory   */
                           /* segments; gather where a quarter of the edges    */
                           /* or fewer fall in segments)                       */
    int32_t reserved[7];
} mg_opts;

enum { MG_PR_LAYOUT_GATHER = 0, MG_PR_LAYOUT_SEGMENTED = 1, MG_PR_LAYOUT_AUTO = 2 };

/* Fill *o with the defaults (exec graph, auto direction, tuned thresholds). */
void mg_opts_default(mg_opts *o);

#define MG_PROFILE_SLOTS 16
typedef struct mg_kernel_time {
    char name[32];
    int32_t launches;
    double total_ms;
} mg_kernel_time;

typedef struct mg_run_info {
    int32_t iterations;      /* frontier iterations / PR sweeps            */
    int32_t pull_iterations; /* iterations that ran the dense (pull) form  */
    double device_ms;        /* cudaEvent time of the run on its stream    */
    double residual;         /* PageRank: final L1 change                  */
    int64_t edges_scanned;   /* edges read by the kernels (when counted)   */
    int32_t nkernels;        /* profile slots used                          */
    mg_kernel_time kernels[MG_PROFILE_SLOTS];
} mg_run_info;

/* Outputs: every run writes its results into device buffers owned by the
 * graph; when the host pointer argument is non-NULL the result is also
 * copied there (nv entries) before the call returns.  mg_result_device
 * returns the device buffer, valid until the next run of the same kind or
 * mg_graph_free. */
enum { MG_RES_LEVEL = 0, MG_RES_DIST = 1, MG_RES_LABEL = 2, MG_RES_RANK = 3,
       MG_RES_SIGMA = 4, MG_RES_DELTA = 5, MG_RES_BC = 6 };
const void *mg_result_device(mg_graph *dg, int32_t which);

/* ------------------------------------------------------------------------ */
/* algorithms (replace the per-binary main.cu loops + MultiGraph_* engines) */
/* ------------------------------------------------------------------------ */

/* BFS levels from source; 0x64646464 marks unreached (common.h:37-39).
 * Replaces initValue/resetValue + while(MultiGraph_V_E_V(...)) with -DBFS
 * (main.cu:26-45, process.cu:1079-1368, user_function.h BFS hooks). */
mg_status mg_bfs(mg_graph *dg, int32_t source, const mg_opts *o, int32_t *level_out, mg_run_info *info);

/* SSSP distances (integer weights), 0x64646464 unreached.  -DSSSP build of
 * the same loop (user_function.h:244-246,276-278,346-360,400-408). */
mg_status mg_sssp(mg_graph *dg, int32_t source, const mg_opts *o, int32_t *dist_out, mg_run_info *info);

/* Connected components; label = minimum vertex id of the component.
 * Replaces MultiGraph_E_E / MultiGraph_V_V (process.cu:940-1077, main.cu:87-126);
 * the reference's labels become canonical after validate.cu:234-242. */
mg_status mg_cc(mg_graph *dg, const mg_opts *o, int32_t *label_out, mg_run_info *info);

/* Single-source Brandes: levels, sigma (FP64 path counts), delta (FP32).
 * Replaces the -DBC forward loop + MultiGraph_V_E_V_pull (process2.cu:263-325).
 * delta[v] is the raw dependency, including delta[source] as validate.cu:182-189.
 * Path counts that pass 2^90 (lattices after a few hundred levels) switch
 * the graph's BC runs to extended counts (FP64 mantissa, 2^512 scale), so
 * delta stays exact to FP32 at any depth; sigma_out then holds +infinity for
 * counts beyond the FP64 range (the reference's int32 counts wrap). */
mg_status mg_bc(mg_graph *dg, int32_t source, const mg_opts *o, int32_t *level_out, double *sigma_out,
                float *delta_out, mg_run_info *info);

/* Multi-source BC scores bc[v] = sum_s delta_s[v] (v != s).  Symmetric
 * graphs traverse 32 sources at a time (one lane per source; up to 2^26
 * vertices, ~1 KB of device memory per vertex), directed graphs one source
 * at a time.  No reference counterpart (the reference runs one source). */
mg_status mg_bc_multi(mg_graph *dg, const int32_t *sources, int32_t nsrc, const mg_opts *o,
                      float *bc_out, mg_run_info *info);

/* PageRank variants.
 *   MG_PR_TOPOLOGY_REF / MG_PR_DATA_REF: the reference recurrences of PR_T /
 *     PR_D (processi.cu:577-670, validate.cu:47-91): unnormalised
 *     0.15 + 0.85*sum, start 0, tolerance 0.01 absolute (T) / relative with a
 *     sticky per-vertex mask (D).
 *   MG_PR_TOPOLOGY: normalised (1-d)/n + d*(sum + dangling/n), start 1/n,
 *     stop when the L1 change <= tol.
 *   MG_PR_DATA: normalised, data-driven: only vertices with an active
 *     in-neighbour are recomputed; a vertex stays active while its change
 *     exceeds tol/nv (processi.cu:182-407 semantics with the normalised form). */
enum { MG_PR_TOPOLOGY_REF = 0, MG_PR_DATA_REF = 1, MG_PR_TOPOLOGY = 2, MG_PR_DATA = 3 };
mg_status mg_pagerank(mg_graph *dg, int32_t variant, const mg_opts *o, float *rank_out, mg_run_info *info);

/* Personalised PageRank for nseeds one-hot seeds in one batched run:
 * x_s = (1-d) e_s + d (P^T x_s + dangling e_s).  out is nseeds x nv (row s =
 * seed s).  No reference counterpart. */
mg_status mg_ppr_batch(mg_graph *dg, const int32_t *seeds, int32_t nseeds, const mg_opts *o, float *out,
                       mg_run_info *info);

/* Weighted PageRank with the float weights of mg_graph_set_float_weights:
 * P_uv = w_uv / S_u, x = (1-d)/n + d (P^T x + dangling/n). */
mg_status mg_wpagerank(mg_graph *dg, const mg_opts *o, float *x_out, mg_run_info *info);
/* Backward of L = sum_i g_i x_i through mg_wpagerank's fixed point.
 * lambda = g + d P lambda (transposed fixed point), then per edge
 * grad_w[e] = d x_u / S_u * (lambda_v - sum_k P_uk lambda_k).
 * The lambda iteration stops when its L1 change is <= tol * |g|_1.
 * Uses the x of the last mg_wpagerank on this graph.  No reference counterpart. */
mg_status mg_wpagerank_backward(mg_graph *dg, const float *g_host, const mg_opts *o, float *grad_w_out,
                                float *lambda_out, mg_run_info *info);

/* ------------------------------------------------------------------------ */
/* multi-graph batches (no reference counterpart)                            */
/* ------------------------------------------------------------------------ */
typedef struct mg_batch mg_batch;
/* One CSR arena holding `count` graphs (vertex ids offset per graph). */
mg_status mg_batch_create(const mg_host_graph *const *graphs, int32_t count, int32_t device, mg_batch **out);
void mg_batch_free(mg_batch *b);
/* BFS from sources[i] in graph i, all graphs in one run; levels_out is the
 * concatenation of the per-graph level arrays. */
mg_status mg_batch_bfs(mg_batch *b, const int32_t *sources, const mg_opts *o, int32_t *levels_out,
                       mg_run_info *info);
/* CC of every graph in one run; labels are per-graph minimum vertex ids. */
mg_status mg_batch_cc(mg_batch *b, const mg_opts *o, int32_t *labels_out, mg_run_info *info);

/* ------------------------------------------------------------------------ */
/* autotuner (replaces the sampling heuristic process.cu:1115-1246 and the   */
/* compile-time constants common.h:10-52)                                   */
/* ------------------------------------------------------------------------ */
/* Times candidate switch thresholds on this graph for `algo` (MG_ALGO_BFS,
 * _SSSP, _BC), writes the best into *tuned and, when cache_path is non-NULL,
 * records it in that file keyed by a graph signature (reused on the next
 * call).  MG_ALGO_PR tunes the pull layout instead: the heavy-row threshold,
 * the chunk size and the thread-bin cutoff of the degree bins, applied to
 * the graph itself (every pull kernel uses them; *tuned is left as passed,
 * `source` is ignored). */
enum { MG_ALGO_BFS = 0, MG_ALGO_SSSP = 1, MG_ALGO_BC = 2, MG_ALGO_CC = 3, MG_ALGO_PR = 4 };
mg_status mg_autotune(mg_graph *dg, int32_t algo, int32_t source, const char *cache_path, mg_opts *tuned);

/* ------------------------------------------------------------------------ */
/* PageRank without allocation (no counterpart in the reference)            */
/* ------------------------------------------------------------------------ */
/* For callers that cannot call cudaMalloc -- code running inside a custom
 * device allocator or pool callback, applications that reserve all device
 * memory at start-up, latency-bound loops where an allocation could
 * synchronise the device.  The caller passes device arrays it already owns:
 * a symmetric CSR (d_row [nv+1] with d_row[0] == 0 and d_row[nv] == ne,
 * checked; d_col [ne], every edge stored both ways as the loader's
 * MG_LOAD_SYM produces it) and d_rank [nv] for the result.  damping 0
 * selects 0.85, otherwise it must lie in (0, 1); tol 0 selects 1e-6,
 * otherwise it must be positive (MG_ERR_INVALID).
 * Every intermediate lives in one fixed device array inside libmg sized for
 * MG_NOALLOC_MAX_VERTICES vertices (about 12 MB, held by each GPU that loads
 * the library until the process exits); larger graphs are rejected with
 * MG_ERR_RANGE.  Nothing is allocated: no cudaMalloc, cudaFree or allocating
 * library call.  Same result as mg_pagerank(MG_PR_TOPOLOGY): normalised
 * PageRank from x = 1/n until the L1 change <= tol.  Works on the current
 * device and enqueues on `stream` (a cudaStream_t, NULL = default stream);
 * the call waits for that stream before it returns (it reads the
 * convergence word back after every batch of 8 sweeps), so it must not be
 * called on a stream that is being captured.  All calls share the array:
 * calls that overlap on the GPU race. */
#define MG_NOALLOC_MAX_VERTICES (1 << 20)
mg_status mg_pagerank_noalloc(const int32_t *d_row, const int32_t *d_col, int32_t nv, int32_t ne, float damping,
                              float tol, int32_t max_iter, float *d_rank, void *stream, int32_t *iterations_out,
                              double *residual_out);

/* ------------------------------------------------------------------------ */
/* self-checks (host only, no GPU)                                           */
/* ------------------------------------------------------------------------ */
/* Build PageRank's segmented shared-memory layout from a host pull CSR
 * (row [nv+1], col [ne], the engine's vertex order) on `threads` host
 * threads and on one, require the two builds to be equal, and verify every
 * invariant the segmented sweep and the row finish rely on: each in-edge
 * below the segments' reach in exactly one piece of its (row, segment) pair,
 * pieces of at most 64 edges with the full ones first, groups of equal-
 * length pieces with padding that reads a zero, every piece in exactly one
 * slot of the row-major sums in segment order, the rest of a row's in-edges
 * in its tail, and the list of rows the finish sums a warp each.  Sums are
 * checked exactly (each edge's id + 1 stands in for its contribution).
 * *pieces_out = the pieces (0 when the layout would not be used).  Returns
 * MG_OK, MG_ERR_INVALID for a malformed CSR, or MG_ERR_INTERNAL with the
 * first violation in mg_last_error().  No counterpart in the reference: it
 * tests this library's layout builder on CPU-only machines. */
mg_status mg_selftest_segmented_layout(int32_t nv, int64_t ne, const int32_t *row, const int32_t *col,
                                       int32_t threads, int64_t *pieces_out);

#ifdef __cplusplus
}
#endif
#endif /* MG_H */
