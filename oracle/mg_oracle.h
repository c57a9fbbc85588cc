/*
 * mg_oracle.h -- CPU oracle for the frontier-processing path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: it restates, in
 * plain C, the CPU algorithms of the reference's code/validate.cu and the
 * MTX loader of code/read_input.cu, plus the FP64 extensions the accuracy
 * contracts need (FP64-sigma Brandes, normalised / personalised PageRank and
 * the PageRank edge-weight adjoint).  Only the tests, the smoke check and the
 * CPU-baseline leg of bench.py may load it; the product library never does.
 *
 * Parity pins: the loader and the BFS / SSSP / CC / PR outputs of this
 * restatement are checked against the reference's own generate_CSC and
 * verifyResults, compiled from the reference sources by oracle/Makefile into
 * oracle/_ref/ (see tests/test_oracle_ref.py and tests/golden/).
 */
#ifndef MG_ORACLE_H
#define MG_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 0x64646464: the reference's "unreached" label (common.h:37-39). */
#define ORC_IUNUSED 0x64646464

/* loader flags (read_input.cu:31-44, :111-113) */
#define ORC_LOAD_SYM     1u  /* -DSYM: force symmetric */
#define ORC_LOAD_NSYM    2u  /* -DNSYM: force general */
#define ORC_LOAD_CC      4u  /* -DCC: keep only src<dst edges */

typedef struct orc_csr {
    int32_t nv, ne;        /* after dedup + compaction                 */
    int32_t start_p;       /* source renumbered through compaction     */
    int32_t tra;           /* any degree >= 128 (read_input.cu:169)     */
    int32_t *csc_v;        /* [nv+1]                                    */
    int32_t *csc_e;        /* [ne]                                      */
    int32_t *csc_ev;       /* [ne] integer weights                      */
} orc_csr;

/* Status codes shared with the product library's mg_status values. */
enum { ORC_OK = 0, ORC_ERR_IO = 1, ORC_ERR_PARSE = 2, ORC_ERR_RANGE = 3, ORC_ERR_OOM = 4 };

/* read_input.cu:11-254.  Pattern files get weights 1 + (splitmix64(seed ^ i) % 64)
 * where i is the 0-based entry index in the file (the reference uses rand()
 * seeded by time(), which is not reproducible). */
int  orc_load_mtx(const char *path, int32_t source, uint32_t flags, uint64_t seed, orc_csr *out);
void orc_csr_free(orc_csr *g);
/* The same pipeline from an in-memory entry list (0-based ids in file order;
 * val may be NULL for weight 1); ORC_LOAD_SYM adds each entry's mirror right
 * after it, as the loader does for symmetric files (read_input.cu:88-96). */
int  orc_from_entries(int32_t nv_decl, int64_t nentries, const int32_t *src, const int32_t *dst,
                      const int32_t *val, int32_t source, uint32_t flags, orc_csr *out);
/* R-MAT (Chakrabarti, Zhan, Faloutsos 2004): edge_factor * 2^scale draws of
 * scale quadrant choices each (probabilities a, b, c, 1-a-b-c), draw i
 * seeded with seed * 0xD1B54A32D192ED03 + i through splitmix64, self-loops
 * dropped, integer weight wmin + (next draw % (wmax - wmin + 1)); then the
 * symmetric loader pipeline above with source 0.  The synthetic input of
 * the benchmarks, generated without the product library. */
int  orc_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed,
                  int32_t wmin, int32_t wmax, orc_csr *out);
uint32_t orc_pattern_weight(uint64_t seed, uint64_t entry);

/* validate.cu:106-130 -- FIFO BFS levels, ORC_IUNUSED for unreached. */
void orc_bfs(const orc_csr *g, int32_t src, int32_t *level);
/* validate.cu:131-148 -- Bellman-Ford sweeps in vertex order.  Returns sweeps. */
int  orc_sssp(const orc_csr *g, int32_t src, int32_t *dist, int32_t max_sweeps);
/* validate.cu:149-189 -- Brandes: int sigma, float delta (reference types). */
void orc_bc(const orc_csr *g, int32_t src, int32_t *level, int32_t *sigma, float *delta);
/* FP64 extension: sigma and delta in double. */
void orc_bc_f64(const orc_csr *g, int32_t src, int32_t *level, double *sigma, double *delta);
/* Multi-source BC scores: sum over sources of delta_s(v), v != s, FP64. */
void orc_bc_multi_f64(const orc_csr *g, const int32_t *src, int32_t nsrc, double *bc);
/* Brandes with long-double path counts (15-bit exponent on x86 and aarch64:
 * counts up to ~1e4932, past the FP64 range that lattices with thousands of
 * levels reach).  log2sigma[v] = log2 of the path count (-1 when unreached),
 * delta in long double rounded to FP64. */
void orc_bc_ext(const orc_csr *g, int32_t src, int32_t *level, double *log2sigma, double *delta);
void orc_bc_multi_ext(const orc_csr *g, const int32_t *src, int32_t nsrc, double *bc);
/* validate.cu:223-273 -- min-label propagation to the fixed point (labels = min id). */
int  orc_cc_minlabel(const orc_csr *g, int32_t *label);
/* validate.cu:234-242 / :263-273 -- relabel by first appearance, in place. */
void orc_cc_relabel(int32_t nv, int32_t *label);
/* validate.cu:34-91 -- reference PR recurrence in FP32 (PR_T: mode 0, PR_D: mode 1).
 * Returns the number of sweeps. */
int  orc_pr_ref(const orc_csr *g, int mode, float *pr, int32_t max_iter);
/* same recurrence in FP64 */
int  orc_pr_ref_f64(const orc_csr *g, int mode, double *pr, int32_t max_iter);
/* Normalised PageRank in FP64: x' = (1-d)/n + d*(sum_u x_u/deg_u + dangling/n).
 * Jacobi sweeps from x = 1/n until the L1 change <= tol.  Returns sweeps. */
int  orc_pr_norm_f64(const orc_csr *g, double damping, double tol, int32_t max_iter, double *x);
/* Personalised PageRank (one-hot seed): x' = (1-d)*e_seed + d*(P^T x + dangling*e_seed). */
int  orc_ppr_f64(const orc_csr *g, int32_t seed, double damping, double tol, int32_t max_iter, double *x);

/* Weighted PageRank and its adjoint (FP64).  w[e] is the weight of CSR entry e
 * (row u -> col v).  P_uv = w_uv / S_u with S_u the row sum.
 *   forward : x = (1-d)/n + d * P^T x
 *   loss    : L = sum_i g_i x_i
 *   adjoint : lambda = g + d * P lambda
 *   grad_w  : dL/dw_e = (d x_u / S_u) * (lambda_v - sum_k P_uk lambda_k)
 *   grad_p  : dL/dP_e = d x_u lambda_v                                    */
int    orc_wpr_f64(const orc_csr *g, const double *w, double damping, double tol, int32_t max_iter, double *x);
int    orc_wpr_adjoint_f64(const orc_csr *g, const double *w, const double *x, const double *gvec,
                           double damping, double tol, int32_t max_iter, double *lambda,
                           double *grad_w, double *grad_p);
double orc_wpr_loss_f64(const orc_csr *g, const double *w, const double *gvec, double damping,
                        double tol, int32_t max_iter);
/* Central finite differences (L(w + eps e_j) - L(w - eps e_j)) / (2 eps) of
 * L = sum_i g_i x_i for the k CSR entries listed, each perturbed loss from a
 * complete FP64 solve (written as the converged x plus the fixed point of
 * the perturbation, all 2k solved together on nthreads host threads, until
 * each one's L1 change <= rtol times its L1 norm).  x: orc_wpr_f64's result
 * for w.  Returns the sweeps taken (-1: out of memory). */
int    orc_wpr_fd_f64(const orc_csr *g, const double *w, const double *x, const double *gvec, double damping,
                      const int32_t *entries, int32_t k, double eps, double rtol, int32_t max_iter,
                      int32_t nthreads, double *fd_out);

#ifdef __cplusplus
}
#endif
#endif
