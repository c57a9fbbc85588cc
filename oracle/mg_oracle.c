/*
 * mg_oracle.c -- CPU oracle (test infrastructure only; see mg_oracle.h).
 *
 * Every function names the reference lines it restates.  The code is written
 * for clarity and for agreement with the reference's sequential order of
 * operations, not for speed: it is the checker, never the thing measured or
 * shipped.
 */
#include "mg_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* loader: read_input.cu:11-254                                              */
/* ------------------------------------------------------------------------ */

typedef struct { int32_t src, dst, val; int64_t ord; } orc_edge;

static int cmp_edge(const void *a, const void *b)
{
    const orc_edge *x = (const orc_edge *)a, *y = (const orc_edge *)b;
    if (x->src != y->src) return x->src < y->src ? -1 : 1;       /* compare1, :4-9 */
    if (x->dst != y->dst) return x->dst < y->dst ? -1 : 1;
    /* the reference's qsort leaves equal (src,dst) pairs unordered; keep file order */
    return x->ord < y->ord ? -1 : (x->ord > y->ord);
}

uint32_t orc_pattern_weight(uint64_t seed, uint64_t entry)
{
    /* splitmix64 finaliser of (seed ^ golden*entry) -> 1..64 */
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (entry + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (uint32_t)(z % 64u) + 1u;
}

int orc_load_mtx(const char *path, int32_t source, uint32_t flags, uint64_t seed, orc_csr *out)
{
    char buf[300];
    int sflag, nflag;
    memset(out, 0, sizeof(*out));

    FILE *fp = fopen(path, "r");
    if (!fp) return ORC_ERR_IO;
    if (!fgets(buf, 300, fp)) { fclose(fp); return ORC_ERR_PARSE; }
    /* banner flags, :31-35 */
    sflag = (strstr(buf, "symmetric") != NULL || strstr(buf, "Hermitian") != NULL) ? 1 : 0;
    if (strstr(buf, "pattern") != NULL) nflag = 0;
    else if (strstr(buf, "complex") != NULL) nflag = -1;
    else nflag = 1;
    if (flags & ORC_LOAD_SYM) sflag = 1;   /* :39-41 */
    if (flags & ORC_LOAD_NSYM) sflag = 0;  /* :42-44 */

    /* skip lines that contain '%', :46-50 / :55-56 */
    long size_line_pos = ftell(fp);
    for (;;) {
        size_line_pos = ftell(fp);
        if (!fgets(buf, 300, fp)) { fclose(fp); return ORC_ERR_PARSE; }
        if (strstr(buf, "%") == NULL) break;
    }
    fseek(fp, size_line_pos, SEEK_SET);

    int nv, dummy, ne;
    if (fscanf(fp, "%d %d %d", &nv, &dummy, &ne) != 3) { fclose(fp); return ORC_ERR_PARSE; }  /* :58 */
    if (nv < 0 || ne < 0) { fclose(fp); return ORC_ERR_PARSE; }
    if (source < 0 || source >= nv) { fclose(fp); return ORC_ERR_RANGE; }
    long long ne_all = (long long)ne * (sflag + 1);                                           /* :59 */
    orc_edge *tv = (orc_edge *)malloc(sizeof(orc_edge) * (size_t)(ne_all > 0 ? ne_all : 1));
    if (!tv) { fclose(fp); return ORC_ERR_OOM; }

    long long i;
    int64_t entry = 0;
    for (i = 0; i < ne_all; i++, entry++) {                                                   /* :69-96 */
        int s, d;
        if (fscanf(fp, "%d %d", &s, &d) != 2) { free(tv); fclose(fp); return ORC_ERR_PARSE; }
        s--; d--;
        if (s < 0 || s >= nv || d < 0 || d >= nv) { free(tv); fclose(fp); return ORC_ERR_RANGE; }
        int val;
        if (nflag == 0) val = (int)orc_pattern_weight(seed, (uint64_t)entry);
        else if (nflag == 1) {
            float f;
            if (fscanf(fp, " %f ", &f) != 1) { free(tv); fclose(fp); return ORC_ERR_PARSE; }
            val = (int)f;
        } else {
            float f1, f2;
            if (fscanf(fp, " %f %f ", &f1, &f2) != 2) { free(tv); fclose(fp); return ORC_ERR_PARSE; }
            val = (int)f1;
        }
        tv[i].src = s; tv[i].dst = d; tv[i].val = val; tv[i].ord = 2 * entry;
        if (sflag == 1) {
            i++;
            tv[i].src = d; tv[i].dst = s; tv[i].val = val; tv[i].ord = 2 * entry + 1;
        }
    }
    fclose(fp);
    long long m0 = ne_all;
    qsort(tv, (size_t)m0, sizeof(orc_edge), cmp_edge);                                         /* :97 */

    /* dedup + unused-vertex removal, :100-139.  Note: valid[] is marked from
     * entry 1 on (entry 0 never marks its endpoints) and entry 0 is always
     * kept, also under the CC filter -- both as in the reference. */
    int32_t *loc = (int32_t *)calloc((size_t)m0 + 1, sizeof(int32_t));
    int32_t *valid = (int32_t *)calloc((size_t)nv + 1, sizeof(int32_t));
    if (!loc || !valid) { free(tv); free(loc); free(valid); return ORC_ERR_OOM; }
    if (m0 > 0) loc[0] = 1;
    for (i = 1; i < m0; i++) {
        valid[tv[i].src] = 1; valid[tv[i].dst] = 1;
        loc[i] = (tv[i].src == tv[i - 1].src && tv[i].dst == tv[i - 1].dst) ? 0 : 1;
        if ((flags & ORC_LOAD_CC) && tv[i].src >= tv[i].dst) loc[i] = 0;
    }
    /* exclusive scans */
    {
        int32_t run = 0;
        for (int v = 0; v <= nv; v++) { int32_t t = valid[v]; valid[v] = run; run += (v < nv) ? t : 0; }
        /* valid[nv] = number of kept vertices */
    }
    {
        int32_t run = 0;
        for (i = 0; i <= m0; i++) { int32_t t = loc[i]; loc[i] = run; run += (i < m0) ? t : 0; }
    }
    out->start_p = valid[source];                                                              /* :130 */
    for (i = 0; i < m0; i++) {                                                                 /* :135-139 */
        int32_t k = loc[i];
        tv[k].src = valid[tv[i].src];
        tv[k].dst = valid[tv[i].dst];
        tv[k].val = tv[i].val;
    }
    int32_t nv2 = valid[nv], ne2 = loc[m0];                                                    /* :147 */
    /* sorted entry 0 never marks its endpoints; if one maps to nv2 the
     * reference writes past csc_v -- report the graph as out of range */
    if (ne2 > 0 && (tv[0].src >= nv2 || tv[0].dst >= nv2)) {
        free(tv); free(loc); free(valid); return ORC_ERR_RANGE;
    }
    out->nv = nv2; out->ne = ne2;

    /* CSR, :152-171 */
    out->csc_v = (int32_t *)calloc((size_t)nv2 + 1, sizeof(int32_t));
    out->csc_e = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ne2 > 0 ? ne2 : 1));
    out->csc_ev = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ne2 > 0 ? ne2 : 1));
    if (!out->csc_v || !out->csc_e || !out->csc_ev) {
        free(tv); free(loc); free(valid); orc_csr_free(out); return ORC_ERR_OOM;
    }
    for (i = 0; i < ne2; i++) {
        out->csc_e[i] = tv[i].dst;
        out->csc_ev[i] = tv[i].val;
        out->csc_v[1 + tv[i].src] = (int32_t)i + 1;
    }
    out->tra = 0;
    for (int v = 1; v < nv2; v++) {
        if (out->csc_v[v] == 0) out->csc_v[v] = out->csc_v[v - 1];
        else if (out->csc_v[v] - out->csc_v[v - 1] >= 128) out->tra = 1;
    }
    out->csc_v[nv2] = ne2;
    free(tv); free(loc); free(valid);
    return ORC_OK;
}

void orc_csr_free(orc_csr *g)
{
    free(g->csc_v); free(g->csc_e); free(g->csc_ev);
    g->csc_v = g->csc_e = g->csc_ev = NULL;
}

/* ------------------------------------------------------------------------ */
/* validate.cu:106-130 -- BFS                                                */
/* ------------------------------------------------------------------------ */
void orc_bfs(const orc_csr *g, int32_t src, int32_t *level)
{
    int32_t nv = g->nv;
    int32_t *q = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nv > 0 ? nv : 1));
    for (int32_t i = 0; i < nv; i++) level[i] = ORC_IUNUSED;
    if (nv == 0) { free(q); return; }
    level[src] = 0; q[0] = src;
    long long head = 0, tail = 1;
    while (head != tail) {
        int32_t u = q[head % nv]; head++;
        for (int32_t j = g->csc_v[u]; j < g->csc_v[u + 1]; j++) {
            int32_t k = g->csc_e[j];
            if (level[k] == ORC_IUNUSED) { level[k] = level[u] + 1; q[tail % nv] = k; tail++; }
        }
    }
    free(q);
}

/* ------------------------------------------------------------------------ */
/* validate.cu:131-148 -- Bellman-Ford in vertex order                       */
/* ------------------------------------------------------------------------ */
int orc_sssp(const orc_csr *g, int32_t src, int32_t *dist, int32_t max_sweeps)
{
    int32_t nv = g->nv;
    for (int32_t i = 0; i < nv; i++) dist[i] = ORC_IUNUSED;
    if (nv == 0) return 0;
    dist[src] = 0;
    int sweeps = 0;
    for (;;) {
        int conv = 1;
        sweeps++;
        for (int32_t i = 0; i < nv; i++) {
            for (int32_t j = g->csc_v[i]; j < g->csc_v[i + 1]; j++) {
                int32_t k = g->csc_e[j];
                if (dist[i] + g->csc_ev[j] < dist[k]) { conv = 0; dist[k] = dist[i] + g->csc_ev[j]; }
            }
        }
        if (conv || (max_sweeps > 0 && sweeps >= max_sweeps)) break;
    }
    return sweeps;
}

/* ------------------------------------------------------------------------ */
/* validate.cu:149-189 -- Brandes (reference types: int sigma, float delta)  */
/* ------------------------------------------------------------------------ */
void orc_bc(const orc_csr *g, int32_t src, int32_t *level, int32_t *sigma, float *delta)
{
    int32_t nv = g->nv;
    int32_t *q = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nv > 0 ? nv : 1));
    for (int32_t i = 0; i < nv; i++) { level[i] = ORC_IUNUSED; sigma[i] = 0; delta[i] = 0.0f; }
    if (nv == 0) { free(q); return; }
    level[src] = 0; sigma[src] = 1; q[0] = src;
    int32_t head = 0, tail = 1;
    while (head != tail) {
        int32_t u = q[head++];
        for (int32_t j = g->csc_v[u]; j < g->csc_v[u + 1]; j++) {
            int32_t k = g->csc_e[j];
            if (level[k] == ORC_IUNUSED) { level[k] = level[u] + 1; q[tail++] = k; }
            if (level[u] + 1 == level[k]) sigma[k] += sigma[u];
        }
    }
    for (int32_t i = tail - 1; i >= 0; i--) {
        int32_t w = q[i];
        for (int32_t j = g->csc_v[w]; j < g->csc_v[w + 1]; j++) {
            int32_t k = g->csc_e[j];
            if (level[k] == level[w] - 1)
                delta[k] += ((float)sigma[k] / sigma[w]) * (1.0f + delta[w]);
        }
    }
    free(q);
}

void orc_bc_f64(const orc_csr *g, int32_t src, int32_t *level, double *sigma, double *delta)
{
    int32_t nv = g->nv;
    int32_t *q = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nv > 0 ? nv : 1));
    for (int32_t i = 0; i < nv; i++) { level[i] = ORC_IUNUSED; sigma[i] = 0.0; delta[i] = 0.0; }
    if (nv == 0) { free(q); return; }
    level[src] = 0; sigma[src] = 1.0; q[0] = src;
    int32_t head = 0, tail = 1;
    while (head != tail) {
        int32_t u = q[head++];
        for (int32_t j = g->csc_v[u]; j < g->csc_v[u + 1]; j++) {
            int32_t k = g->csc_e[j];
            if (level[k] == ORC_IUNUSED) { level[k] = level[u] + 1; q[tail++] = k; }
            if (level[u] + 1 == level[k]) sigma[k] += sigma[u];
        }
    }
    for (int32_t i = tail - 1; i >= 0; i--) {
        int32_t w = q[i];
        for (int32_t j = g->csc_v[w]; j < g->csc_v[w + 1]; j++) {
            int32_t k = g->csc_e[j];
            if (level[k] == level[w] - 1) delta[k] += (sigma[k] / sigma[w]) * (1.0 + delta[w]);
        }
    }
    free(q);
}

void orc_bc_multi_f64(const orc_csr *g, const int32_t *src, int32_t nsrc, double *bc)
{
    int32_t nv = g->nv;
    int32_t *lv = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nv > 0 ? nv : 1));
    double *sg = (double *)malloc(sizeof(double) * (size_t)(nv > 0 ? nv : 1));
    double *dl = (double *)malloc(sizeof(double) * (size_t)(nv > 0 ? nv : 1));
    for (int32_t i = 0; i < nv; i++) bc[i] = 0.0;
    for (int32_t s = 0; s < nsrc; s++) {
        orc_bc_f64(g, src[s], lv, sg, dl);
        for (int32_t i = 0; i < nv; i++) if (i != src[s]) bc[i] += dl[i];
    }
    free(lv); free(sg); free(dl);
}

/* The same Brandes sweeps (validate.cu:149-189 order) with long-double path
 * counts and dependencies. */
void orc_bc_ext(const orc_csr *g, int32_t src, int32_t *level, double *log2sigma, double *delta)
{
    int32_t nv = g->nv;
    size_t cnt = (size_t)(nv > 0 ? nv : 1);
    int32_t *q = (int32_t *)malloc(sizeof(int32_t) * cnt);
    long double *sg = (long double *)malloc(sizeof(long double) * cnt);
    long double *dl = (long double *)malloc(sizeof(long double) * cnt);
    for (int32_t i = 0; i < nv; i++) { level[i] = ORC_IUNUSED; sg[i] = 0.0L; dl[i] = 0.0L; }
    if (nv > 0) {
        level[src] = 0; sg[src] = 1.0L; q[0] = src;
        int32_t head = 0, tail = 1;
        while (head != tail) {
            int32_t u = q[head++];
            for (int32_t j = g->csc_v[u]; j < g->csc_v[u + 1]; j++) {
                int32_t k = g->csc_e[j];
                if (level[k] == ORC_IUNUSED) { level[k] = level[u] + 1; q[tail++] = k; }
                if (level[u] + 1 == level[k]) sg[k] += sg[u];
            }
        }
        for (int32_t i = tail - 1; i >= 0; i--) {
            int32_t w = q[i];
            for (int32_t j = g->csc_v[w]; j < g->csc_v[w + 1]; j++) {
                int32_t k = g->csc_e[j];
                if (level[k] == level[w] - 1) dl[k] += (sg[k] / sg[w]) * (1.0L + dl[w]);
            }
        }
    }
    for (int32_t i = 0; i < nv; i++) {
        log2sigma[i] = sg[i] > 0.0L ? (double)log2l(sg[i]) : -1.0;
        delta[i] = (double)dl[i];
    }
    free(q); free(sg); free(dl);
}

void orc_bc_multi_ext(const orc_csr *g, const int32_t *src, int32_t nsrc, double *bc)
{
    int32_t nv = g->nv;
    size_t cnt = (size_t)(nv > 0 ? nv : 1);
    int32_t *lv = (int32_t *)malloc(sizeof(int32_t) * cnt);
    double *ls = (double *)malloc(sizeof(double) * cnt);
    double *dl = (double *)malloc(sizeof(double) * cnt);
    for (int32_t i = 0; i < nv; i++) bc[i] = 0.0;
    for (int32_t s = 0; s < nsrc; s++) {
        orc_bc_ext(g, src[s], lv, ls, dl);
        for (int32_t i = 0; i < nv; i++) if (i != src[s]) bc[i] += dl[i];
    }
    free(lv); free(ls); free(dl);
}

/* ------------------------------------------------------------------------ */
/* validate.cu:223-308 -- CC                                                 */
/* ------------------------------------------------------------------------ */
int orc_cc_minlabel(const orc_csr *g, int32_t *c)
{
    int32_t nv = g->nv;
    for (int32_t i = 0; i < nv; i++) c[i] = i;                      /* :245-246 */
    int sweeps = 0;
    for (;;) {                                                      /* :249-261 */
        int pflag = 0;
        sweeps++;
        for (int32_t i = 0; i < nv; i++) {
            for (int32_t j = g->csc_v[i]; j < g->csc_v[i + 1]; j++) {
                int32_t k = g->csc_e[j];
                if (c[i] != c[k]) {
                    int32_t a = c[i] < c[k] ? c[i] : c[k];
                    c[i] = a;
                    c[k] = a < c[k] ? a : c[k];
                    pflag = 1;
                }
            }
        }
        if (!pflag) break;
    }
    return sweeps;
}

void orc_cc_relabel(int32_t nv, int32_t *label)
{
    /* :263-273: first appearance in vertex order gets 0, 1, 2, ...  Labels
     * are vertex ids in [0, nv). */
    int32_t *adj = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nv > 0 ? nv : 1));
    for (int32_t i = 0; i < nv; i++) adj[i] = -1;
    int32_t k = 0;
    for (int32_t i = 0; i < nv; i++) if (adj[label[i]] < 0) adj[label[i]] = k++;
    for (int32_t i = 0; i < nv; i++) label[i] = adj[label[i]];
    free(adj);
}

/* ------------------------------------------------------------------------ */
/* validate.cu:34-91 -- reference PR recurrences (PR_T mode 0, PR_D mode 1)  */
/* constants: common.h:58-61                                                 */
/* ------------------------------------------------------------------------ */
int orc_pr_ref(const orc_csr *g, int mode, float *pr, int32_t max_iter)
{
    const float D = 0.85f, TOL = 0.01f;
    int32_t nv = g->nv;
    float *nx = (float *)malloc(sizeof(float) * (size_t)(nv > 0 ? nv : 1));
    int32_t *mark = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nv > 0 ? nv : 1));
    for (int32_t i = 0; i < nv; i++) { pr[i] = 0.0f; mark[i] = 1; }
    int it = 0;
    for (;;) {
        int flag = 0;
        it++;
        memset(nx, 0, sizeof(float) * (size_t)nv);
        for (int32_t i = 0; i < nv; i++) {
            int32_t deg = g->csc_v[i + 1] - g->csc_v[i];
            for (int32_t j = g->csc_v[i]; j < g->csc_v[i + 1]; j++)
                if (deg > 0) nx[g->csc_e[j]] += pr[i] / (float)deg;
        }
        for (int32_t i = 0; i < nv; i++) {
            float f1 = (1 - D) + nx[i] * D;
            float f2 = pr[i];
            if (mode == 0) {
                if (fabsf(f1 - f2) > TOL) { pr[i] = f1; flag = 1; }
            } else {
                if (mark[i] == 1 && fabsf(f1 - f2) > TOL * f2) { pr[i] = f1; flag = 1; }
                else { pr[i] = f1; mark[i] = 0; }
            }
        }
        if (!flag || (max_iter > 0 && it >= max_iter)) break;
    }
    free(nx); free(mark);
    return it;
}

int orc_pr_ref_f64(const orc_csr *g, int mode, double *pr, int32_t max_iter)
{
    const double D = 0.85, TOL = 0.01;
    int32_t nv = g->nv;
    double *nx = (double *)malloc(sizeof(double) * (size_t)(nv > 0 ? nv : 1));
    int32_t *mark = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nv > 0 ? nv : 1));
    for (int32_t i = 0; i < nv; i++) { pr[i] = 0.0; mark[i] = 1; }
    int it = 0;
    for (;;) {
        int flag = 0;
        it++;
        for (int32_t i = 0; i < nv; i++) nx[i] = 0.0;
        for (int32_t i = 0; i < nv; i++) {
            int32_t deg = g->csc_v[i + 1] - g->csc_v[i];
            for (int32_t j = g->csc_v[i]; j < g->csc_v[i + 1]; j++)
                if (deg > 0) nx[g->csc_e[j]] += pr[i] / (double)deg;
        }
        for (int32_t i = 0; i < nv; i++) {
            double f1 = (1 - D) + nx[i] * D, f2 = pr[i];
            if (mode == 0) { if (fabs(f1 - f2) > TOL) { pr[i] = f1; flag = 1; } }
            else {
                if (mark[i] == 1 && fabs(f1 - f2) > TOL * f2) { pr[i] = f1; flag = 1; }
                else { pr[i] = f1; mark[i] = 0; }
            }
        }
        if (!flag || (max_iter > 0 && it >= max_iter)) break;
    }
    free(nx); free(mark);
    return it;
}

/* ------------------------------------------------------------------------ */
/* Normalised and personalised PageRank (FP64 extension)                     */
/* ------------------------------------------------------------------------ */
static int pr_norm_core(const orc_csr *g, int32_t seed, double d, double tol, int32_t max_iter, double *x)
{
    int32_t nv = g->nv;
    if (nv == 0) return 0;
    double *c = (double *)malloc(sizeof(double) * (size_t)nv);
    double *nx = (double *)malloc(sizeof(double) * (size_t)nv);
    for (int32_t i = 0; i < nv; i++) x[i] = (seed < 0) ? 1.0 / nv : (i == seed ? 1.0 : 0.0);
    int it = 0;
    for (;;) {
        it++;
        double dangling = 0.0;
        for (int32_t u = 0; u < nv; u++) {
            int32_t deg = g->csc_v[u + 1] - g->csc_v[u];
            if (deg > 0) c[u] = x[u] / deg; else { c[u] = 0.0; dangling += x[u]; }
        }
        /* push over out-edges: nx[v] = sum over edges (u -> v) of x_u / deg_u */
        for (int32_t v = 0; v < nv; v++) nx[v] = 0.0;
        for (int32_t u = 0; u < nv; u++)
            for (int32_t j = g->csc_v[u]; j < g->csc_v[u + 1]; j++) nx[g->csc_e[j]] += c[u];
        double resid = 0.0;
        for (int32_t v = 0; v < nv; v++) {
            double base;
            if (seed < 0) base = (1.0 - d) / nv + d * dangling / nv;
            else base = (v == seed) ? (1.0 - d) + d * dangling : 0.0;
            nx[v] = base + d * nx[v];
            resid += fabs(nx[v] - x[v]);
        }
        memcpy(x, nx, sizeof(double) * (size_t)nv);
        if (resid <= tol || (max_iter > 0 && it >= max_iter)) break;
    }
    free(c); free(nx);
    return it;
}

int orc_pr_norm_f64(const orc_csr *g, double damping, double tol, int32_t max_iter, double *x)
{
    return pr_norm_core(g, -1, damping, tol, max_iter, x);
}

int orc_ppr_f64(const orc_csr *g, int32_t seed, double damping, double tol, int32_t max_iter, double *x)
{
    return pr_norm_core(g, seed, damping, tol, max_iter, x);
}

/* ------------------------------------------------------------------------ */
/* Weighted PageRank + adjoint (FP64 extension)                              */
/* ------------------------------------------------------------------------ */
int orc_wpr_f64(const orc_csr *g, const double *w, double d, double tol, int32_t max_iter, double *x)
{
    int32_t nv = g->nv;
    if (nv == 0) return 0;
    double *S = (double *)calloc((size_t)nv, sizeof(double));
    double *nx = (double *)malloc(sizeof(double) * (size_t)nv);
    for (int32_t u = 0; u < nv; u++)
        for (int32_t j = g->csc_v[u]; j < g->csc_v[u + 1]; j++) S[u] += w[j];
    for (int32_t i = 0; i < nv; i++) x[i] = 1.0 / nv;
    int it = 0;
    for (;;) {
        it++;
        double dangling = 0.0;
        for (int32_t u = 0; u < nv; u++) { nx[u] = 0.0; if (S[u] == 0.0) dangling += x[u]; }
        /* push form: nx[v] += P_uv x_u over every CSR entry (u -> v) */
        for (int32_t u = 0; u < nv; u++) {
            if (S[u] == 0.0) continue;
            for (int32_t j = g->csc_v[u]; j < g->csc_v[u + 1]; j++) nx[g->csc_e[j]] += w[j] / S[u] * x[u];
        }
        double resid = 0.0;
        for (int32_t v = 0; v < nv; v++) {
            double val = (1.0 - d) / nv + d * dangling / nv + d * nx[v];
            resid += fabs(val - x[v]);
            nx[v] = val;
        }
        memcpy(x, nx, sizeof(double) * (size_t)nv);
        if (resid <= tol || (max_iter > 0 && it >= max_iter)) break;
    }
    free(S); free(nx);
    return it;
}

int orc_wpr_adjoint_f64(const orc_csr *g, const double *w, const double *x, const double *gv,
                        double d, double tol, int32_t max_iter, double *lam, double *grad_w, double *grad_p)
{
    /* Adjoint of x = (1-d)/n + d*(P^T x + dangling(x)/n):
     *   lambda = g + d*(P lambda + [S_u == 0] * mean(lambda))
     * For graphs with no dangling rows the second term vanishes. */
    int32_t nv = g->nv;
    if (nv == 0) return 0;
    double *S = (double *)calloc((size_t)nv, sizeof(double));
    double *nl = (double *)malloc(sizeof(double) * (size_t)nv);
    double *t = (double *)malloc(sizeof(double) * (size_t)nv);
    for (int32_t u = 0; u < nv; u++)
        for (int32_t j = g->csc_v[u]; j < g->csc_v[u + 1]; j++) S[u] += w[j];
    for (int32_t i = 0; i < nv; i++) lam[i] = gv[i];
    int it = 0;
    for (;;) {
        it++;
        double mean = 0.0;
        for (int32_t i = 0; i < nv; i++) mean += lam[i];
        mean /= nv;
        double resid = 0.0;
        for (int32_t u = 0; u < nv; u++) {
            double s = 0.0;
            if (S[u] != 0.0) {
                for (int32_t j = g->csc_v[u]; j < g->csc_v[u + 1]; j++) s += w[j] / S[u] * lam[g->csc_e[j]];
            } else {
                s = mean;
            }
            nl[u] = gv[u] + d * s;
            resid += fabs(nl[u] - lam[u]);
        }
        memcpy(lam, nl, sizeof(double) * (size_t)nv);
        if (resid <= tol || (max_iter > 0 && it >= max_iter)) break;
    }
    for (int32_t u = 0; u < nv; u++) {
        double s = 0.0;
        if (S[u] != 0.0)
            for (int32_t j = g->csc_v[u]; j < g->csc_v[u + 1]; j++) s += w[j] / S[u] * lam[g->csc_e[j]];
        t[u] = s;
    }
    for (int32_t u = 0; u < nv; u++) {
        for (int32_t j = g->csc_v[u]; j < g->csc_v[u + 1]; j++) {
            int32_t v = g->csc_e[j];
            if (grad_p) grad_p[j] = d * x[u] * lam[v];
            if (grad_w) grad_w[j] = (S[u] != 0.0) ? d * x[u] / S[u] * (lam[v] - t[u]) : 0.0;
        }
    }
    free(S); free(nl); free(t);
    return it;
}

double orc_wpr_loss_f64(const orc_csr *g, const double *w, const double *gv, double d, double tol, int32_t max_iter)
{
    int32_t nv = g->nv;
    double *x = (double *)malloc(sizeof(double) * (size_t)(nv > 0 ? nv : 1));
    orc_wpr_f64(g, w, d, tol, max_iter, x);
    double L = 0.0;
    for (int32_t i = 0; i < nv; i++) L += gv[i] * x[i];
    free(x);
    return L;
}
