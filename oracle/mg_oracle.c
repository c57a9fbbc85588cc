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

uint32_t orc_pattern_weight(uint64_t seed, uint64_t entry)
{
    /* splitmix64 finaliser of (seed ^ golden*entry) -> 1..64 */
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (entry + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (uint32_t)(z % 64u) + 1u;
}

static int cmp_u64(const void *a, const void *b)
{
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : (x > y);
}

/* read_input.cu:97-171 from the expanded entry list (esrc/edst/eval[i], i
 * in file order with the symmetric mirror right after its entry, :69-96):
 * sort by (src, dst, file order) (compare1, :4-9; the reference's qsort
 * leaves equal pairs unordered, the file order is kept here), drop repeated
 * (src, dst) pairs keeping the first (and src >= dst under the CC filter),
 * remove unused vertices and build the CSR.  The sort is a stable counting
 * sort by src followed by a per-row sort of (dst, rank in row) keys, which
 * gives the same total order as a comparison sort on (src, dst, order). */
static int loader_finish(int32_t nv, int64_t m0, const int32_t *esrc, const int32_t *edst, const int32_t *eval,
                         int32_t source, uint32_t flags, orc_csr *out)
{
    memset(out, 0, sizeof(*out));
    if (m0 > 2147483647LL) return ORC_ERR_RANGE;
    int64_t *rs = (int64_t *)calloc((size_t)nv + 1, sizeof(int64_t));
    int32_t *perm = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m0 > 0 ? m0 : 1));
    uint64_t *key = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(m0 > 0 ? m0 : 1));
    int32_t *ss = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m0 > 0 ? m0 : 1));
    int32_t *sd = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m0 > 0 ? m0 : 1));
    int32_t *sv = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m0 > 0 ? m0 : 1));
    int32_t *loc = (int32_t *)calloc((size_t)m0 + 1, sizeof(int32_t));
    int32_t *valid = (int32_t *)calloc((size_t)nv + 1, sizeof(int32_t));
    int rc = ORC_OK;
    int64_t i;
    if (!rs || !perm || !key || !ss || !sd || !sv || !loc || !valid) { rc = ORC_ERR_OOM; goto done; }
    for (i = 0; i < m0; i++) rs[esrc[i] + 1]++;
    for (int32_t v = 0; v < nv; v++) rs[v + 1] += rs[v];
    {
        int64_t *pos = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nv > 0 ? nv : 1));
        if (!pos) { rc = ORC_ERR_OOM; goto done; }
        memcpy(pos, rs, sizeof(int64_t) * (size_t)nv);
        for (i = 0; i < m0; i++) perm[pos[esrc[i]]++] = (int32_t)i;   /* stable: file order per row */
        free(pos);
    }
    for (int32_t v = 0; v < nv; v++) {
        int64_t b = rs[v], e = rs[v + 1];
        for (int64_t p = b; p < e; p++) key[p] = ((uint64_t)(uint32_t)edst[perm[p]] << 32) | (uint64_t)(p - b);
        qsort(key + b, (size_t)(e - b), sizeof(uint64_t), cmp_u64);
        for (int64_t p = b; p < e; p++) {
            int32_t o = perm[b + (int64_t)(key[p] & 0xffffffffu)];
            ss[p] = v; sd[p] = edst[o]; sv[p] = eval[o];
        }
    }
    /* dedup + unused-vertex removal, :100-139.  Note: valid[] is marked from
     * entry 1 on (entry 0 never marks its endpoints) and entry 0 is always
     * kept, also under the CC filter -- both as in the reference. */
    if (m0 > 0) loc[0] = 1;
    for (i = 1; i < m0; i++) {
        valid[ss[i]] = 1; valid[sd[i]] = 1;
        loc[i] = (ss[i] == ss[i - 1] && sd[i] == sd[i - 1]) ? 0 : 1;
        if ((flags & ORC_LOAD_CC) && ss[i] >= sd[i]) loc[i] = 0;
    }
    {   /* exclusive scans; valid[nv] = number of kept vertices */
        int32_t run = 0;
        for (int32_t v = 0; v <= nv; v++) { int32_t t = valid[v]; valid[v] = run; run += (v < nv) ? t : 0; }
    }
    {
        int32_t run = 0;
        for (i = 0; i <= m0; i++) { int32_t t = loc[i]; loc[i] = run; run += (i < m0) ? t : 0; }
    }
    out->start_p = valid[source];                                                              /* :130 */
    for (i = 0; i < m0; i++) {                                                                 /* :135-139 */
        int32_t k = loc[i];
        ss[k] = valid[ss[i]];
        sd[k] = valid[sd[i]];
        sv[k] = sv[i];
    }
    {
        int32_t nv2 = valid[nv], ne2 = loc[m0];                                                /* :147 */
        /* sorted entry 0 never marks its endpoints; if one maps to nv2 the
         * reference writes past csc_v -- report the graph as out of range */
        if (ne2 > 0 && (ss[0] >= nv2 || sd[0] >= nv2)) { rc = ORC_ERR_RANGE; goto done; }
        out->nv = nv2; out->ne = ne2;
        /* CSR, :152-171 */
        out->csc_v = (int32_t *)calloc((size_t)nv2 + 1, sizeof(int32_t));
        out->csc_e = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ne2 > 0 ? ne2 : 1));
        out->csc_ev = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ne2 > 0 ? ne2 : 1));
        if (!out->csc_v || !out->csc_e || !out->csc_ev) { orc_csr_free(out); rc = ORC_ERR_OOM; goto done; }
        for (i = 0; i < ne2; i++) {
            out->csc_e[i] = sd[i];
            out->csc_ev[i] = sv[i];
            out->csc_v[1 + ss[i]] = (int32_t)i + 1;
        }
        out->tra = 0;
        for (int32_t v = 1; v < nv2; v++) {
            if (out->csc_v[v] == 0) out->csc_v[v] = out->csc_v[v - 1];
            else if (out->csc_v[v] - out->csc_v[v - 1] >= 128) out->tra = 1;
        }
        out->csc_v[nv2] = ne2;
    }
done:
    free(rs); free(perm); free(key); free(ss); free(sd); free(sv); free(loc); free(valid);
    return rc;
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
    size_t cap = (size_t)(ne_all > 0 ? ne_all : 1);
    int32_t *es = (int32_t *)malloc(sizeof(int32_t) * cap);
    int32_t *ed = (int32_t *)malloc(sizeof(int32_t) * cap);
    int32_t *ev = (int32_t *)malloc(sizeof(int32_t) * cap);
    if (!es || !ed || !ev) { free(es); free(ed); free(ev); fclose(fp); return ORC_ERR_OOM; }
    int rc = ORC_OK;
    long long i;
    int64_t entry = 0;
    for (i = 0; i < ne_all; i++, entry++) {                                                   /* :69-96 */
        int s_, d_;
        if (fscanf(fp, "%d %d", &s_, &d_) != 2) { rc = ORC_ERR_PARSE; break; }
        s_--; d_--;
        if (s_ < 0 || s_ >= nv || d_ < 0 || d_ >= nv) { rc = ORC_ERR_RANGE; break; }
        int val;
        if (nflag == 0) val = (int)orc_pattern_weight(seed, (uint64_t)entry);
        else if (nflag == 1) {
            float f;
            if (fscanf(fp, " %f ", &f) != 1) { rc = ORC_ERR_PARSE; break; }
            val = (int)f;
        } else {
            float f1, f2;
            if (fscanf(fp, " %f %f ", &f1, &f2) != 2) { rc = ORC_ERR_PARSE; break; }
            val = (int)f1;
        }
        es[i] = s_; ed[i] = d_; ev[i] = val;
        if (sflag == 1) {
            i++;
            es[i] = d_; ed[i] = s_; ev[i] = val;
        }
    }
    fclose(fp);
    if (rc == ORC_OK) rc = loader_finish(nv, ne_all, es, ed, ev, source, flags, out);
    free(es); free(ed); free(ev);
    return rc;
}

int orc_from_entries(int32_t nv_decl, int64_t nentries, const int32_t *src, const int32_t *dst, const int32_t *val,
                     int32_t source, uint32_t flags, orc_csr *out)
{
    memset(out, 0, sizeof(*out));
    if (nv_decl < 0 || nentries < 0) return ORC_ERR_PARSE;
    if (source < 0 || source >= nv_decl) return ORC_ERR_RANGE;
    const int sym = (flags & ORC_LOAD_SYM) ? 1 : 0;
    int64_t m0 = nentries * (sym + 1);
    size_t cap = (size_t)(m0 > 0 ? m0 : 1);
    int32_t *es = (int32_t *)malloc(sizeof(int32_t) * cap);
    int32_t *ed = (int32_t *)malloc(sizeof(int32_t) * cap);
    int32_t *ev = (int32_t *)malloc(sizeof(int32_t) * cap);
    if (!es || !ed || !ev) { free(es); free(ed); free(ev); return ORC_ERR_OOM; }
    int64_t o = 0;
    for (int64_t i = 0; i < nentries; i++) {
        if (src[i] < 0 || src[i] >= nv_decl || dst[i] < 0 || dst[i] >= nv_decl) {
            free(es); free(ed); free(ev);
            return ORC_ERR_RANGE;
        }
        es[o] = src[i]; ed[o] = dst[i]; ev[o] = val ? val[i] : 1; o++;
        if (sym) { es[o] = dst[i]; ed[o] = src[i]; ev[o] = val ? val[i] : 1; o++; }
    }
    int rc = loader_finish(nv_decl, m0, es, ed, ev, source, flags, out);
    free(es); free(ed); free(ev);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* R-MAT generator (Chakrabarti, Zhan, Faloutsos, SDM 2004)                  */
/* ------------------------------------------------------------------------ */
static uint64_t orc_splitmix(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int orc_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed, int32_t wmin,
                 int32_t wmax, orc_csr *out)
{
    memset(out, 0, sizeof(*out));
    if (scale < 1 || scale > 30 || edge_factor < 1 || wmin > wmax) return ORC_ERR_PARSE;
    const int64_t ndraw = (int64_t)edge_factor << scale;
    if (ndraw > 2147483647LL / 2) return ORC_ERR_RANGE;
    const uint64_t ta = (uint64_t)(a * 4294967296.0), tb = (uint64_t)((a + b) * 4294967296.0),
                   tc = (uint64_t)((a + b + c) * 4294967296.0);
    int32_t *es = (int32_t *)malloc(sizeof(int32_t) * (size_t)ndraw);
    int32_t *ed = (int32_t *)malloc(sizeof(int32_t) * (size_t)ndraw);
    int32_t *ev = (int32_t *)malloc(sizeof(int32_t) * (size_t)ndraw);
    if (!es || !ed || !ev) { free(es); free(ed); free(ev); return ORC_ERR_OOM; }
    int64_t n = 0;
    for (int64_t i = 0; i < ndraw; i++) {
        /* draw i: its own splitmix64 stream; two quadrant choices per 64-bit
         * draw (low half for even levels, high half for odd ones) */
        uint64_t st = seed * 0xD1B54A32D192ED03ull + (uint64_t)i, r = 0;
        uint32_t s_ = 0, d_ = 0;
        for (int l = 0; l < scale; l++) {
            if ((l & 1) == 0) r = orc_splitmix(&st);
            uint64_t x = (l & 1) ? (r >> 32) : (r & 0xffffffffull);
            uint32_t sb = x >= tb, db = (x >= ta && x < tb) || x >= tc;
            s_ = (s_ << 1) | sb; d_ = (d_ << 1) | db;
        }
        if (s_ == d_) continue;   /* self-loops removed */
        uint64_t wr = orc_splitmix(&st);
        es[n] = (int32_t)s_; ed[n] = (int32_t)d_;
        ev[n] = wmin + (int32_t)(wr % (uint64_t)(wmax - wmin + 1));
        n++;
    }
    int rc = orc_from_entries((int32_t)(1u << scale), n, es, ed, ev, 0, ORC_LOAD_SYM, out);
    free(es); free(ed); free(ev);
    return rc;
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

/* ------------------------------------------------------------------------ */
/* Central finite differences of the weighted-PageRank loss (FP64)           */
/* ------------------------------------------------------------------------ */
/* For each listed CSR entry e = (u0 -> v0) and s = +1, -1 the weight w_e
 * becomes w_e + s*eps; only row u0 of P changes (P'_u0k = w'_u0k / S'_u0).
 * The perturbed fixed point is x* + D with
 *     D = d P'^T D + d dangling(D)/n + d (P' - P)^T x*,
 * iterated from D = 0 (Jacobi) for all 2k perturbations at once (vertex-major
 * D[v][j], a pull over in-edges split across host threads), until every
 * column's L1 change is <= rtol times its L1 norm.  Then
 *     fd_e = (g.D(+) - g.D(-)) / (2 eps),
 * which is (L(w + eps) - L(w - eps)) / (2 eps) with both losses taken from
 * complete FP64 solves around the converged x* (x must be orc_wpr_f64's
 * result at a tolerance near FP64 resolution). */
#include <pthread.h>

typedef struct {
    int32_t nv, K;
    const int64_t *toff;       /* in-edges of v: [toff[v], toff[v+1]) */
    const int32_t *tsrc;
    const double *tP;          /* P_uv of each in-edge */
    const double *D;           /* [nv][K] current */
    double *ND;                /* [nv][K] next */
    const double *dang;        /* [K] d * dangling(D) / n */
    double d;
    int32_t v0, v1;
    double *resid, *norm;      /* [K] per-thread partials */
} fd_job;

static void *fd_pull(void *arg)
{
    fd_job *j = (fd_job *)arg;
    const int K = j->K;
    double *acc = (double *)malloc(sizeof(double) * (size_t)K);
    for (int r = 0; r < K; r++) { j->resid[r] = 0.0; j->norm[r] = 0.0; }
    for (int32_t v = j->v0; v < j->v1; v++) {
        for (int r = 0; r < K; r++) acc[r] = 0.0;
        for (int64_t p = j->toff[v]; p < j->toff[v + 1]; p++) {
            const double P = j->tP[p];
            const double *Du = j->D + (size_t)j->tsrc[p] * K;
            for (int r = 0; r < K; r++) acc[r] += P * Du[r];
        }
        double *out = j->ND + (size_t)v * K;
        for (int r = 0; r < K; r++) out[r] = j->d * acc[r] + j->dang[r];
    }
    free(acc);
    return NULL;
}

static void *fd_resid(void *arg)
{
    fd_job *j = (fd_job *)arg;
    const int K = j->K;
    for (int r = 0; r < K; r++) { j->resid[r] = 0.0; j->norm[r] = 0.0; }
    for (int32_t v = j->v0; v < j->v1; v++) {
        const double *a = j->ND + (size_t)v * K, *b = j->D + (size_t)v * K;
        for (int r = 0; r < K; r++) { j->resid[r] += fabs(a[r] - b[r]); j->norm[r] += fabs(a[r]); }
    }
    return NULL;
}

static void fd_run(fd_job *jobs, int nt, void *(*fn)(void *))
{
    pthread_t th[256];
    for (int t = 1; t < nt; t++)
        if (pthread_create(&th[t], NULL, fn, &jobs[t]) != 0) { fn(&jobs[t]); th[t] = 0; }
    fn(&jobs[0]);
    for (int t = 1; t < nt; t++)
        if (th[t]) pthread_join(th[t], NULL);
}

int orc_wpr_fd_f64(const orc_csr *g, const double *w, const double *x, const double *gv, double d,
                   const int32_t *entries, int32_t k, double eps, double rtol, int32_t max_iter, int32_t nthreads,
                   double *fd_out)
{
    const int32_t nv = g->nv, ne = g->ne;
    const int K = 2 * k;
    if (nv <= 0 || k <= 0) return 0;
    int nt = nthreads > 0 ? nthreads : 1;
    if (nt > 256) nt = 256;
    double *S = (double *)calloc((size_t)nv, sizeof(double));
    int32_t *owner = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ne > 0 ? ne : 1));
    int64_t *toff = (int64_t *)calloc((size_t)nv + 1, sizeof(int64_t));
    int32_t *tsrc = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ne > 0 ? ne : 1));
    double *tP = (double *)malloc(sizeof(double) * (size_t)(ne > 0 ? ne : 1));
    double *D = (double *)calloc((size_t)nv * K, sizeof(double));
    double *ND = (double *)calloc((size_t)nv * K, sizeof(double));
    double *dang = (double *)calloc((size_t)K, sizeof(double));
    double *part = (double *)calloc((size_t)nt * 2 * K, sizeof(double));
    fd_job *jobs = (fd_job *)calloc((size_t)nt, sizeof(fd_job));
    int it = 0;
    if (!S || !owner || !toff || !tsrc || !tP || !D || !ND || !dang || !part || !jobs) { it = -1; goto out; }
    for (int32_t u = 0; u < nv; u++)
        for (int32_t p = g->csc_v[u]; p < g->csc_v[u + 1]; p++) { S[u] += w[p]; owner[p] = u; }
    for (int32_t p = 0; p < ne; p++) toff[g->csc_e[p] + 1]++;
    for (int32_t v = 0; v < nv; v++) toff[v + 1] += toff[v];
    {
        int64_t *pos = (int64_t *)malloc(sizeof(int64_t) * (size_t)nv);
        if (!pos) { it = -1; goto out; }
        memcpy(pos, toff, sizeof(int64_t) * (size_t)nv);
        for (int32_t p = 0; p < ne; p++) {
            int32_t u = owner[p];
            int64_t q = pos[g->csc_e[p]]++;
            tsrc[q] = u;
            tP[q] = S[u] != 0.0 ? w[p] / S[u] : 0.0;
        }
        free(pos);
    }
    /* rows split by in-edge count */
    {
        int64_t per = (toff[nv] + nv) / nt + 1, acc = 0;
        int32_t v = 0;
        for (int t = 0; t < nt; t++) {
            jobs[t].v0 = v;
            int64_t goal = (int64_t)(t + 1) * per;
            while (v < nv && (t == nt - 1 || acc < goal)) { acc += toff[v + 1] - toff[v] + 1; v++; }
            jobs[t].v1 = v;
            jobs[t].nv = nv; jobs[t].K = K; jobs[t].toff = toff; jobs[t].tsrc = tsrc; jobs[t].tP = tP;
            jobs[t].dang = dang; jobs[t].d = d;
            jobs[t].resid = part + (size_t)t * 2 * K; jobs[t].norm = part + (size_t)t * 2 * K + K;
        }
    }
    for (;;) {
        it++;
        for (int r = 0; r < K; r++) dang[r] = 0.0;
        for (int32_t u = 0; u < nv; u++)
            if (S[u] == 0.0)
                for (int r = 0; r < K; r++) dang[r] += D[(size_t)u * K + r];
        for (int r = 0; r < K; r++) dang[r] *= d / nv;
        for (int t = 0; t < nt; t++) { jobs[t].D = D; jobs[t].ND = ND; }
        fd_run(jobs, nt, fd_pull);
        /* row u0 of each perturbation: ND[v][r] += d (P'_u0v - P_u0v) (x_u0 + D_u0) */
        for (int32_t j = 0; j < k; j++) {
            const int32_t e0 = entries[j], u0 = owner[e0];
            for (int sgn = 0; sgn < 2; sgn++) {
                const int r = 2 * j + sgn;
                const double de = sgn == 0 ? eps : -eps;
                const double S1 = S[u0] + de;
                const double xu = x[u0] + D[(size_t)u0 * K + r];
                for (int32_t p = g->csc_v[u0]; p < g->csc_v[u0 + 1]; p++) {
                    const double w1 = w[p] + (p == e0 ? de : 0.0);
                    const double dP = (S1 != 0.0 ? w1 / S1 : 0.0) - (S[u0] != 0.0 ? w[p] / S[u0] : 0.0);
                    ND[(size_t)g->csc_e[p] * K + r] += d * dP * xu;
                }
            }
        }
        fd_run(jobs, nt, fd_resid);
        int done = 1;
        for (int r = 0; r < K; r++) {
            double R = 0.0, N = 0.0;
            for (int t = 0; t < nt; t++) { R += jobs[t].resid[r]; N += jobs[t].norm[r]; }
            if (R > rtol * N) done = 0;
        }
        double *tmp = D; D = ND; ND = tmp;
        if (done || (max_iter > 0 && it >= max_iter)) break;
    }
    for (int32_t j = 0; j < k; j++) {
        double lp = 0.0, lm = 0.0;
        for (int32_t v = 0; v < nv; v++) {
            lp += gv[v] * D[(size_t)v * K + 2 * j];
            lm += gv[v] * D[(size_t)v * K + 2 * j + 1];
        }
        fd_out[j] = (lp - lm) / (2.0 * eps);
    }
out:
    free(S); free(owner); free(toff); free(tsrc); free(tP); free(D); free(ND); free(dang); free(part); free(jobs);
    return it;
}
