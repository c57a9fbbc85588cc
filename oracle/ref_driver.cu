/*
 * ref_driver.cu -- a small driver of our own around the reference's
 * generate_CSC (read_input.cu:11) and verifyResults (validate.cu:6).
 * oracle/Makefile compiles it together with those two reference files, once
 * per algorithm macro, into oracle/_ref/ref_<ALG>.  Test infrastructure only.
 *
 *   ref_<ALG> load     <file.mtx> <source> <out.bin>
 *       runs the reference loader and writes
 *       int32 nv, ne, start_p, tra, has_ev, csc_v[nv+1], csc_e[ne], [csc_ev[ne]]
 *   ref_<ALG> validate <file.mtx> <source> <result.bin>
 *       loads the graph with the reference loader, reads nv values of the
 *       algorithm's output (V1T; BC also reads sigma int32[nv] and delta
 *       float[nv] after it) in compacted vertex ids and lets the reference's
 *       verifyResults print "validation : PASS" or "validation : FAIL".
 */
#include "user_function.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

void generate_CSC(struct csc_package *, char **);
void verifyResults(struct csc_package *, GRAPHTYPE *, struct OUTPUT *, int);

static int write_all(FILE *f, const void *p, size_t bytes)
{
    return fwrite(p, 1, bytes, f) == bytes ? 0 : 1;
}

int main(int argc, char **argv)
{
    if (argc != 5) {
        fprintf(stderr, "usage: %s load|validate file.mtx source file.bin\n", argv[0]);
        return 2;
    }
    struct csc_package inp;
    memset(&inp, 0, sizeof(inp));
    char *largv[4] = {argv[0], argv[2], argv[3], (char *)"1"};
    generate_CSC(&inp, largv);

    if (strcmp(argv[1], "load") == 0) {
        FILE *f = fopen(argv[4], "wb");
        if (!f) return 3;
        int has_ev = 0;
#ifdef E1
        has_ev = 1;
#endif
        int hdr[5] = {inp.nv, inp.ne, inp.start_p, inp.tra, has_ev};
        int rc = write_all(f, hdr, sizeof(hdr));
        rc |= write_all(f, inp.csc_v, sizeof(int) * (size_t)(inp.nv + 1));
        rc |= write_all(f, inp.csc_e, sizeof(int) * (size_t)inp.ne);
#ifdef E1
        rc |= write_all(f, inp.csc_ev, sizeof(int) * (size_t)inp.ne);
#endif
        fclose(f);
        return rc ? 4 : 0;
    }
    if (strcmp(argv[1], "validate") == 0) {
        int nv = inp.nv;
        FILE *f = fopen(argv[4], "rb");
        if (!f) return 3;
        std::vector<V1T> r((size_t)nv + 1);
        if (fread(r.data(), sizeof(V1T), (size_t)nv, f) != (size_t)nv) { fclose(f); return 5; }
        GRAPHTYPE m;
        memset(&m, 0, sizeof(m));
        m.nv = nv;
        m.ne = inp.ne;
        struct OUTPUT out;
        memset(&out, 0, sizeof(out));
        out.r = r.data();
#ifndef CC
        std::vector<int> itable((size_t)nv + 1);
        for (int i = 0; i <= nv; i++) itable[i] = i;
        m._itable = itable.data();
#endif
#ifdef V2
        std::vector<V2T> r2((size_t)nv + 1, 0);
        out.r2 = r2.data();
#endif
#ifdef V3
        std::vector<V3T> r3((size_t)nv + 1, 0);
        out.r3 = r3.data();
#endif
#ifdef BC
        if (fread(r2.data(), sizeof(V2T), (size_t)nv, f) != (size_t)nv) { fclose(f); return 5; }
        if (fread(r3.data(), sizeof(V3T), (size_t)nv, f) != (size_t)nv) { fclose(f); return 5; }
#endif
        fclose(f);
        fflush(stdout);
        verifyResults(&inp, &m, &out, inp.start_p);
        fflush(stdout);
        return 0;
    }
    fprintf(stderr, "unknown mode %s\n", argv[1]);
    return 2;
}
