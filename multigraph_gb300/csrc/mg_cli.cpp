// mg_cli.cpp -- the reference's command line, unchanged:
//
//     ./BFS file.mtx source iters      (also SSSP, BC, CC, DATA_DRIVEN_PR,
//                                       TOPOLOGY_DRIVEN_PR; main.cu:18-159)
//
// The algorithm comes from the program name (symlinks to `mg`), or from the
// first argument when called as `mg ALG file.mtx source iters`.  Output
// lines keep the reference's format:
//     processing : <ms> ms,<MTEPS> MTEPS,validation : PASS
// with MTEPS = directed edges / us (2x for BC, main.cu:76), ms = mean of the
// `iters` timed runs (device time of each run, load and reset excluded,
// main.cu:37-43).  The reference's binary names are kept with their
// install.sh meaning: DATA_DRIVEN_PR runs the PR_T recurrence and
// TOPOLOGY_DRIVEN_PR the PR_D recurrence (install.sh:23-24).
//
// The trailing "validation" check (the reference's -DVALIDATE verifyResults,
// validate.cu:6) is a small sequential CPU recomputation in this file; set
// MG_VALIDATE=0 to skip it.  Environment options: MG_EXEC=host|graph,
// MG_DIRECTION=auto|push|pull, MG_WEIGHT_SEED (pattern-file weights),
// MG_TUNE_CACHE=<file> (use the autotuner), MG_JSON=1 (extra JSON line),
// MG_CSR_SAVE=<file.mgcsr> (write the loaded CSR as a binary cache).  A
// `.mgcsr` input file is read with mg_load_csr instead of the MTX parser.

#include "mg.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

namespace {

enum Alg { BFS, SSSP, BC, CC, PR_T, PR_D, NONE };

Alg alg_of(const std::string &n)
{
    if (n == "BFS") return BFS;
    if (n == "SSSP") return SSSP;
    if (n == "BC") return BC;
    if (n == "CC") return CC;
    if (n == "DATA_DRIVEN_PR") return PR_T;
    if (n == "TOPOLOGY_DRIVEN_PR") return PR_D;
    return NONE;
}

int die(mg_status s, const char *what)
{
    std::fprintf(stderr, "%s failed: %s (%s)\n", what, mg_status_string(s), mg_last_error());
    return 10 + s;
}

const char *env(const char *k, const char *def)
{
    const char *v = std::getenv(k);
    return v ? v : def;
}

// --- CPU checks (the reference's verifyResults semantics) -----------------
bool check_bfs(const mg_csr_view &g, int src, const std::vector<int32_t> &lv)
{
    std::vector<int32_t> c(g.nv, 0x64646464);
    std::deque<int32_t> q{src};
    c[src] = 0;
    while (!q.empty()) {
        int u = q.front(); q.pop_front();
        for (int p = g.csc_v[u]; p < g.csc_v[u + 1]; p++)
            if (c[g.csc_e[p]] == 0x64646464) { c[g.csc_e[p]] = c[u] + 1; q.push_back(g.csc_e[p]); }
    }
    return c == lv;
}

bool check_sssp(const mg_csr_view &g, int src, const std::vector<int32_t> &d)
{
    std::vector<int32_t> c(g.nv, 0x64646464);
    c[src] = 0;
    for (bool ch = true; ch;) {
        ch = false;
        for (int u = 0; u < g.nv; u++)
            for (int p = g.csc_v[u]; p < g.csc_v[u + 1]; p++)
                if (c[u] + g.csc_ev[p] < c[g.csc_e[p]]) { c[g.csc_e[p]] = c[u] + g.csc_ev[p]; ch = true; }
    }
    return c == d;
}

bool check_cc(const mg_csr_view &g, const std::vector<int32_t> &lab)
{
    std::vector<int32_t> c(g.nv);
    for (int i = 0; i < g.nv; i++) c[i] = i;
    for (bool ch = true; ch;) {
        ch = false;
        for (int u = 0; u < g.nv; u++)
            for (int p = g.csc_v[u]; p < g.csc_v[u + 1]; p++) {
                int v = g.csc_e[p], m = std::min(c[u], c[v]);
                if (c[u] != m || c[v] != m) { c[u] = c[v] = m; ch = true; }
            }
    }
    return c == lab;  // both are minimum-id labels
}

bool check_pr(const mg_csr_view &g, int mode, const std::vector<float> &pr)
{
    std::vector<float> x(g.nv, 0.0f), nx(g.nv);
    std::vector<int> mark(g.nv, 1);
    for (int it = 0; it < 100000; it++) {
        bool flag = false;
        std::fill(nx.begin(), nx.end(), 0.0f);
        for (int u = 0; u < g.nv; u++) {
            int deg = g.csc_v[u + 1] - g.csc_v[u];
            for (int p = g.csc_v[u]; p < g.csc_v[u + 1]; p++) nx[g.csc_e[p]] += x[u] / (float)deg;
        }
        for (int v = 0; v < g.nv; v++) {
            float f1 = 0.15f + nx[v] * 0.85f, f2 = x[v];
            if (mode == 0) { if (std::fabs(f1 - f2) > 0.01f) { x[v] = f1; flag = true; } }
            else {
                if (mark[v] && std::fabs(f1 - f2) > 0.01f * f2) flag = true;
                else mark[v] = 0;
                x[v] = f1;
            }
        }
        if (!flag) break;
    }
    for (int v = 0; v < g.nv; v++) {
        float t = std::max(pr[v], x[v]);
        if (t > 0 && std::fabs(pr[v] - x[v]) / t > 0.05f) return false;  // validate.cu:93-100 (THR)
    }
    return true;
}

bool check_bc_levels(const mg_csr_view &g, int src, const std::vector<int32_t> &lv) { return check_bfs(g, src, lv); }

}  // namespace

int main(int argc, char **argv)
{
    std::string prog = argv[0];
    size_t sl = prog.find_last_of('/');
    if (sl != std::string::npos) prog = prog.substr(sl + 1);
    int a0 = 1;
    Alg alg = alg_of(prog);
    if (alg == NONE && argc > 1) { alg = alg_of(argv[1]); a0 = 2; }
    if (alg == NONE || argc - a0 < 3) {
        std::fprintf(stderr, "usage: BFS|SSSP|BC|CC|DATA_DRIVEN_PR|TOPOLOGY_DRIVEN_PR file.mtx source iters\n");
        return 2;
    }
    const char *file = argv[a0];
    int source = std::atoi(argv[a0 + 1]);
    int iters = std::max(1, std::atoi(argv[a0 + 2]));
    uint32_t flags = MG_LOAD_SYM | (alg == CC ? MG_LOAD_CC : 0u);
    uint64_t seed = std::strtoull(env("MG_WEIGHT_SEED", "1"), nullptr, 10);
    if (alg == CC || alg == PR_T || alg == PR_D) source = 0;  // main.cu:579,614 use source 0

    // a binary CSR cache (mg_save_csr) loads without parsing; its source
    // argument is already a loader (compacted) vertex id
    const std::string fname(file);
    const bool binary = fname.size() > 6 && fname.compare(fname.size() - 6, 6, ".mgcsr") == 0;
    mg_host_graph *hg = nullptr;
    mg_status s = binary ? mg_load_csr(file, &hg) : mg_load_mtx(file, source, flags, seed, 0, &hg);
    if (s != MG_OK) return die(s, "load");
    if (!binary && std::getenv("MG_CSR_SAVE")) {
        s = mg_save_csr(hg, std::getenv("MG_CSR_SAVE"));
        if (s != MG_OK) return die(s, "save");
    }
    mg_csr_view view;
    mg_host_graph_view(hg, &view);
    if (binary && alg != CC && alg != PR_T && alg != PR_D) {
        if (source < 0 || source >= view.nv) return die(MG_ERR_RANGE, "source");
        view.start_p = source;
    }
    mg_graph *dg = nullptr;
    s = mg_graph_upload(hg, 0, &dg);
    if (s != MG_OK) return die(s, "upload");

    mg_opts o;
    mg_opts_default(&o);
    if (std::string(env("MG_EXEC", "graph")) == "host") o.exec = MG_EXEC_HOST;
    std::string dir = env("MG_DIRECTION", "auto");
    if (dir == "push") o.direction = MG_DIR_PUSH;
    if (dir == "pull") o.direction = MG_DIR_PULL;
    const char *cache = std::getenv("MG_TUNE_CACHE");
    int src = view.start_p;
    if (cache && (alg == BFS || alg == SSSP || alg == BC)) {
        s = mg_autotune(dg, alg == BFS ? MG_ALGO_BFS : alg == SSSP ? MG_ALGO_SSSP : MG_ALGO_BC, src, cache, &o);
        if (s != MG_OK) return die(s, "autotune");
    }
    const int n = view.nv;
    std::vector<int32_t> iout(n);
    std::vector<float> fout(n);
    std::vector<double> sig(n);
    double total_ms = 0.0;
    mg_run_info info;
    for (int it = 0; it < iters + 1; it++) {  // first run warms the CUDA graph, not timed
        switch (alg) {
        case BFS: s = mg_bfs(dg, src, &o, iout.data(), &info); break;
        case SSSP: s = mg_sssp(dg, src, &o, iout.data(), &info); break;
        case BC: s = mg_bc(dg, src, &o, iout.data(), sig.data(), fout.data(), &info); break;
        case CC: s = mg_cc(dg, &o, iout.data(), &info); break;
        case PR_T: s = mg_pagerank(dg, MG_PR_TOPOLOGY_REF, &o, fout.data(), &info); break;
        case PR_D: s = mg_pagerank(dg, MG_PR_DATA_REF, &o, fout.data(), &info); break;
        default: break;
        }
        if (s != MG_OK) return die(s, "run");
        if (it > 0) total_ms += info.device_ms;
    }
    double ms = total_ms / iters;
    double mteps = (double)view.ne * (alg == BC ? 2 : 1) / (ms * 1000.0);
    std::printf("processing : %f ms,%f MTEPS,", ms, mteps);
    std::fflush(stdout);
    if (std::string(env("MG_VALIDATE", "1")) != "0") {
        bool ok = false;
        switch (alg) {
        case BFS: ok = check_bfs(view, src, iout); break;
        case SSSP: ok = check_sssp(view, src, iout); break;
        case BC: ok = check_bc_levels(view, src, iout); break;
        case CC: ok = check_cc(view, iout); break;
        case PR_T: ok = check_pr(view, 0, fout); break;
        case PR_D: ok = check_pr(view, 1, fout); break;
        default: break;
        }
        std::printf("validation : %s\n", ok ? "PASS" : "FAIL");
    } else {
        std::printf("\n");
    }
    if (std::string(env("MG_JSON", "0")) == "1")
        std::printf("{\"alg\": \"%s\", \"nv\": %d, \"ne\": %d, \"ms\": %.6f, \"mteps\": %.3f, \"iterations\": %d, "
                    "\"pull_iterations\": %d}\n",
                    prog.c_str(), view.nv, view.ne, ms, mteps, info.iterations, info.pull_iterations);
    mg_graph_free(dg);
    mg_host_graph_free(hg);
    return 0;
}
