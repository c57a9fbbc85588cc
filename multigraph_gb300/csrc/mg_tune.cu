// mg_tune.cu -- autotuner for the sparse/dense (push/pull) switch and the
// pull layout's chunk sizes.
//
// The reference decides between its sparse and dense paths with a runtime
// sampler that times a pseudo iteration of each (process.cu:1115-1246,
// pseudo_phase1/11/2 and pseudo_process_f1 with real side effects) and with
// compile-time constants (common.h:10-52: DENSE_THRESHOLD, sampling factors,
// partition sizes).  Here the switch rule is fixed (Beamer's frontier-edges
// vs unvisited-edges test for BFS/BC, frontier-edges vs m for SSSP) and its
// two thresholds are tuned per graph; for PageRank the tuner picks the
// heavy-row threshold, the chunk size and the thread-bin cutoff of the pull
// layout (re-binned on the device graph).  Every candidate runs the real algorithm in a CUDA
// graph, the median of three timed runs decides, and the winner is cached
// in a text file keyed by a graph signature (n, m and a log2 degree
// histogram).  Cache lines: signature, algorithm, then alpha / beta /
// direction, or heavy threshold / chunk edges / thread-bin cutoff for
// PageRank, the winner's time, and for PageRank the layout that
// MG_PR_LAYOUT_AUTO takes on the graph (gather or segmented, whichever ran
// faster once the gather layout's bins were tuned).

#include "mg_device.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

uint64_t graph_signature(mg_graph *g)
{
    std::vector<int32_t> row(g->nv + 1);
    cudaMemcpy(row.data(), g->row.p, (size_t)(g->nv + 1) * 4, cudaMemcpyDeviceToHost);
    uint64_t hist[33] = {0};
    for (int32_t v = 0; v < g->nv; v++) {
        int32_t d = row[v + 1] - row[v];
        int b = 0;
        while (d > 0) { b++; d >>= 1; }
        hist[b]++;
    }
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t x) { h = (h ^ x) * 1099511628211ull; };
    mix((uint64_t)g->nv);
    mix((uint64_t)g->ne);
    for (uint64_t x : hist) mix(x);
    return h;
}

bool cache_lookup(const char *path, uint64_t sig, int algo, mg_opts *o)
{
    if (!path) return false;
    FILE *f = std::fopen(path, "r");
    if (!f) return false;
    char line[256];
    bool found = false;
    while (std::fgets(line, sizeof(line), f)) {
        unsigned long long s;
        int a, alpha, beta, dir, lay = -1;
        double ms;
        const int k = std::sscanf(line, "%llx %d %d %d %d %lf %d", &s, &a, &alpha, &beta, &dir, &ms, &lay);
        if (k >= 5 && s == sig && a == algo) {
            o->alpha = alpha;
            o->beta = beta;
            o->direction = dir;
            if (algo == MG_ALGO_PR && k == 7) o->pr_layout = lay;   // the layout MG_PR_LAYOUT_AUTO takes
            found = true;  // the last entry wins
        }
    }
    std::fclose(f);
    return found;
}

void cache_store(const char *path, uint64_t sig, int algo, const mg_opts &o, double ms)
{
    if (!path) return;
    FILE *f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%llx %d %d %d %d %.4f %d\n", (unsigned long long)sig, algo, o.alpha, o.beta, o.direction, ms,
                 o.pr_layout);
    std::fclose(f);
}

// median device time of four PageRank runs after a warm-up run
static mg_status pr_median_ms(mg_graph *g, const mg_opts &o, double *ms)
{
    std::vector<double> t;
    for (int rep = 0; rep < 4; rep++) {
        mg_run_info info;
        MG_TRY(mg_pagerank(g, MG_PR_TOPOLOGY, &o, nullptr, &info));
        if (rep > 0) t.push_back(info.device_ms);  // first run warms the graph
    }
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return MG_OK;
}

// PageRank: heavy-row threshold x chunk size x thread-bin cutoff of the
// gather layout's degree bins (timed with that layout), then whether the
// segmented layout beats the tuned gather layout on this graph (the choice
// of MG_PR_LAYOUT_AUTO); for the segmented layout also the split of the
// sweep's work among the CTAs (mgi::hub_rebalance)
mg_status tune_pr_layout(mg_graph *g, const char *cache_path, uint64_t sig, const mg_opts &base)
{
    mg_opts cached = base;
    cached.pr_layout = -1;   // set by a cache line that records the layout
    if (cache_lookup(cache_path, sig, MG_ALGO_PR, &cached)) {
        if (cached.pr_layout == MG_PR_LAYOUT_GATHER || cached.pr_layout == MG_PR_LAYOUT_SEGMENTED)
            g->pr_prefer_gather = cached.pr_layout == MG_PR_LAYOUT_GATHER;
        return mgi::rebin(g, cached.alpha, cached.beta, cached.direction);
    }
    struct Cand { int heavy, chunk, tbin; };
    std::vector<Cand> cands;
    const int hc[][2] = {{256, 1024}, {256, 2048}, {512, 1024}, {512, 2048}, {512, 4096}, {1024, 2048},
                         {1024, 4096}, {1024, 8192}, {2048, 4096}, {2048, 8192}};
    for (int tb : {8, 16, 32})
        for (const auto &p : hc) cands.push_back({p[0], p[1], tb});
    double best_ms = 1e30;
    Cand best = {512, 2048, 32};
    for (const Cand &c : cands) {
        MG_TRY(mgi::rebin(g, c.heavy, c.chunk, c.tbin));
        mg_opts o = base;
        o.exec = MG_EXEC_GRAPH;
        o.profile = 0;
        o.pr_layout = MG_PR_LAYOUT_GATHER;
        double med = 0.0;
        MG_TRY(pr_median_ms(g, o, &med));
        if (med < best_ms) { best_ms = med; best = c; }
    }
    MG_TRY(mgi::rebin(g, best.heavy, best.chunk, best.tbin));
    {
        mg_opts o = base;
        o.exec = MG_EXEC_GRAPH;
        o.profile = 0;
        o.pr_layout = MG_PR_LAYOUT_SEGMENTED;
        double seg_ms = 0.0;
        MG_TRY(pr_median_ms(g, o, &seg_ms));
        // the segmented sweep's split among the CTAs, re-cut three times
        // from measured per-CTA times; kept only if the runs got faster
        std::vector<double> w0;
        if (mgi::hub_weights(g, &w0, nullptr)) {
            for (int it = 0; it < 3; it++) {
                MG_TRY(mg_pagerank(g, MG_PR_TOPOLOGY, &o, nullptr, nullptr));
                MG_TRY(mgi::hub_rebalance(g));
            }
            double reb_ms = 0.0;
            MG_TRY(pr_median_ms(g, o, &reb_ms));
            if (reb_ms < seg_ms) seg_ms = reb_ms;
            else mgi::hub_weights(g, nullptr, &w0);
        }
        g->pr_prefer_gather = seg_ms > best_ms;
    }
    mg_opts rec = base;
    rec.alpha = best.heavy;
    rec.beta = best.chunk;
    rec.direction = best.tbin;
    rec.pr_layout = g->pr_prefer_gather ? MG_PR_LAYOUT_GATHER : MG_PR_LAYOUT_SEGMENTED;
    cache_store(cache_path, sig, MG_ALGO_PR, rec, best_ms);
    return MG_OK;
}

}  // namespace

extern "C" mg_status mg_autotune(mg_graph *g, int32_t algo, int32_t source, const char *cache_path, mg_opts *tuned)
{
    mgi::clear_error();
    if (!g || !tuned) return mgi::fail(MG_ERR_INVALID, "null argument");
    if (algo != MG_ALGO_BFS && algo != MG_ALGO_SSSP && algo != MG_ALGO_BC && algo != MG_ALGO_PR)
        return mgi::fail(MG_ERR_UNSUPPORTED, "nothing to tune for algorithm %d", algo);
    if (algo != MG_ALGO_PR && (source < 0 || source >= g->nv)) return mgi::fail(MG_ERR_RANGE, "source out of range");
    MG_CUDA(cudaSetDevice(g->device));
    mg_opts base = *tuned;
    uint64_t sig = graph_signature(g);
    if (algo == MG_ALGO_PR) return tune_pr_layout(g, cache_path, sig, base);
    if (cache_lookup(cache_path, sig, algo, tuned)) return MG_OK;

    struct Cand { int alpha, beta, dir; };
    std::vector<Cand> cands;
    if (algo == MG_ALGO_SSSP) {
        for (int a : {1, 2, 4, 8, 16, 64}) cands.push_back({a, 18, MG_DIR_AUTO});
        cands.push_back({4, 18, MG_DIR_PUSH});
    } else {
        for (int a : {4, 8, 15, 30, 60})
            for (int b : {6, 18, 54}) cands.push_back({a, b, MG_DIR_AUTO});
        cands.push_back({15, 18, MG_DIR_PUSH});
    }
    double best_ms = 1e30;
    Cand best = cands[0];
    for (const Cand &c : cands) {
        mg_opts o = base;
        o.alpha = c.alpha;
        o.beta = c.beta;
        o.direction = c.dir;
        o.exec = MG_EXEC_GRAPH;
        o.profile = 0;
        std::vector<double> t;
        for (int rep = 0; rep < 4; rep++) {
            mg_run_info info;
            mg_status s;
            if (algo == MG_ALGO_BFS) s = mg_bfs(g, source, &o, nullptr, &info);
            else if (algo == MG_ALGO_SSSP) s = mg_sssp(g, source, &o, nullptr, &info);
            else s = mg_bc(g, source, &o, nullptr, nullptr, nullptr, &info);
            if (s != MG_OK) return s;
            if (rep > 0) t.push_back(info.device_ms);  // first run warms the graph
        }
        std::sort(t.begin(), t.end());
        double med = t[t.size() / 2];
        if (med < best_ms) { best_ms = med; best = c; }
    }
    tuned->alpha = best.alpha;
    tuned->beta = best.beta;
    tuned->direction = best.dir;
    cache_store(cache_path, sig, algo, *tuned, best_ms);
    return MG_OK;
}
