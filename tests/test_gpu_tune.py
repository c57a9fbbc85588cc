"""The autotuner (the reference's sampling heuristic, process.cu:1115-1246,
and its compile-time thresholds, common.h:10-52): tuned switch thresholds
and a tuned PageRank pull layout keep every result equal to the oracle, and
the cache file is reused."""
import os
import tempfile

import numpy as np
import pytest

import multigraph_gb300 as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pair(h):
    rp, col, wt = h.arrays()
    return mg.Graph(h), O.csr_from_arrays(rp, col, wt)


def test_switch_thresholds_and_cache():
    g, og = _pair(mg.HostGraph.rmat(11, 16, seed=41))
    cache = os.path.join(tempfile.mkdtemp(), "tune.txt")
    for algo in (mg.ALGO_BFS, mg.ALGO_SSSP, mg.ALGO_BC):
        o = g.autotune(algo, 0, cache)
        assert o.alpha > 0 and o.beta > 0
        again = g.autotune(algo, 0, cache)             # from the cache file
        assert (again.alpha, again.beta, again.direction) == (o.alpha, o.beta, o.direction)
        lv, _ = g.bfs(0, o)
        assert np.array_equal(lv, O.bfs(og, 0))
        d, _ = g.sssp(0, o)
        assert np.array_equal(d, O.sssp(og, 0)[0])
    assert len(open(cache).read().splitlines()) == 3
    g.free()


def test_pagerank_layout_tuning_keeps_results():
    g, og = _pair(mg.HostGraph.rmat(13, 16, seed=42))
    cache = os.path.join(tempfile.mkdtemp(), "tune.txt")
    g.autotune(mg.ALGO_PR, 0, cache)
    line = open(cache).read().split()
    heavy, chunk, tbin = int(line[2]), int(line[3]), int(line[4])
    assert heavy in (256, 512, 1024, 2048) and chunk in (1024, 2048, 4096, 8192) and tbin in (8, 16, 32)
    x, info = g.pagerank(mg.PR_TOPOLOGY, tol=1e-6)
    ref, _ = O.pr_norm_f64(og, 0.85, 1e-6, info.iterations)
    assert float(np.max(np.abs(x.astype(np.float64) - ref))) < 1e-6
    lv, _ = g.bfs(0)
    assert np.array_equal(lv, O.bfs(og, 0))
    d, _ = g.sssp(0)
    assert np.array_equal(d, O.sssp(og, 0)[0])
    lab, _ = g.cc()
    assert np.array_equal(lab, O.cc_minlabel(og))
    bc, _ = g.bc_multi([0, 5, 9])
    ref_bc = O.bc_multi_f64(og, [0, 5, 9])
    assert float(np.max(np.abs(bc - ref_bc)) / np.max(np.abs(ref_bc))) < 1e-5
    # a second graph with the same signature takes the cached layout
    g2, _ = _pair(mg.HostGraph.rmat(13, 16, seed=42))
    g2.autotune(mg.ALGO_PR, 0, cache)
    assert len(open(cache).read().splitlines()) == 1
    x2, _ = g2.pagerank(mg.PR_TOPOLOGY, tol=1e-6)
    assert np.array_equal(x, x2)
    g.free()
    g2.free()


def test_segmented_pagerank_independent_of_work_split():
    """The segmented sweep's work split among the SMs is re-cut from
    measured times by the autotuner; every piece is summed in edge order by
    one lane wherever it runs, so a tuned graph and an untuned one give the
    same bits (and the gather layout, whose bins the tuner also sets,
    agrees with the oracle)."""
    h = mg.HostGraph.rmat(16, 16, seed=16)
    rp, col, wt = h.arrays()
    og = O.csr_from_arrays(rp, col, wt)
    g1, g2 = mg.Graph(h), mg.Graph(h)
    try:
        x1, i1 = g1.pagerank(mg.PR_TOPOLOGY, tol=1e-6, pr_layout=mg.PR_LAYOUT_SEGMENTED)
        g2.autotune(mg.ALGO_PR, 0)
        for _ in range(2):
            x2, i2 = g2.pagerank(mg.PR_TOPOLOGY, tol=1e-6, pr_layout=mg.PR_LAYOUT_SEGMENTED)
            assert i1.iterations == i2.iterations and np.array_equal(x1, x2)
        ref, _ = O.pr_norm_f64(og, 0.85, 1e-6, i1.iterations)
        assert float(np.max(np.abs(x1.astype(np.float64) - ref))) < 1e-6
        xg, ig = g2.pagerank(mg.PR_TOPOLOGY, tol=1e-6, pr_layout=mg.PR_LAYOUT_GATHER)
        refg, _ = O.pr_norm_f64(og, 0.85, 1e-6, ig.iterations)
        assert float(np.max(np.abs(xg.astype(np.float64) - refg))) < 1e-6
    finally:
        g1.free()
        g2.free()
        h.free()
