"""Edge cases on the GPU path against the oracle: an empty graph, a single
edge, a self-loop, a long path (thousands of levels through the persistent
push kernel), a star (one heavy row), and out-of-range sources."""
import numpy as np
import pytest

import multigraph_gb300 as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pair(h):
    rp, col, wt = h.arrays()
    return mg.Graph(h), O.csr_from_arrays(rp, col, wt)


def _all(g, og, src):
    lv, _ = g.bfs(src)
    assert np.array_equal(lv, O.bfs(og, src))
    d, _ = g.sssp(src)
    assert np.array_equal(d, O.sssp(og, src)[0])
    lab, _ = g.cc()
    assert np.array_equal(lab, O.cc_minlabel(og))
    (blv, sg, dl), _ = g.bc(src)
    rlv, rsg, rdl = O.bc_f64(og, src)
    assert np.array_equal(blv, rlv) and np.array_equal(sg, rsg)
    assert np.allclose(dl, rdl, rtol=1e-5, atol=1e-6)
    for layout in (mg.PR_LAYOUT_GATHER, mg.PR_LAYOUT_SEGMENTED):
        x, info = g.pagerank(mg.PR_TOPOLOGY, tol=1e-6, pr_layout=layout)
        ref, _ = O.pr_norm_f64(og, 0.85, 1e-6, info.iterations)
        assert float(np.max(np.abs(x.astype(np.float64) - ref))) < 1e-6, layout
    bc, _ = g.bc_multi([src, src])
    assert np.allclose(bc, O.bc_multi_f64(og, [src, src]), rtol=1e-5, atol=1e-5)


def test_single_edge_and_self_loop():
    g, og = _pair(mg.HostGraph.from_entries(2, [0], [1]))
    assert og.nv == 2
    _all(g, og, 0)
    _all(g, og, 1)
    g.free()
    g, og = _pair(mg.HostGraph.from_entries(3, [0, 1], [0, 2]))   # self-loop kept by the loader
    _all(g, og, 0)
    g.free()


def test_long_path_many_levels():
    n = 3000
    src = np.arange(n - 1)
    h = mg.HostGraph.from_entries(n, src, src + 1, (src % 7 + 1).astype(np.int32))
    g, og = _pair(h)
    _all(g, og, 0)
    _all(g, og, n // 2)
    _, info = g.bfs(0)
    assert info.iterations >= n - 1
    g.free()


def test_star_heavy_row():
    n = 20000
    leaves = np.arange(1, n)
    h = mg.HostGraph.from_entries(n, np.zeros(n - 1, np.int32), leaves)
    g, og = _pair(h)
    _all(g, og, 0)
    _all(g, og, 5)
    g.free()


def test_empty_graph_and_bad_sources():
    h = mg.HostGraph.from_entries(4, [], [])
    g = mg.Graph(h)
    assert g.nv == 0 and g.ne == 0
    lab, _ = g.cc()
    assert lab.size == 0
    x, _ = g.pagerank(mg.PR_TOPOLOGY)
    assert x.size == 0
    with pytest.raises(mg.MGError) as e:
        g.bfs(0)
    assert e.value.status == mg.MG_ERR_RANGE
    g.free()
    g, og = _pair(mg.HostGraph.rmat(8, 8, seed=1))
    for bad in (-1, og.nv):
        with pytest.raises(mg.MGError) as e:
            g.sssp(bad)
        assert e.value.status == mg.MG_ERR_RANGE
        with pytest.raises(mg.MGError) as e:
            g.bc_multi([0, bad])
        assert e.value.status == mg.MG_ERR_RANGE
    g.free()


def test_unsupported_and_directed_paths():
    rng = np.random.default_rng(11)
    s = rng.integers(0, 300, 2500)
    d = (s + rng.integers(1, 30, 2500)) % 300
    h = mg.HostGraph.from_entries(300, s, d, rng.integers(1, 64, 2500), flags=mg.LOAD_NSYM)
    g, og = _pair(h)
    # weighted PageRank needs float weights, then a symmetric structure
    with pytest.raises(mg.MGError) as e:
        g.wpagerank()
    assert e.value.status == mg.MG_ERR_UNSUPPORTED
    g.set_float_weights(np.ones(og.ne, np.float32))
    with pytest.raises(mg.MGError) as e:
        g.wpagerank()
    assert e.value.status == mg.MG_ERR_UNSUPPORTED
    # multi-source BC on a directed graph: one traversal per source, equal
    # to the sum of the single-source deltas
    srcs = [0, 5, 5, 120]
    bc, _ = g.bc_multi(srcs)
    acc = np.zeros(og.nv)
    for x in srcs:
        (_, _, dl), _ = g.bc(x)
        dd = dl.astype(np.float64)
        dd[x] = 0.0
        acc += dd
    assert np.allclose(bc, acc, rtol=1e-5, atol=1e-5)
    # BFS / SSSP / CC on the directed graph against the oracle
    lv, _ = g.bfs(5)
    assert np.array_equal(lv, O.bfs(og, 5))
    dist, _ = g.sssp(5)
    assert np.array_equal(dist, O.sssp(og, 5)[0])
    lab, _ = g.cc()
    assert np.array_equal(lab, O.cc_minlabel(og))
    g.free()
