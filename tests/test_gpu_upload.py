"""Re-uploading graphs on the GPU: mg_graph_reload with new weights, with a
new structure of the same size, and the double-buffered mg_graph_stage /
mg_graph_commit pair (runs before the commit still see the old graph)."""
import numpy as np
import pytest

import multigraph_gb300 as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _csr(rp, col, wt):
    return mg.HostGraph.from_csr(rp, col, wt), O.csr_from_arrays(rp, col, wt)


def _permuted(rp, col, wt, seed):
    """Same n and m, vertices renamed (so the row degrees move)."""
    n = len(rp) - 1
    perm = np.random.default_rng(seed).permutation(n).astype(np.int32)
    src = np.repeat(np.arange(n, dtype=np.int32), np.diff(rp))
    s2, d2 = perm[src], perm[col]
    order = np.lexsort((d2, s2))
    rp2 = np.zeros(n + 1, np.int32)
    rp2[1:] = np.cumsum(np.bincount(s2, minlength=n))
    return rp2, d2[order].astype(np.int32), wt[order].astype(np.int32)


def _check_all(g, og, src):
    lv, _ = g.bfs(src)
    assert np.array_equal(lv, O.bfs(og, src))
    dist, _ = g.sssp(src)
    assert np.array_equal(dist, O.sssp(og, src)[0])
    lab, _ = g.cc()
    assert np.array_equal(lab, O.cc_minlabel(og))
    x, info = g.pagerank(mg.PR_TOPOLOGY, tol=1e-6)
    ref, _ = O.pr_norm_f64(og, 0.85, 1e-6, info.iterations)
    assert float(np.max(np.abs(x.astype(np.float64) - ref))) < 1e-6
    # personalised PageRank keeps its own heavy-row table (rows above 256
    # in-edges in chunks): it must follow a re-layout
    seeds = [src, og.nv - 1]
    pp, pinfo = g.ppr_batch(seeds, tol=1e-6)
    for i, s_ in enumerate(seeds):
        pref, _ = O.ppr_f64(og, s_, 0.85, 0.0, pinfo.iterations)
        assert float(np.max(np.abs(pp[i].astype(np.float64) - pref))) < 1e-6, s_


@pytest.mark.parametrize("kind", ["rmat", "lattice"])   # relabeled / not relabeled
def test_reload_new_weights_and_new_structure(kind):
    h0 = mg.HostGraph.rmat(11, 16, seed=31) if kind == "rmat" else mg.HostGraph.lattice(40, 33, 0.05, seed=4)
    rp, col, wt = h0.arrays()
    g = mg.Graph(h0)
    _check_all(g, O.csr_from_arrays(rp, col, wt), 0)
    # same structure, new weights
    wt2 = (np.random.default_rng(1).integers(1, 64, len(wt))).astype(np.int32)
    h1, og1 = _csr(rp, col, wt2)
    g.reload(h1)
    _check_all(g, og1, 0)
    # same n and m, different degrees: laid out again
    h2, og2 = _csr(*_permuted(rp, col, wt2, 2))
    if kind == "rmat":
        assert int(np.max(np.diff(og2.csc_v))) > 256  # heavy personalised-PageRank rows
    g.reload(h2)
    _check_all(g, og2, 3)
    g.free()


def test_stage_overlaps_and_commit_switches():
    h0 = mg.HostGraph.rmat(12, 16, seed=32)
    rp, col, wt = h0.arrays()
    og0 = O.csr_from_arrays(rp, col, wt)
    wt2 = (np.random.default_rng(5).integers(1, 64, len(wt))).astype(np.int32)
    h1, og1 = _csr(rp, col, wt2)
    h1.pin()
    g = mg.Graph(h0)
    g.stage(h1)
    d_old, _ = g.sssp(0)                        # still the uploaded graph
    assert np.array_equal(d_old, O.sssp(og0, 0)[0])
    g.commit()
    d_new, _ = g.sssp(0)
    assert np.array_equal(d_new, O.sssp(og1, 0)[0])
    # a pipeline of alternating inputs
    for k in range(4):
        nxt = h0 if k % 2 == 0 else h1
        g.stage(nxt)
        g.commit()
        d, _ = g.sssp(0)
        assert np.array_equal(d, O.sssp(og0 if k % 2 == 0 else og1, 0)[0]), k
    g.free()


def test_stage_commit_errors():
    h0 = mg.HostGraph.rmat(8, 8, seed=3)
    g = mg.Graph(h0)
    with pytest.raises(mg.MGError) as e:
        g.commit()
    assert e.value.status == mg.MG_ERR_INVALID
    other = mg.HostGraph.rmat(9, 8, seed=3)
    with pytest.raises(mg.MGError) as e:
        g.stage(other)
    assert e.value.status == mg.MG_ERR_INVALID
    g.free()


def test_weighted_runs_between_stage_and_commit():
    """Runs between mg_graph_stage and mg_graph_commit use the current
    graph's caller-order arrays (the staged copy goes to separate buffers)."""
    h0 = mg.HostGraph.rmat(11, 16, seed=33)
    rp, col, wt = h0.arrays()
    og0 = O.csr_from_arrays(rp, col, wt)
    h1, og1 = _csr(*_permuted(rp, col, wt, 7))
    rng = np.random.default_rng(9)
    w0 = rng.uniform(0.05, 1.0, og0.ne).astype(np.float32)
    w1 = rng.uniform(0.05, 1.0, og1.ne).astype(np.float32)
    g = mg.Graph(h0)
    g.stage(h1)
    g.set_float_weights(w0)                     # weights of the current graph
    x0, _ = g.wpagerank(tol=1e-7)
    ref0 = O.wpr_f64(og0, w0.astype(np.float64), 0.85, 1e-13)[0]
    assert float(np.max(np.abs(x0 - ref0))) < 1e-6
    g.commit()
    g.set_float_weights(w1)
    x1, _ = g.wpagerank(tol=1e-7)
    ref1 = O.wpr_f64(og1, w1.astype(np.float64), 0.85, 1e-13)[0]
    assert float(np.max(np.abs(x1 - ref1))) < 1e-6
    # the same structure again: the fast path (relabel only) then weights
    g.stage(h1)
    g.commit()
    g.set_float_weights(w1)
    x2, _ = g.wpagerank(tol=1e-7)
    assert np.array_equal(x1, x2)
    d, _ = g.sssp(5)
    assert np.array_equal(d, O.sssp(og1, 5)[0])
    g.free()


@pytest.mark.parametrize("kind", ["rmat", "lattice"])   # relabeled / not relabeled
@pytest.mark.parametrize("wmax", [64, 1000])
def test_staged_pinned_weights(kind, wmax):
    """A pinned host graph is staged with its int32 weights (row offsets,
    column ids and weights: 4(n+1) + 8m bytes) and relabeled at commit."""
    h0 = mg.HostGraph.rmat(11, 16, seed=34) if kind == "rmat" else mg.HostGraph.lattice(40, 33, 0.05, seed=5)
    rp, col, wt = h0.arrays()
    n, m = len(rp) - 1, len(col)
    src = np.repeat(np.arange(n), np.diff(rp))
    lo, hi = np.minimum(src, col), np.maximum(src, col)
    w = ((lo.astype(np.int64) * 7919 + hi * 104729) % wmax + 1).astype(np.int32)   # symmetric, in [1, wmax]
    h1, og1 = _csr(rp, col, w)
    h1.pin()
    assert h1.stage_bytes() == 4 * (n + 1) + 8 * m
    g = mg.Graph(h0)
    g.stage(h1)
    g.commit()
    for s in (0, 3):
        d, _ = g.sssp(s)
        assert np.array_equal(d, O.sssp(og1, s)[0]), (kind, wmax, s)
    # and back to the first graph (not pinned)
    g.stage(h0)
    g.commit()
    d, _ = g.sssp(0)
    assert np.array_equal(d, O.sssp(O.csr_from_arrays(rp, col, wt), 0)[0])
    g.free()


def _pairs(h):
    rp, col, wt = h.arrays()
    n = len(rp) - 1
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp))
    keep = src < col
    return n, src[keep], col[keep].astype(np.int64), wt[keep].astype(np.int64)


def _sym_csr(n, u, v, w):
    """Symmetric CSR (both directions, one weight per pair)."""
    s = np.concatenate([u, v])
    d = np.concatenate([v, u])
    ww = np.concatenate([w, w])
    order = np.lexsort((d, s))
    rp = np.zeros(n + 1, np.int64)
    rp[1:] = np.cumsum(np.bincount(s, minlength=n))
    return rp.astype(np.int32), d[order].astype(np.int32), ww[order].astype(np.int32)


@pytest.mark.parametrize("direction", [mg.DIR_AUTO, mg.DIR_PULL])
@pytest.mark.parametrize("pin", [False, True])   # int32 / byte-weight staging
def test_commit_lowers_least_weight(direction, pin):
    """New weights on the same structure with a smaller least weight: the
    SSSP pull's settled-row bound must use the new least weight (also in
    loops captured before the commit), and a negative weight must be
    refused after the commit."""
    n, u, v, _ = _pairs(mg.HostGraph.rmat(12, 16, seed=41))
    rng = np.random.default_rng(3)
    h0, og0 = _csr(*_sym_csr(n, u, v, rng.integers(40, 64, len(u))))
    h1, og1 = _csr(*_sym_csr(n, u, v, rng.integers(1, 64, len(u))))
    if pin:
        h1.pin()
    g = mg.Graph(h0)
    for ex in (mg.EXEC_GRAPH, mg.EXEC_HOST):
        d, _ = g.sssp(0, direction=direction, exec=ex)
        assert np.array_equal(d, O.sssp(og0, 0)[0])
    g.stage(h1)
    g.commit()
    for ex in (mg.EXEC_GRAPH, mg.EXEC_HOST):
        for s in (0, 77, n - 1):
            d, _ = g.sssp(s, direction=direction, exec=ex)
            assert np.array_equal(d, O.sssp(og1, s)[0]), (ex, s)
    w2 = rng.integers(1, 64, len(u))
    w2[5] = -3
    h2, _ = _csr(*_sym_csr(n, u, v, w2))
    g.stage(h2)
    g.commit()
    with pytest.raises(mg.MGError) as e:
        g.sssp(0)
    assert e.value.status == mg.MG_ERR_INVALID
    g.free()


def test_commit_new_degrees_same_size_rebuilds_loops():
    """Same n and m, hub edges rewired to low-degree vertices: the commit
    lays the graph out again (the hub leaves the heavy-row chunks), and
    loops captured before it must not replay the old bins."""
    n, u, v, w = _pairs(mg.HostGraph.rmat(12, 16, seed=42))
    deg = np.bincount(np.concatenate([u, v]), minlength=n)
    hub = int(np.argmax(deg))
    at_hub = np.nonzero((u == hub) | (v == hub))[0]
    k = len(at_hub) - 8
    assert deg[hub] > 600 and k > 500
    keep = np.ones(len(u), bool)
    keep[at_hub[:k]] = False
    have = set(zip(u[keep].tolist(), v[keep].tolist()))
    rng = np.random.default_rng(9)
    low = np.nonzero(deg <= 4)[0]
    nu, nv_ = [], []
    while len(nu) < k:
        a, b = sorted(rng.choice(low, 2, replace=False).tolist())
        if (a, b) not in have:
            have.add((a, b))
            nu.append(a)
            nv_.append(b)
    u2 = np.concatenate([u[keep], nu])
    v2 = np.concatenate([v[keep], nv_])
    w2 = np.concatenate([w[keep], rng.integers(1, 64, k)])
    h0, og0 = _csr(*_sym_csr(n, u, v, w))
    h2, og2 = _csr(*_sym_csr(n, u2, v2, w2))
    g = mg.Graph(h0)
    _check_all(g, og0, 0)
    g.stage(h2)
    g.commit()
    _check_all(g, og2, 0)
    _check_all(g, og2, hub)
    (_, sg, dl), _ = g.bc(3)
    _, rsg, rdl = O.bc_f64(og2, 3)
    assert np.array_equal(sg, rsg)
    assert float(np.max(np.abs(dl - rdl) / np.maximum(np.abs(rdl), 1.0))) < 1e-5
    g.free()
