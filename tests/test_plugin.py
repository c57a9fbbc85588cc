"""The pluggable operator surface: an operator defined only in
tests/plugins/widest_path.cu (a relaxed max-min operator, unlike any
built-in one) is compiled against include/mg_ops.cuh + mg_plugin.cuh into
its own library, which runs it on libmg's frontier engine.

CPU: the plugin builds for sm_103a and exports its entry point.
GPU: its labels equal a widest-path oracle (a max-bottleneck Dijkstra on
the host) bit for bit, with the engine forced to push, forced to pull and
switching, as a captured graph loop and as a host loop; a second call on
the same graph after BFS / SSSP runs (shared workspace, separate captured
loops) gives the same labels.
"""
import ctypes as C
import heapq
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import multigraph_gb300 as mg  # noqa: E402
from plugin_build import build_plugin  # noqa: E402


def _lib():
    L = C.CDLL(build_plugin("widest_path"))
    L.mg_widest_path.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
    L.mg_widest_path.restype = C.c_int32
    return L


def test_plugin_builds_and_exports():
    L = _lib()
    assert hasattr(L, "mg_widest_path")


def widest_oracle(rp, col, wt, src):
    """Largest bottleneck weight from src (0 unreachable, INT32_MAX for src)."""
    n = len(rp) - 1
    best = np.zeros(n, np.int64)
    best[src] = 2**31 - 1
    heap = [(-best[src], src)]
    done = np.zeros(n, bool)
    while heap:
        nb, u = heapq.heappop(heap)
        if done[u]:
            continue
        done[u] = True
        bu = -nb
        for p in range(rp[u], rp[u + 1]):
            v = col[p]
            cand = min(bu, int(wt[p]))
            if cand > best[v]:
                best[v] = cand
                heapq.heappush(heap, (-cand, v))
    return best.astype(np.int32)


def _run(L, g, src, **kw):
    o = g._opts(None, kw)
    out = np.empty(g.nv, np.int32)
    info = mg.RunInfo()
    st = L.mg_widest_path(g._h, src, C.byref(o), out.ctypes.data_as(C.c_void_p), C.byref(info))
    if st != mg.MG_OK:
        raise mg.MGError(st, "mg_widest_path", mg.lib.mg_last_error().decode())
    return out, info


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["rmat", "lattice"])
def test_widest_path_operator_matches_oracle(kind):
    L = _lib()
    h = mg.HostGraph.rmat(12, 16, seed=5) if kind == "rmat" else mg.HostGraph.lattice(40, 30, 0.05, seed=2)
    rp, col, wt = h.arrays()
    if kind == "lattice":   # symmetric integer weights 1..64 (one per undirected pair)
        src_ = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
        lo, hi = np.minimum(src_, col), np.maximum(src_, col)
        wt = ((lo.astype(np.int64) * 7919 + hi * 104729) % 64 + 1).astype(np.int32)
        h = mg.HostGraph.from_csr(rp, col, wt)
    g = mg.Graph(h)
    try:
        for s in (0, g.nv // 3, g.nv - 1):
            ref = widest_oracle(rp, col, wt, s)
            for direction in (mg.DIR_AUTO, mg.DIR_PUSH, mg.DIR_PULL):
                for ex in (mg.EXEC_GRAPH, mg.EXEC_HOST):
                    lab, info = _run(L, g, s, direction=direction, exec=ex)
                    assert np.array_equal(lab, ref), (kind, s, direction, ex, int(np.sum(lab != ref)))
        # built-in operators on the same graph in between: their loops and
        # the plugin's are kept apart, the workspace is shared
        g.bfs(0)
        g.sssp(0)
        lab, _ = _run(L, g, 0)
        assert np.array_equal(lab, widest_oracle(rp, col, wt, 0))
        with pytest.raises(mg.MGError) as e:
            _run(L, g, g.nv)
        assert e.value.status == mg.MG_ERR_RANGE
    finally:
        g.free()
