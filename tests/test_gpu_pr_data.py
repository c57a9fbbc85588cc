"""Data-driven PageRank (MG_PR_DATA) where its queue sweeps engage.

The graph is a 1024 x 1024 torus (4-regular, so the uniform start vector is
already its fixed point and every torus vertex freezes after the first
sweep) plus a disjoint R-MAT 12 component with its isolated vertices
dropped (no vertex is dangling, so the torus values never move).  After the
first sweep the active vertices' in-edges are about 2 % of m, below m/16,
and every later sweep runs over the queue of active vertices only
(processi.cu:182-407: _process_f1 from the active vertices, process_f3
applying and requeueing).  The result is checked against the FP64 fixed
point of the oracle and against the topology-driven form on the same graph.
"""
import numpy as np
import pytest

import multigraph_gb300 as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def torus_plus_rmat(side: int, scale: int, seed: int):
    """Edge list (0-based, each undirected edge once) of a side x side torus
    followed by an R-MAT component whose isolated vertices are dropped."""
    n_t = side * side
    v = np.arange(n_t, dtype=np.int64)
    r, c = v // side, v % side
    src = [v, v]
    dst = [r * side + (c + 1) % side, ((r + 1) % side) * side + c]
    h = mg.HostGraph.rmat(scale, 16, seed=seed)
    rp, col, _ = h.arrays()
    h.free()
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    keep = np.flatnonzero(np.diff(rp) > 0)
    newid = np.full(len(rp) - 1, -1, np.int64)
    newid[keep] = np.arange(len(keep))
    up = rows < col
    src.append(n_t + newid[rows[up]])
    dst.append(n_t + newid[col[up]])
    return n_t + len(keep), np.concatenate(src).astype(np.int32), np.concatenate(dst).astype(np.int32)


@pytest.fixture(scope="module")
def mixed():
    nv, s, d = torus_plus_rmat(1024, 12, seed=12)
    h = mg.HostGraph.from_entries(nv, s, d)
    rp, col, wt = h.arrays()
    og = O.csr_from_arrays(rp, col, wt)
    g = mg.Graph(h)
    yield g, og
    g.free()
    h.free()


def test_data_driven_queue_sweeps(mixed):
    g, og = mixed
    tol = 1e-8
    exact, _ = O.pr_norm_f64(og, 0.85, 1e-14, 1000)
    xd, info = g.pagerank(mg.PR_DATA, tol=tol)
    xt, tinfo = g.pagerank(mg.PR_TOPOLOGY, tol=tol)
    # one sweep over every row, then the queue: the switch happened
    assert info.pull_iterations <= 4 and info.iterations - info.pull_iterations >= 5, \
        (info.iterations, info.pull_iterations)
    ed = np.abs(xd.astype(np.float64) - exact)
    et = np.abs(xt.astype(np.float64) - exact)
    print(f"data-driven: {info.iterations} sweeps ({info.pull_iterations} over every row), "
          f"max-abs {ed.max():.3e}, L1 {ed.sum():.3e}; topology-driven: {tinfo.iterations} sweeps, "
          f"max-abs {et.max():.3e}, L1 {et.sum():.3e}")
    assert ed.max() < 5e-9 and ed.sum() < 3e-7, (ed.max(), ed.sum())
    assert et.max() < 5e-9 and et.sum() < 3e-7, (et.max(), et.sum())
    # the same answer in host-driven and graph-captured loops
    xh, hinfo = g.pagerank(mg.PR_DATA, tol=tol, exec=mg.EXEC_HOST)
    assert hinfo.iterations == info.iterations and np.array_equal(xh, xd)
