"""Failure detection on the GPU without a GPU fault: MG_FAIL_BARRIER makes
the grid barriers of the persistent kernels never complete, so their
bounded waits (about 10 ms under injection) run out.  The run must end with
MG_ERR_CUDA naming the barrier, and the context must stay usable: the same
graph then runs correctly."""
import os

import numpy as np
import pytest

import multigraph_gb300 as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture
def path_graph():
    n = 400
    src = np.arange(n - 1)
    h = mg.HostGraph.from_entries(n, src, src + 1)
    rp, col, wt = h.arrays()
    g = mg.Graph(h)
    yield g, O.csr_from_arrays(rp, col, wt)
    g.free()


def _with_injection(fn):
    os.environ["MG_FAIL_BARRIER"] = "1"
    try:
        with pytest.raises(mg.MGError) as e:
            fn()
    finally:
        del os.environ["MG_FAIL_BARRIER"]
    assert e.value.status == mg.MG_ERR_CUDA
    assert "barrier" in str(e.value)


@pytest.mark.parametrize("exec_mode", [mg.EXEC_GRAPH, mg.EXEC_HOST])
def test_push_barrier_timeout_is_reported_and_recoverable(path_graph, exec_mode):
    g, og = path_graph
    _with_injection(lambda: g.bfs(0, exec=exec_mode))
    lv, _ = g.bfs(0, exec=exec_mode)                      # same graph, no injection
    assert np.array_equal(lv, O.bfs(og, 0))
    _with_injection(lambda: g.sssp(7, exec=exec_mode))
    d, _ = g.sssp(7, exec=exec_mode)
    assert np.array_equal(d, O.sssp(og, 7)[0])


def test_backward_barrier_timeout_is_reported_and_recoverable(path_graph):
    g, og = path_graph
    # a pull-only forward sweep has no barriers, so the backward sweep's fail
    _with_injection(lambda: g.bc(3, direction=mg.DIR_PULL))
    (lv, sg, dl), _ = g.bc(3)
    rlv, rsg, rdl = O.bc_f64(og, 3)
    assert np.array_equal(lv, rlv) and np.array_equal(sg, rsg)
    assert np.allclose(dl, rdl, rtol=1e-5, atol=1e-6)
