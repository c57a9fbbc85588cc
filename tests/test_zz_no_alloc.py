"""mg_pagerank_noalloc: PageRank for callers that cannot allocate device memory.

Such callers (custom allocators and pool callbacks, applications that reserve
all device memory up front, latency-bound loops) hand libmg their own device
buffers; the entry point keeps its intermediates in a fixed device array
inside the library.  The test plays such a caller: it owns the CSR and the
result buffer (allocated here with torch), calls the entry point twice in a
row through the C ABI and checks both results against mg_pagerank
(MG_PR_TOPOLOGY) and against the FP64 oracle, within the PageRank tolerance
used by the parity tests (1e-6 max-abs).  It also checks that the device's
free memory does not move across a call, and that graphs above the size
limit, damping outside (0, 1) and row offsets that do not end at ne are
refused.
"""
import numpy as np
import pytest

import multigraph_gb300 as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_noalloc_matches_pagerank_twice():
    torch = pytest.importorskip("torch")
    h = mg.HostGraph.rmat(14, 16, seed=21)
    rp, col, _ = h.arrays()
    g = mg.Graph(h)
    ref, info = g.pagerank(mg.PR_TOPOLOGY, tol=1e-6)
    g.free()
    exact, _ = O.pr_norm_f64(O.csr_from_arrays(rp, col), 0.85, 1e-6, info.iterations)

    dev = torch.device("cuda", 0)
    d_row = torch.from_numpy(rp).to(dev)
    d_col = torch.from_numpy(col).to(dev)
    d_rank = torch.empty(len(rp) - 1, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize(dev)
    for call in range(2):
        free_before = torch.cuda.mem_get_info(dev)[0]
        d_rank.fill_(-1.0)
        torch.cuda.synchronize(dev)
        iters, resid = mg.pagerank_noalloc(d_row.data_ptr(), d_col.data_ptr(), len(rp) - 1, len(col),
                                           d_rank.data_ptr(), stream, tol=1e-6)
        torch.cuda.synchronize(dev)
        free_after = torch.cuda.mem_get_info(dev)[0]
        x = d_rank.cpu().numpy()
        err = float(np.max(np.abs(x.astype(np.float64) - ref.astype(np.float64))))
        assert err < 1e-6, (call, err)
        assert iters == info.iterations, (call, iters, info.iterations)
        err64 = float(np.max(np.abs(x.astype(np.float64) - exact)))
        assert err64 < 1e-6, (call, err64)
        assert resid <= 1e-6 and iters > 0, (call, iters, resid)
        if call == 1:
            assert free_after == free_before, (free_before, free_after)


def test_noalloc_rejects_too_many_vertices():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.int32, device=dev)
    out = torch.zeros(16, dtype=torch.float32, device=dev)
    with pytest.raises(mg.MGError) as e:
        mg.pagerank_noalloc(buf.data_ptr(), buf.data_ptr(), mg.NOALLOC_MAX_VERTICES + 1, 8, out.data_ptr())
    assert e.value.status == mg.MG_ERR_RANGE


def test_noalloc_rejects_bad_damping_and_offsets():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    rp = torch.tensor([0, 1, 2], dtype=torch.int32, device=dev)   # two vertices, one edge each way
    col = torch.tensor([1, 0], dtype=torch.int32, device=dev)
    out = torch.zeros(2, dtype=torch.float32, device=dev)
    for d in (1.0, 1.5, -0.5, float("nan")):
        with pytest.raises(mg.MGError) as e:
            mg.pagerank_noalloc(rp.data_ptr(), col.data_ptr(), 2, 2, out.data_ptr(), damping=d)
        assert e.value.status == mg.MG_ERR_INVALID, d
    with pytest.raises(mg.MGError) as e:   # d_row[nv] = 2, not ne = 3
        mg.pagerank_noalloc(rp.data_ptr(), col.data_ptr(), 2, 3, out.data_ptr())
    assert e.value.status == mg.MG_ERR_INVALID
    it, _ = mg.pagerank_noalloc(rp.data_ptr(), col.data_ptr(), 2, 2, out.data_ptr())
    assert it >= 1 and np.allclose(out.cpu().numpy(), 0.5)
