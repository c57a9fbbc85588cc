"""GPU parity at the benchmark configurations' full sizes, against the oracle.

Each test builds the configuration's synthetic input at its stated size and
checks the GPU result through the C ABI against the CPU oracle:

  C1  R-MAT 16 (edge factor 16) written as MTX and read back by the loader:
      loader CSR, BFS from 0 and CC labels bit-exact; the CC loader rule
      (src < dst entries only) on the same file, CC bit-exact.
  C2  R-MAT 22 (edge factor 16, weights 1..64): SSSP from 0 bit-exact;
      normalised topology- and data-driven PageRank (d 0.85, L1 tol 1e-6)
      within 1e-6 max-abs of FP64; the reference PR_T / PR_D recurrences
      within validate.cu's 5 % rule.
  C3  4096 x 4096 lattice + 5 % diagonal shortcuts: BFS bit-exact; BC of
      two of the 64 benchmark sources within 1e-5 relative of a
      long-double-sigma Brandes (path counts here pass the FP64 range).
  C4  R-MAT 20: all 256 BC sources in one batched call within 1e-5
      relative of the FP64 multi-source oracle; 256 personalised
      PageRanks within 1e-6 max-abs of FP64 run for the same sweeps; the
      64-graph batch (scales 10-18, edge factor 8-32) BFS + CC bit-exact.
  C5  R-MAT 21 with FP32 weights in (0, 1]: forward within 1e-6 max-abs of
      FP64; edge gradient within 1e-4 (normwise relative) of the FP64
      adjoint, and of FP64 central differences (eps 1e-3) on 32 edges.

Oracle work is spread over host threads (the oracle's C calls release the
interpreter lock).  Inputs and seeds match bench.py's.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import multigraph_gb300 as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NT = max(1, min(16, os.cpu_count() or 1))


def _pmap(fn, items):
    with ThreadPoolExecutor(max_workers=NT) as ex:
        return list(ex.map(fn, items))


def _og(h):
    rp, col, wt = h.arrays()
    return O.csr_from_arrays(rp, col, wt)


def test_c1_rmat16_mtx_bfs_cc(tmp_path):
    h0 = mg.HostGraph.rmat(16, 16, seed=16)
    path = str(tmp_path / "rmat16.mtx")
    h0.write_mtx(path, with_weights=True)
    h0.free()
    for flags in (mg.LOAD_NSYM, mg.LOAD_SYM):
        h = mg.HostGraph.load_mtx(path, 0, flags=flags)
        og = O.load_mtx(path, 0, flags=flags)
        rp, col, wt = h.arrays()
        assert np.array_equal(rp, og.csc_v) and np.array_equal(col, og.csc_e) and np.array_equal(wt, og.csc_ev)
        g = mg.Graph(h)
        lv, _ = g.bfs(og.start_p)
        assert np.array_equal(lv, O.bfs(og, og.start_p))
        lab, _ = g.cc()
        assert np.array_equal(lab, O.cc_minlabel(og))
        g.free()
        h.free()
    # the CC build's loader keeps src < dst entries only (read_input.cu:111-113)
    hc = mg.HostGraph.load_mtx(path, 0, flags=mg.LOAD_NSYM | mg.LOAD_CC)
    ogc = O.load_mtx(path, 0, flags=mg.LOAD_NSYM | mg.LOAD_CC)
    rp, col, _ = hc.arrays()
    assert np.array_equal(rp, ogc.csc_v) and np.array_equal(col, ogc.csc_e)
    assert np.all(col > np.repeat(np.arange(len(rp) - 1), np.diff(rp)))
    g = mg.Graph(hc)
    lab, _ = g.cc()
    ref = O.cc_minlabel(ogc)
    assert np.array_equal(lab, ref)
    assert np.array_equal(O.cc_relabel(lab), O.cc_relabel(ref))
    g.free()
    hc.free()


@pytest.fixture(scope="module")
def rmat22():
    h = mg.HostGraph.rmat(22, 16, seed=22)
    og = _og(h)
    g = mg.Graph(h)
    yield g, og
    g.free()
    h.free()


def test_c2_rmat22_sssp_bit_exact(rmat22):
    g, og = rmat22
    for direction in (mg.DIR_AUTO, mg.DIR_PULL):
        d, _ = g.sssp(0, direction=direction)
        ref, _ = O.sssp(og, 0)
        assert np.array_equal(d, ref), (direction, int(np.sum(d != ref)))


def test_c2_rmat22_pagerank(rmat22):
    g, og = rmat22
    x, info = g.pagerank(mg.PR_TOPOLOGY, tol=1e-6, damping=0.85)
    ref, it = O.pr_norm_f64(og, 0.85, 1e-6, info.iterations)
    assert it == info.iterations
    err = float(np.max(np.abs(x.astype(np.float64) - ref)))
    assert err < 1e-6, err
    # data-driven form: vertices freeze once their change is <= tol / n;
    # against the converged FP64 fixed point
    xd, dinfo = g.pagerank(mg.PR_DATA, tol=1e-6, damping=0.85)
    exact, _ = O.pr_norm_f64(og, 0.85, 1e-10, 400)
    errd = float(np.max(np.abs(xd.astype(np.float64) - exact)))
    assert errd < 1e-6, errd
    assert dinfo.iterations >= 1


def test_c2_rmat22_reference_recurrences(rmat22):
    g, og = rmat22
    (rt, _), (rd, _) = _pmap(lambda mode: O.pr_ref_f64(og, mode), [0, 1])
    for variant, ref in ((mg.PR_TOPOLOGY_REF, rt), (mg.PR_DATA_REF, rd)):
        x, _ = g.pagerank(variant)
        rel = float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-12)))
        assert rel < 0.05, (variant, rel)   # validate.cu:93-100 (THR = 5 %)


def test_c3_lattice4096_bfs_bc():
    h = mg.HostGraph.lattice(4096, 4096, 0.05, seed=3)
    og = _og(h)
    g = mg.Graph(h)
    try:
        src = np.random.default_rng(64).integers(0, g.nv, 64).astype(np.int32)
        lv, _ = g.bfs(int(src[0]))
        assert np.array_equal(lv, O.bfs(og, int(src[0])))
        pick = src[:2]
        bc, _ = g.bc_multi(pick)
        ref = O.bc_multi_ext(og, pick)
        assert np.all(np.isfinite(bc))
        err = float(np.max(np.abs(bc.astype(np.float64) - ref)) / np.max(np.abs(ref)))
        assert err < 1e-5, err
    finally:
        g.free()
        h.free()


@pytest.fixture(scope="module")
def rmat20():
    h = mg.HostGraph.rmat(20, 16, seed=20)
    og = _og(h)
    g = mg.Graph(h)
    yield g, og
    g.free()
    h.free()


def test_c4_bc_256_sources(rmat20):
    g, og = rmat20
    src = np.random.default_rng(20).integers(0, g.nv, 256).astype(np.int32)
    bc, info = g.bc_multi(src)
    parts = _pmap(lambda k: O.bc_multi_f64(og, src[k:k + 32]), range(0, 256, 32))
    ref = np.sum(parts, axis=0)
    err = float(np.max(np.abs(bc.astype(np.float64) - ref)) / np.max(np.abs(ref)))
    assert err < 1e-5, err


def test_c4_ppr_256_seeds(rmat20):
    g, og = rmat20
    seeds = np.random.default_rng(20).integers(0, g.nv, 256).astype(np.int32)
    x, _ = g.ppr_batch(seeds, tol=1e-6)
    assert x.shape == (256, g.nv)
    # sweeps of each 32-seed group: the same group run on its own (same
    # kernels, so the same iterates) gives its count; the oracle then runs
    # that many FP64 sweeps for one seed of each group
    checks = []
    for k in range(0, 256, 32):
        xg, gi = g.ppr_batch(seeds[k:k + 32], tol=1e-6)
        assert np.array_equal(xg, x[k:k + 32]), k
        for i in (k, k + 31):
            checks.append((i, gi.iterations))
    refs = _pmap(lambda c: O.ppr_f64(og, int(seeds[c[0]]), 0.85, 0.0, c[1])[0], checks)
    for (i, _), ref in zip(checks, refs):
        err = float(np.max(np.abs(x[i].astype(np.float64) - ref)))
        assert err < 1e-6, (i, err)


def test_c4_batch_64_graphs():
    rng = np.random.default_rng(64)
    hs = [mg.HostGraph.rmat(int(sc), int(ef), seed=int(i) + 1) for i, (sc, ef) in
          enumerate(zip(rng.integers(10, 19, 64), rng.integers(8, 33, 64)))]
    ogs = [_og(h) for h in hs]
    b = mg.Batch(hs)
    srcs = [0] * len(hs)
    levels, _ = b.bfs(srcs)
    labels, _ = b.cc()
    b.free()
    refs = _pmap(lambda og: (O.bfs(og, 0), O.cc_minlabel(og)), ogs)
    for k, (rl, rc) in enumerate(refs):
        assert np.array_equal(levels[k], rl), k
        assert np.array_equal(labels[k], rc), k
    for h in hs:
        h.free()


def test_c5_rmat21_adjoint_fd32():
    h = mg.HostGraph.rmat(21, 16, seed=21)
    og = _og(h)
    g = mg.Graph(h)
    try:
        rng = np.random.default_rng(21)
        w = rng.uniform(0.0, 1.0, g.ne)
        w = np.where(w == 0.0, 1.0, w).astype(np.float32)
        g.set_float_weights(w)
        gv = rng.standard_normal(g.nv).astype(np.float32)
        # the gradient inherits the forward's relative error: an L1 change of
        # 1e-9 (x to ~3e-5 relative) keeps it near 1e-5, 1e-6 leaves it near
        # 4e-3; the adjoint needs its own 1e-6 (1e-5 gives ~2e-4)
        x, _ = g.wpagerank(tol=1e-9)
        (grad, _), _ = g.wpagerank_backward(gv, tol=1e-6)
        w64, g64 = w.astype(np.float64), gv.astype(np.float64)
        x64, _ = O.wpr_f64(og, w64, 0.85, 1e-14, 400)
        assert float(np.max(np.abs(x.astype(np.float64) - x64))) < 1e-6
        idx = rng.choice(g.ne, 32, replace=False).astype(np.int32)
        with ThreadPoolExecutor(max_workers=1) as ex:   # the adjoint beside the threaded differences
            adj = ex.submit(O.wpr_adjoint_f64, og, w64, x64, g64, 0.85, 1e-9 * float(np.sum(np.abs(g64))), 400)
            fd, sweeps = O.wpr_fd_f64(og, w64, x64, g64, idx, eps=1e-3, rtol=1e-9, max_iter=400,
                                      nthreads=max(1, NT - 1))
            _, gw64, _, _ = adj.result()
        scale = float(np.max(np.abs(gw64)))
        rel = float(np.max(np.abs(grad.astype(np.float64) - gw64))) / scale
        assert rel < 1e-4, rel
        rel_fd = float(np.max(np.abs(grad[idx].astype(np.float64) - fd))) / scale
        assert rel_fd < 1e-4, rel_fd
        assert float(np.max(np.abs(fd - gw64[idx]))) / scale < 1e-6   # the two FP64 references agree
    finally:
        g.free()
        h.free()
