"""The oracle's additions for the full-size checks, pinned on the CPU:

* its R-MAT generator gives, byte for byte, the CSR the library's generator
  gives (the reference arm of bench.py builds its input with it, without
  loading the product library);
* its in-memory loader pipeline equals its file loader on the same entries
  (the file loader is pinned against the reference's own generate_CSC in
  test_golden.py);
* its batched central differences of the weighted-PageRank loss equal
  differences of two complete FP64 solves per edge, and the FP64 adjoint.
"""
import numpy as np
import pytest

import multigraph_gb300 as mg
from oracle import oracle as O


@pytest.mark.parametrize("scale,ef,seed", [(6, 4, 1), (10, 16, 3), (13, 8, 22)])
def test_rmat_generator_matches_library(scale, ef, seed):
    og = O.gen_rmat(scale, ef, seed=seed)
    h = mg.HostGraph.rmat(scale, ef, seed=seed)
    rp, col, wt = h.arrays()
    assert og.nv == len(rp) - 1 and og.ne == len(col)
    assert np.array_equal(og.csc_v, rp)
    assert np.array_equal(og.csc_e, col)
    assert np.array_equal(og.csc_ev, wt)
    h.free()


@pytest.mark.parametrize("flags", [O.LOAD_SYM, O.LOAD_NSYM, O.LOAD_NSYM | O.LOAD_CC])
def test_entry_loader_matches_file_loader(tmp_path, flags):
    rng = np.random.default_rng(5)
    n, k = 300, 2500
    src = rng.integers(0, n, k)
    dst = rng.integers(0, n, k)
    val = rng.integers(1, 64, k)
    src[:40] = 7    # a row of 40+ entries with repeats
    path = tmp_path / "g.mtx"
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate integer general\n% comment\n")
        f.write(f"{n} {n} {k}\n")
        for s, d, v in zip(src, dst, val):
            f.write(f"{s + 1} {d + 1} {v}\n")
    a = O.load_mtx(str(path), 7, flags=flags)
    b = O.from_entries(n, src, dst, val, source=7, flags=flags)
    assert (a.nv, a.ne, a.start_p, a.tra) == (b.nv, b.ne, b.start_p, b.tra)
    assert np.array_equal(a.csc_v, b.csc_v) and np.array_equal(a.csc_e, b.csc_e)
    assert np.array_equal(a.csc_ev, b.csc_ev)


def test_batched_differences_match_full_solves():
    og = O.gen_rmat(9, 8, seed=4)
    rng = np.random.default_rng(4)
    w = rng.uniform(0.0, 1.0, og.ne)
    w = np.where(w == 0.0, 1.0, w)
    gv = rng.standard_normal(og.nv)
    x, _ = O.wpr_f64(og, w, 0.85, 1e-15, 2000)
    idx = rng.choice(og.ne, 5, replace=False).astype(np.int32)
    fd, sweeps = O.wpr_fd_f64(og, w, x, gv, idx, eps=1e-3, rtol=1e-11, nthreads=3)
    assert 0 < sweeps < 2000
    full = []
    for e in idx:
        wp, wm = w.copy(), w.copy()
        wp[e] += 1e-3
        wm[e] -= 1e-3
        full.append((O.wpr_loss_f64(og, wp, gv, tol=1e-15, max_iter=2000)
                     - O.wpr_loss_f64(og, wm, gv, tol=1e-15, max_iter=2000)) / 2e-3)
    _, gw, _, _ = O.wpr_adjoint_f64(og, w, x, gv, 0.85, 1e-15, 2000)
    scale = float(np.max(np.abs(gw)))
    assert float(np.max(np.abs(fd - np.array(full)))) / scale < 1e-8
    assert float(np.max(np.abs(fd - gw[idx]))) / scale < 1e-6
