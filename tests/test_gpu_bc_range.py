"""Betweenness on graphs whose shortest-path counts leave the FP64 range.

The number of shortest paths on a lattice grows like 2^distance, so after
about a thousand levels the counts pass 1.8e308.  The engines then switch to
extended path counts (FP64 mantissa with a 2^512 scale) and the dependencies
stay exact to FP32; the checks use the oracle's long-double Brandes."""
import numpy as np
import pytest

import multigraph_gb300 as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pair(h):
    rp, col, wt = h.arrays()
    return mg.Graph(h), O.csr_from_arrays(rp, col, wt)


def _check_single(g, og, src):
    (lv, sg, dl), _ = g.bc(src)
    rlv, rls, rdl = O.bc_ext(og, src)
    assert np.array_equal(lv, rlv)
    reached = rls >= 0
    fits = reached & (rls < 1023.0)
    assert np.all(np.isinf(sg[reached & (rls > 1024.5)]))
    assert np.allclose(np.log2(sg[fits]), rls[fits], rtol=0, atol=1e-9)
    err = float(np.max(np.abs(dl.astype(np.float64) - rdl)) / np.max(np.abs(rdl)))
    assert err < 1e-5, err
    return rls


def test_counts_past_2_512_match_fp64_oracle():
    # 1024 x 1024: counts reach ~2^618 (extended mode) but stay inside FP64,
    # so the plain FP64 oracle is a second check
    h = mg.HostGraph.lattice(1024, 1024, 0.05, seed=5)
    g, og = _pair(h)
    rls = _check_single(g, og, 7)
    assert rls.max() > 512
    (_, sg, dl), _ = g.bc(7)
    _, rsg, rdl = O.bc_f64(og, 7)
    assert np.allclose(sg, rsg, rtol=1e-12, atol=0)
    g.free()


def test_counts_past_fp64_range():
    h = mg.HostGraph.lattice(1800, 1800, 0.05, seed=6)
    g, og = _pair(h)
    rls = _check_single(g, og, 0)
    assert rls.max() > 1100           # genuinely past FP64
    srcs = [0, og.nv // 2 + 37]
    bc, _ = g.bc_multi(srcs)
    ref = O.bc_multi_ext(og, srcs)
    assert np.all(np.isfinite(bc))
    err = float(np.max(np.abs(bc.astype(np.float64) - ref)) / np.max(np.abs(ref)))
    assert err < 1e-5, err
    g.free()
