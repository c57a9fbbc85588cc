"""CPU tests: the oracle and the product loader against the golden vectors.

tests/golden/expected.json was produced by tests/golden/make_golden.py from
the reference's own generate_CSC and verifyResults (compiled from the
reference sources into oracle/_ref/).  These tests need no GPU and no
reference tree.
"""
import json
import os

import numpy as np
import pytest

import multigraph_gb300 as mg
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "expected.json")))
MTX = os.path.join(HERE, "golden", "mtx")
NAMES = sorted(GOLD)


def _same_csr(g, d, with_ev):
    assert g.nv == d["nv"] and g.ne == d["ne"] and g.start_p == d["start_p"]
    assert np.array_equal(g.csc_v, d["csc_v"]) and np.array_equal(g.csc_e, d["csc_e"])
    if with_ev and "csc_ev" in d:
        assert np.array_equal(g.csc_ev, d["csc_ev"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_loader_matches_reference(name):
    e = GOLD[name]
    path = os.path.join(MTX, name)
    _same_csr(O.load_mtx(path, e["source"], O.LOAD_SYM), e["csr_sym"], True)
    _same_csr(O.load_mtx(path, e["source"], O.LOAD_NSYM), e["csr_nsym"], False)
    _same_csr(O.load_mtx(path, 0, O.LOAD_SYM | O.LOAD_CC), e["csr_cc"], False)


@pytest.mark.parametrize("name", NAMES)
def test_product_loader_matches_reference(name):
    e = GOLD[name]
    path = os.path.join(MTX, name)
    for flags, src, key, ev in ((mg.LOAD_SYM, e["source"], "csr_sym", True),
                                (mg.LOAD_NSYM, e["source"], "csr_nsym", False),
                                (mg.LOAD_SYM | mg.LOAD_CC, 0, "csr_cc", False)):
        for nthreads in (1, 3):
            h = mg.HostGraph.load_mtx(path, src, flags, nthreads=nthreads)
            rp, col, wt = h.arrays()
            g = O.CSR(h.nv, h.ne, h.start_p, 0, rp, col, wt)
            _same_csr(g, e[key], ev)
            h.free()


@pytest.mark.parametrize("name", NAMES)
def test_oracle_algorithms_match_golden(name):
    e = GOLD[name]
    assert all(v.endswith("PASS") for v in e["reference_verdicts"].values()), e["reference_verdicts"]
    path = os.path.join(MTX, name)
    g = O.load_mtx(path, e["source"], O.LOAD_SYM)
    s = g.start_p
    assert np.array_equal(O.bfs(g, s), e["bfs"])
    if "sssp" in e:
        assert np.array_equal(O.sssp(g, s)[0], e["sssp"])
    lv, sg, dl = O.bc(g, s)
    assert np.array_equal(lv, e["bc_level"]) and np.array_equal(sg, e["bc_sigma"])
    assert np.array_equal(dl, np.array(e["bc_delta"], dtype=np.float32))
    for mode, key in ((0, "pr_t"), (1, "pr_d")):
        pr, it = O.pr_ref(g, mode)
        assert it == e[key + "_sweeps"]
        assert np.array_equal(pr, np.array(e[key], dtype=np.float32))
    gc = O.load_mtx(path, 0, O.LOAD_SYM | O.LOAD_CC)
    assert np.array_equal(O.cc_minlabel(gc), e["cc_minlabel"])


def test_hand_derived_cases():
    # path 1-2-3-4-5, symmetrised: levels from vertex 0
    g = O.load_mtx(os.path.join(MTX, "path5.mtx"), 0, O.LOAD_SYM)
    assert O.bfs(g, 0).tolist() == [0, 1, 2, 3, 4]
    # star: centre 3 (1-based) renumbered to 2; every leaf at level 1 from it
    g = O.load_mtx(os.path.join(MTX, "star6.mtx"), 2, O.LOAD_SYM)
    assert g.start_p == 2 and O.bfs(g, 2).tolist() == [1, 1, 0, 1, 1, 1]
    # weighted 4-clique: shortest paths from vertex 0 (edge weights 3,1,7,2,5,4)
    g = O.load_mtx(os.path.join(MTX, "clique4_w.mtx"), 0, O.LOAD_SYM)
    assert O.sssp(g, 0)[0].tolist() == [0, 3, 1, 5]
    # two components (vertices 1, 6, 9 unused): compaction keeps 7 vertices
    g = O.load_mtx(os.path.join(MTX, "twocomp.mtx"), 1, O.LOAD_SYM)
    assert g.nv == 7
    assert O.cc_relabel(O.cc_minlabel(g)).tolist() == [0, 0, 0, 1, 1, 1, 1]
    # duplicates: (1,2) appears three times; the first value read (3.7 -> 3) is kept
    g = O.load_mtx(os.path.join(MTX, "dups_real.mtx"), 0, O.LOAD_SYM)
    assert g.csc_e[0] == 1 and g.csc_ev[0] == 3
    # the self-loop (2,2) is kept once in symmetric mode
    row1 = g.csc_e[g.csc_v[1]:g.csc_v[2]].tolist()
    assert row1.count(1) == 1


def test_pattern_weights_identical_in_oracle_and_product():
    for seed in (1, 7):
        for entry in (0, 1, 100, 12345):
            assert 1 <= O.pattern_weight(seed, entry) <= 64
        for name in ("twocomp.mtx", "star6.mtx", "path5.mtx"):  # pattern files
            h = mg.HostGraph.load_mtx(os.path.join(MTX, name), 0, mg.LOAD_SYM, weight_seed=seed)
            o = O.load_mtx(os.path.join(MTX, name), 0, O.LOAD_SYM, seed)
            assert np.array_equal(h.arrays()[2], o.csc_ev)
            assert o.csc_ev.min() >= 1 and o.csc_ev.max() <= 64
