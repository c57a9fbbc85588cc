"""CPU tests of the host side: loader error handling, generators, the C ABI
surface, failure injection, the CLI shell, and (where oracle/_ref was built
from the reference sources) the oracle and product loader against the
reference's own loader and validator on random graphs."""
import os
import re
import subprocess
import sys
import tempfile

import numpy as np
import pytest

import multigraph_gb300 as mg
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HAVE_REF = O.RefTool.available("BFS") and O.RefTool.available("SSSP")


def _write(tmp, name, text):
    p = os.path.join(tmp, name)
    with open(p, "w") as f:
        f.write(text)
    return p


# --------------------------------------------------------------------------
# C ABI surface
# --------------------------------------------------------------------------
def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "mg.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    declared = set(re.findall(r"\b(mg_[a-z0-9_]+)\s*\(", hdr))
    assert declared == set(mg.EXPORTED), declared ^ set(mg.EXPORTED)
    nm = subprocess.run(["nm", "-D", "--defined-only", mg.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(mg_[a-z0-9_]+)$", nm, flags=re.M))
    missing = declared - exported
    assert not missing, missing
    for name in declared:
        assert getattr(mg.lib, name) is not None


def test_status_strings_and_version():
    assert mg.version().startswith("multigraph-gb300")
    for s in range(10):
        assert mg.lib.mg_status_string(s)
    o = mg.default_opts()
    assert o.alpha > 0 and o.beta > 0 and abs(o.damping - 0.85) < 1e-6


# --------------------------------------------------------------------------
# PageRank's segmented layout, built and checked on the host
# --------------------------------------------------------------------------
def _hub_first(rp, col):
    """The engine's pull CSR of a host graph: vertices renumbered by
    descending floor(log2 degree), input order kept within a degree class,
    each row's columns in the input row's order."""
    n = len(rp) - 1
    deg = np.diff(rp).astype(np.int64)
    lg = np.floor(np.log2(np.maximum(deg, 1))).astype(np.int64)
    new2old = np.lexsort((np.arange(n), -lg))
    old2new = np.empty(n, np.int64)
    old2new[new2old] = np.arange(n)
    ndeg = deg[new2old]
    nrp = np.zeros(n + 1, np.int64)
    nrp[1:] = np.cumsum(ndeg)
    starts = rp[:-1].astype(np.int64)[new2old]
    idx = np.repeat(starts - nrp[:-1], ndeg) + np.arange(nrp[-1])
    return nrp.astype(np.int32), old2new[col[idx]].astype(np.int32)


@pytest.mark.parametrize("scale", [12, 16, 17])
def test_segmented_layout_rmat(scale):
    """R-MAT graphs in the engine's hub-first order: one, two and three
    source segments; every invariant of the layout, and the same layout on
    one host thread as on four."""
    h = mg.HostGraph.rmat(scale, 16, seed=scale)
    rp, col, _ = h.arrays()
    h.free()
    nrp, ncol = _hub_first(rp, col)
    pieces = mg.selftest_segmented_layout(nrp, ncol, threads=4)
    assert len(ncol) / 64 <= pieces <= len(ncol)


def test_segmented_layout_star_and_long_pairs():
    """A star's centre (19,999 in-edges from one segment: 312 full pieces
    and one of 31) and a row whose edges alternate between two segments."""
    n = 70000
    src = np.concatenate([np.zeros(n - 1, np.int64), np.full(200, 5), np.full(200, 65000)])
    dst = np.concatenate([np.arange(1, n), np.arange(60000, 60200), np.arange(0, 200)])
    h = mg.HostGraph.from_entries(n, src.astype(np.int32), dst.astype(np.int32), flags=mg.LOAD_NSYM)
    rp, col, _ = h.arrays()
    h.free()
    assert mg.selftest_segmented_layout(rp, col, threads=3) > 0


def test_segmented_layout_ids_past_the_segments():
    """A 2000 x 2000 lattice (4 M vertices, more than the 64 segments'
    3.67 M): the in-edges from ids past the segments go to the rows' tails."""
    h = mg.HostGraph.lattice(2000, 2000, 0.05, seed=3)
    rp, col, _ = h.arrays()
    h.free()
    assert len(rp) - 1 > 64 * 57344
    assert mg.selftest_segmented_layout(rp, col, threads=8) > 0


def _csr_from_rows(n, rows):
    """CSR with rows[v] = list of column ids (rows not given are empty)."""
    rp = np.zeros(n + 1, np.int64)
    for v, cols in rows.items():
        rp[v + 1] = len(cols)
    rp = np.cumsum(rp)
    col = np.zeros(int(rp[-1]), np.int32)
    for v, cols in rows.items():
        col[rp[v]:rp[v + 1]] = cols
    return rp.astype(np.int32), col


@pytest.mark.parametrize("n", [57344, 57345, 2 * 57344 + 7])
def test_segmented_layout_piece_boundaries(n):
    """Rows with exactly 64, 65, 128 and 129 in-edges from one segment (full
    pieces only, a full piece and one edge, two full pieces, ...), rows split
    across segments, empty rows, and segment counts at the boundary of one
    segment (57,344 vertices) and one past it (a second segment of one
    vertex)."""
    rng = np.random.default_rng(n)
    rows = {0: list(range(64)), 1: list(range(100, 165)), 2: list(range(0, 128)), 3: list(range(1, 130)),
            4: [n - 1] * 3 + [0, 1], 5: [n - 1], 7: [57343, 57344 % n, 5]}
    for v in range(8, 200):
        rows[v] = sorted(rng.integers(0, n, size=int(rng.integers(1, 300))).tolist())
    rp, col = _csr_from_rows(n, rows)
    assert mg.selftest_segmented_layout(rp, col, threads=4) > 0


def test_segmented_layout_tail_boundary_and_unused():
    """One vertex past the 64 segments (a tail of one id), and a graph whose
    in-edges mostly come from past the segments (the layout is not used)."""
    cover = 64 * 57344
    n = cover + 1
    rows = {0: [cover, 1, 2, 3], 1: [0] * 10, 2: [cover - 1, cover]}
    rp, col = _csr_from_rows(n, rows)
    assert mg.selftest_segmented_layout(rp, col, threads=2) > 0
    n = cover + 64
    rows = {v: list(range(cover, cover + 64)) for v in range(10)}
    rows[10] = [0]
    rp, col = _csr_from_rows(n, rows)
    assert mg.selftest_segmented_layout(rp, col, threads=2) == 0


def test_segmented_layout_rejects_bad_csr():
    rp = np.array([0, 2, 3], np.int32)
    with pytest.raises(mg.MGError) as e:
        mg.selftest_segmented_layout(rp, np.array([0, 5, 1], np.int32))
    assert e.value.status == mg.MG_ERR_INVALID
    with pytest.raises(mg.MGError) as e:
        mg.selftest_segmented_layout(np.array([0, 2, 1], np.int32), np.array([0, 1], np.int32))
    assert e.value.status == mg.MG_ERR_INVALID


# --------------------------------------------------------------------------
# loader errors (the reference exits or crashes on these, read_input.cu:24,73-76)
# --------------------------------------------------------------------------
def test_loader_errors():
    tmp = tempfile.mkdtemp()
    with pytest.raises(mg.MGError) as e:
        mg.HostGraph.load_mtx(os.path.join(tmp, "missing.mtx"))
    assert e.value.status == mg.MG_ERR_IO
    p = _write(tmp, "trunc.mtx", "%%MatrixMarket matrix coordinate pattern general\n4 4 3\n1 2\n2 3\n")
    with pytest.raises(mg.MGError) as e:
        mg.HostGraph.load_mtx(p)
    assert e.value.status == mg.MG_ERR_PARSE
    p = _write(tmp, "range.mtx", "%%MatrixMarket matrix coordinate pattern general\n4 4 2\n1 2\n2 5\n")
    with pytest.raises(mg.MGError) as e:
        mg.HostGraph.load_mtx(p)
    assert e.value.status == mg.MG_ERR_RANGE
    p = _write(tmp, "ok.mtx", "%%MatrixMarket matrix coordinate pattern general\n4 4 2\n1 2\n2 3\n")
    with pytest.raises(mg.MGError) as e:
        mg.HostGraph.load_mtx(p, source=9)
    assert e.value.status == mg.MG_ERR_RANGE
    p = _write(tmp, "nosize.mtx", "%%MatrixMarket matrix coordinate pattern general\n% only comments\n")
    with pytest.raises(mg.MGError) as e:
        mg.HostGraph.load_mtx(p)
    assert e.value.status == mg.MG_ERR_PARSE
    # general file whose only entry is dropped by compaction: the reference
    # would write past its arrays; the loader refuses the graph
    p = _write(tmp, "degenerate.mtx", "%%MatrixMarket matrix coordinate pattern general\n6 6 1\n6 5\n")
    with pytest.raises(mg.MGError) as e:
        mg.HostGraph.load_mtx(p, flags=mg.LOAD_NSYM)
    assert e.value.status == mg.MG_ERR_INVALID
    with pytest.raises(OSError):
        O.load_mtx(p, 0, O.LOAD_NSYM)


def test_multi_line_entries_use_stream_parser():
    tmp = tempfile.mkdtemp()
    p1 = _write(tmp, "a.mtx", "%%MatrixMarket matrix coordinate integer general\n4 4 3\n1 2 5\n2 3 6\n3 4 7\n")
    p2 = _write(tmp, "b.mtx", "%%MatrixMarket matrix coordinate integer general\n4 4 3\n1 2\n5 2 3 6\n\n3\n4 7\n")
    a, b = mg.HostGraph.load_mtx(p1).arrays(), mg.HostGraph.load_mtx(p2).arrays()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_from_entries_and_csr_validation():
    h = mg.HostGraph.from_entries(5, [0, 1, 2], [1, 2, 3], [4, 5, 6])
    rp, col, wt = h.arrays()
    assert h.nv == 4 and h.ne == 6 and rp.tolist() == [0, 1, 3, 5, 6]
    with pytest.raises(mg.MGError):
        mg.HostGraph.from_entries(3, [0], [5])
    with pytest.raises(mg.MGError):
        mg.HostGraph.from_csr([0, 2, 1], [0, 1])
    g = mg.HostGraph.from_csr([0, 1, 2], [1, 0])
    assert g.nv == 2 and g.ne == 2


# --------------------------------------------------------------------------
# generators and the writer
# --------------------------------------------------------------------------
def test_rmat_deterministic_and_threads_independent():
    a = mg.HostGraph.rmat(10, 8, seed=5, nthreads=1).arrays()
    b = mg.HostGraph.rmat(10, 8, seed=5, nthreads=4).arrays()
    c = mg.HostGraph.rmat(10, 8, seed=6).arrays()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert not np.array_equal(a[1], c[1])
    rp, col, wt = a
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    assert not np.any(rows == col)                      # no self-loops
    key = rows.astype(np.int64) * n + col
    assert len(np.unique(key)) == len(key)              # no duplicates
    assert np.all(np.diff(rp) > 0)                      # compaction: no isolated vertices
    assert wt.min() >= 1 and wt.max() <= 64
    rkey = col.astype(np.int64) * n + rows
    assert np.array_equal(np.sort(rkey), np.sort(key))  # symmetric


def test_lattice_shape():
    h = mg.HostGraph.lattice(5, 4, 0.0)
    assert h.nv == 20 and h.ne == 2 * (5 * 3 + 4 * 4)
    h2 = mg.HostGraph.lattice(30, 30, 0.05, seed=1)
    assert h2.ne > 2 * (30 * 29 * 2)


def test_write_mtx_round_trip():
    tmp = tempfile.mkdtemp()
    h = mg.HostGraph.rmat(9, 8, seed=2)
    p = os.path.join(tmp, "r.mtx")
    h.write_mtx(p, True)
    back = mg.HostGraph.load_mtx(p, 0, mg.LOAD_SYM)
    for x, y in zip(h.arrays(), back.arrays()):
        assert np.array_equal(x, y)
    o = O.load_mtx(p, 0, O.LOAD_SYM)
    assert np.array_equal(o.csc_e, h.arrays()[1])


def test_binary_csr_cache_round_trip_and_corruption():
    tmp = tempfile.mkdtemp()
    src = _write(tmp, "s.mtx", "%%MatrixMarket matrix coordinate integer symmetric\n6 6 4\n2 1 5\n3 2 7\n5 4 1\n6 5 9\n")
    for h in (mg.HostGraph.rmat(10, 8, seed=5), mg.HostGraph.load_mtx(src, 3, mg.LOAD_SYM)):
        p = os.path.join(tmp, "g.mgcsr")
        h.save_csr(p)
        back = mg.HostGraph.load_csr(p)
        assert (back.nv, back.ne, back.view().start_p, back.view().tra) == \
            (h.nv, h.ne, h.view().start_p, h.view().tra)
        for x, y in zip(h.arrays(), back.arrays()):
            assert np.array_equal(x, y)
    raw = bytearray(open(p, "rb").read())
    bad = []
    flip = bytearray(raw)
    flip[-5] ^= 0x40                                   # a weight bit: checksum
    bad.append(("flip.mgcsr", flip))
    bad.append(("trunc.mgcsr", raw[:-4]))              # size check
    magic = bytearray(raw)
    magic[0:8] = b"NOTACSR!"
    bad.append(("magic.mgcsr", magic))
    bad.append(("short.mgcsr", raw[:20]))              # header cut
    for name, data in bad:
        q = os.path.join(tmp, name)
        with open(q, "wb") as f:
            f.write(data)
        with pytest.raises(mg.MGError) as e:
            mg.HostGraph.load_csr(q)
        assert e.value.status == mg.MG_ERR_PARSE, name
    with pytest.raises(mg.MGError) as e:
        mg.HostGraph.load_csr(os.path.join(tmp, "missing.mgcsr"))
    assert e.value.status == mg.MG_ERR_IO


# --------------------------------------------------------------------------
# failure injection (host side): the k-th allocation fails
# --------------------------------------------------------------------------
def test_allocation_failure_injection():
    code = ("import multigraph_gb300 as mg\n"
            "try:\n    mg.HostGraph.rmat(8, 8)\n    print('NOFAIL')\n"
            "except mg.MGError as e:\n    print('STATUS', e.status)\n")
    for k in (1, 3, 6):
        env = dict(os.environ, MG_FAIL_ALLOC_AT=str(k), PYTHONPATH=ROOT)
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=120)
        assert f"STATUS {mg.MG_ERR_OOM}" in r.stdout, (k, r.stdout, r.stderr)


# --------------------------------------------------------------------------
# CLI shell (no GPU needed for the argument checks)
# --------------------------------------------------------------------------
def test_cli_usage_and_errors():
    cli = os.path.join(mg.BIN_DIR, "BFS")
    r = subprocess.run([cli], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([cli, "/nonexistent.mtx", "0", "1"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 10 + mg.MG_ERR_IO and "load failed" in r.stderr


# --------------------------------------------------------------------------
# against the reference's own loader / validator (oracle/_ref), random graphs
# --------------------------------------------------------------------------
@pytest.mark.skipif(not HAVE_REF, reason="oracle/_ref not built (needs the reference tree)")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_loaders_and_oracle_against_reference(seed):
    tmp = tempfile.mkdtemp()
    p = os.path.join(tmp, "g.mtx")
    mg.HostGraph.rmat(9 + seed, 8, seed=seed).write_mtx(p, True)
    src = 3 * seed
    ref = O.RefTool("SSSP").load(p, src, tmp)
    orc = O.load_mtx(p, src, O.LOAD_SYM)
    prod = mg.HostGraph.load_mtx(p, src, mg.LOAD_SYM)
    for a, b, c in zip((ref.csc_v, ref.csc_e, ref.csc_ev), (orc.csc_v, orc.csc_e, orc.csc_ev), prod.arrays()):
        assert np.array_equal(a, b) and np.array_equal(a, c)
    assert ref.start_p == orc.start_p == prod.start_p
    s = orc.start_p
    assert O.RefTool("BFS").validate(p, src, [O.bfs(orc, s)], tmp).endswith("PASS")
    assert O.RefTool("SSSP").validate(p, src, [O.sssp(orc, s)[0]], tmp).endswith("PASS")
    assert O.RefTool("BC").validate(p, src, list(O.bc(orc, s)), tmp).endswith("PASS")
    occ = O.load_mtx(p, 0, O.LOAD_SYM | O.LOAD_CC)
    assert O.RefTool("CC").validate(p, 0, [O.cc_minlabel(occ)], tmp).endswith("PASS")
    for mode, alg in ((0, "PR_T"), (1, "PR_D")):
        assert O.RefTool(alg).validate(p, 0, [O.pr_ref(orc, mode)[0]], tmp).endswith("PASS")


@pytest.mark.skipif(not HAVE_REF, reason="oracle/_ref not built (needs the reference tree)")
def test_reference_validator_catches_planted_mistakes():
    tmp = tempfile.mkdtemp()
    p = os.path.join(tmp, "g.mtx")
    mg.HostGraph.rmat(9, 8, seed=4).write_mtx(p, True)
    orc = O.load_mtx(p, 0, O.LOAD_SYM)
    lv = O.bfs(orc, 0)
    lv[lv.argmax()] -= 1  # planted in the oracle's result, on the CPU
    assert "FAIL" in O.RefTool("BFS").validate(p, 0, [lv], tmp)
    d = O.sssp(orc, 0)[0]
    d[5] += 1
    assert "FAIL" in O.RefTool("SSSP").validate(p, 0, [d], tmp)


def test_oracle_long_double_brandes_matches_fp64():
    """The long-double Brandes of the oracle agrees with the FP64 one where
    FP64 path counts are exact."""
    from oracle import oracle as O
    h = mg.HostGraph.lattice(30, 20, 0.05, seed=4)
    rp, col, wt = h.arrays()
    og = O.csr_from_arrays(rp, col, wt)
    lv, sg, dl = O.bc_f64(og, 3)
    lv2, ls, dl2 = O.bc_ext(og, 3)
    assert np.array_equal(lv, lv2)
    assert np.allclose(np.exp2(ls), sg, rtol=1e-12, atol=0)
    assert np.allclose(dl2, dl, rtol=1e-12, atol=1e-12)
    assert np.allclose(O.bc_multi_ext(og, [3, 9]), O.bc_multi_f64(og, [3, 9]), rtol=1e-12, atol=1e-12)


def test_stage_bytes_unpinned():
    h = mg.HostGraph.rmat(8, 8, seed=1)
    rp, col, _ = h.arrays()
    assert h.stage_bytes() == 4 * len(rp) + 8 * len(col)


def test_bench_clock_summary_from_nvml_samples():
    """bench.py's clock record: median SM clock over samples taken under
    load, and the throttle reasons seen under load (NVML clock-event bits)."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    class FakeNvml:
        shut = False

        def nvmlShutdown(self):
            FakeNvml.shut = True
            return 0

    c = bench.ClockSampler.__new__(bench.ClockSampler)
    c.device, c.thread, c.running, c.lib = 0, None, False, FakeNvml()
    # (sm MHz, max MHz, utilisation %, clock-event reason bits, W)
    c.samples = [(2070, 2070, 0, 0x1, 90.0), (2070, 2070, 97, 0x4, 1390.0), (1995, 2070, 99, 0x4, 1400.0),
                 (2070, 2070, 98, 0x0, 1200.0)]
    r = c.stop()
    assert FakeNvml.shut
    assert r["sm_mhz"] == 2070 and r["sm_max_mhz"] == 2070
    assert r["reasons"] == ["sw_power_cap"]
    assert r["samples"] == 4 and r["samples_under_load"] == 3
    c2 = bench.ClockSampler.__new__(bench.ClockSampler)
    c2.device, c2.thread, c2.running, c2.lib, c2.samples = 0, None, False, None, []
    c2.start()  # no NVML: nothing to poll
    assert c2.stop()["reasons"] == ["NVML unavailable"]
