#!/usr/bin/env python3
"""Regenerate tests/golden/expected.json from the reference itself.

For every fixture in tests/golden/mtx/ this script
  * runs the reference's own loader (generate_CSC, read_input.cu:11) compiled
    into oracle/_ref/ (oracle/Makefile `ref` target) in three builds: -DSYM
    (what install.sh builds), -DNSYM (general matrices) and -DCC -DSYM (the
    src<dst filter), and records the CSR each produces;
  * runs the oracle's restatement of validate.cu on the -DSYM CSR (BFS, SSSP,
    BC, PR_T, PR_D) and on the -DCC CSR (CC), hands each result to the
    reference's own verifyResults, and records the result together with the
    reference's verdict ("validation : PASS").
Pattern files get random weights in the reference (rand() seeded by time,
read_input.cu:21,77), so their weights and SSSP results are not recorded.

Needs the reference tree (only present where oracle/_ref was built):
    make -C oracle ref && python tests/golden/make_golden.py
"""
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from oracle import oracle as O  # noqa: E402

SOURCES = {"renumber.mtx": 5, "star6.mtx": 2}


def is_pattern(path):
    with open(path) as f:
        return "pattern" in f.readline()


def csr_dict(g, with_ev):
    d = {"nv": g.nv, "ne": g.ne, "start_p": g.start_p, "tra": g.tra,
         "csc_v": g.csc_v.tolist(), "csc_e": g.csc_e.tolist()}
    if with_ev:
        d["csc_ev"] = g.csc_ev.tolist()
    return d


def main():
    if not O.RefTool.available("SSSP"):
        sys.exit("oracle/_ref is missing: run `make -C oracle ref` where the reference tree exists")
    out = {}
    tmp = tempfile.mkdtemp()
    for name in sorted(os.listdir(os.path.join(HERE, "mtx"))):
        path = os.path.join(HERE, "mtx", name)
        src = SOURCES.get(name, 0)
        pattern = is_pattern(path)
        e = {"source": src, "pattern": pattern}
        g_sym = O.RefTool("SSSP").load(path, src, tmp)
        e["csr_sym"] = csr_dict(g_sym, not pattern)
        e["csr_nsym"] = csr_dict(O.RefTool("NSYM_BFS").load(path, src, tmp), False)
        g_cc = O.RefTool("CC").load(path, 0, tmp)
        e["csr_cc"] = csr_dict(g_cc, False)
        s = g_sym.start_p
        verdicts = {}
        lv = O.bfs(g_sym, s)
        verdicts["BFS"] = O.RefTool("BFS").validate(path, src, [lv], tmp)
        e["bfs"] = lv.tolist()
        if not pattern:
            d, _ = O.sssp(g_sym, s)
            verdicts["SSSP"] = O.RefTool("SSSP").validate(path, src, [d], tmp)
            e["sssp"] = d.tolist()
        blv, bsg, bdl = O.bc(g_sym, s)
        verdicts["BC"] = O.RefTool("BC").validate(path, src, [blv, bsg, bdl], tmp)
        e["bc_level"] = blv.tolist()
        e["bc_sigma"] = bsg.tolist()
        e["bc_delta"] = [float(x) for x in bdl]
        lab = O.cc_minlabel(g_cc)
        verdicts["CC"] = O.RefTool("CC").validate(path, 0, [lab], tmp)
        e["cc_minlabel"] = lab.tolist()
        for mode, alg in ((0, "PR_T"), (1, "PR_D")):
            pr, it = O.pr_ref(g_sym, mode)
            verdicts[alg] = O.RefTool(alg).validate(path, 0, [pr], tmp)
            e[alg.lower()] = [float(x) for x in pr]
            e[alg.lower() + "_sweeps"] = it
        e["reference_verdicts"] = verdicts
        out[name] = e
        bad = {k: v for k, v in verdicts.items() if not v.endswith("PASS")}
        print(f"{name:18s} nv={g_sym.nv:4d} ne={g_sym.ne:5d} " + ("ok" if not bad else f"REFERENCE REJECTS {bad}"))
    with open(os.path.join(HERE, "expected.json"), "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
