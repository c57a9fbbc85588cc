"""In-tree build of libmg.so (CUDA kernels + C ABI) and the CLI binaries.

Compiles every translation unit for sm_103a only (one -gencode), in
parallel, into ``multigraph_gb300/_build/`` and links
``multigraph_gb300/libmg.so`` plus ``multigraph_gb300/bin/mg`` with the
reference's binary names (BFS, SSSP, BC, CC, DATA_DRIVEN_PR,
TOPOLOGY_DRIVEN_PR) as symlinks.  No cmake, no torch extension machinery.

    python -m multigraph_gb300.build
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "libmg.so")
BIN = os.path.join(PKG, "bin")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
CU_SOURCES = ["mg_device.cu", "mg_frontier.cu", "mg_pr.cu", "mg_hub.cu", "mg_cc.cu", "mg_tune.cu", "mg_noalloc.cu",
              "mg_bcb.cu"]
CU_FLAGS = {}  # per-file extra nvcc flags
CPP_SOURCES = ["mg_host.cpp"]
CLI_NAMES = ["BFS", "SSSP", "BC", "CC", "DATA_DRIVEN_PR", "TOPOLOGY_DRIVEN_PR"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return [os.path.join(d, f) for d in (CSRC, INCLUDE) for f in os.listdir(d) if f.endswith((".h", ".cuh"))]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Build libmg.so and the CLI; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            cmd = [nvcc, GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I", INCLUDE, "-I", CSRC] + CU_FLAGS.get(src, []) + ["-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(3, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-pthread", "-I", INCLUDE, "-I", CSRC,
                         "-c", s, "-o", o])
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    if verbose:
        for line in logs:
            if line.strip():
                print(line)
    if _stale(LIB, objs):
        _run([nvcc, GENCODE, "-shared", "-Xcompiler", "-fPIC", "-o", LIB] + objs + ["-lpthread"])
    cli_src = os.path.join(CSRC, "mg_cli.cpp")
    cli = os.path.join(BIN, "mg")
    if _stale(cli, [cli_src, LIB, os.path.join(INCLUDE, "mg.h")]):
        _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, cli_src, "-o", cli, "-L", PKG, "-lmg",
              "-Wl,-rpath,$ORIGIN/..", "-pthread"])
    for name in CLI_NAMES:
        link = os.path.join(BIN, name)
        if not os.path.lexists(link):
            os.symlink("mg", link)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
