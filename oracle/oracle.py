"""CPU oracle bindings (test infrastructure only).

Loads ``oracle/liboracle.so`` -- the C restatement of the reference's
``code/validate.cu`` CPU algorithms and ``code/read_input.cu`` loader -- and
exposes numpy-level helpers.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` import this module; the product library
``multigraph_gb300`` never does.

``RefTool`` drives the reference's own loader and validator compiled from the
reference sources into ``oracle/_ref/`` (oracle/Makefile); those binaries only
exist where the reference tree was available at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

IUNUSED = 0x64646464
LOAD_SYM, LOAD_NSYM, LOAD_CC = 1, 2, 4

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class _OrcCSR(C.Structure):
    _fields_ = [("nv", C.c_int32), ("ne", C.c_int32), ("start_p", C.c_int32), ("tra", C.c_int32),
                ("csc_v", C.POINTER(C.c_int32)), ("csc_e", C.POINTER(C.c_int32)),
                ("csc_ev", C.POINTER(C.c_int32))]


_lib = None


def build() -> str:
    """Compile liboracle.so with gcc (no GPU needed)."""
    src = os.path.join(HERE, "mg_oracle.c")
    if (not os.path.exists(LIB_PATH)) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "mg_oracle.h"))):
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
                               "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_load_mtx.argtypes = [C.c_char_p, C.c_int32, C.c_uint32, C.c_uint64, C.POINTER(_OrcCSR)]
        L.orc_load_mtx.restype = C.c_int
        L.orc_csr_free.argtypes = [C.POINTER(_OrcCSR)]
        L.orc_pattern_weight.argtypes = [C.c_uint64, C.c_uint64]
        L.orc_pattern_weight.restype = C.c_uint32
        L.orc_bfs.argtypes = [C.c_void_p, C.c_int32, _i32p]
        L.orc_sssp.argtypes = [C.c_void_p, C.c_int32, _i32p, C.c_int32]
        L.orc_sssp.restype = C.c_int
        L.orc_bc.argtypes = [C.c_void_p, C.c_int32, _i32p, _i32p, _f32p]
        L.orc_bc_f64.argtypes = [C.c_void_p, C.c_int32, _i32p, _f64p, _f64p]
        L.orc_bc_multi_f64.argtypes = [C.c_void_p, _i32p, C.c_int32, _f64p]
        L.orc_bc_ext.argtypes = [C.c_void_p, C.c_int32, _i32p, _f64p, _f64p]
        L.orc_bc_multi_ext.argtypes = [C.c_void_p, _i32p, C.c_int32, _f64p]
        L.orc_cc_minlabel.argtypes = [C.c_void_p, _i32p]
        L.orc_cc_minlabel.restype = C.c_int
        L.orc_cc_relabel.argtypes = [C.c_int32, _i32p]
        L.orc_pr_ref.argtypes = [C.c_void_p, C.c_int, _f32p, C.c_int32]
        L.orc_pr_ref.restype = C.c_int
        L.orc_pr_ref_f64.argtypes = [C.c_void_p, C.c_int, _f64p, C.c_int32]
        L.orc_pr_ref_f64.restype = C.c_int
        L.orc_pr_norm_f64.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int32, _f64p]
        L.orc_pr_norm_f64.restype = C.c_int
        L.orc_ppr_f64.argtypes = [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_int32, _f64p]
        L.orc_ppr_f64.restype = C.c_int
        L.orc_wpr_f64.argtypes = [C.c_void_p, _f64p, C.c_double, C.c_double, C.c_int32, _f64p]
        L.orc_wpr_f64.restype = C.c_int
        L.orc_wpr_adjoint_f64.argtypes = [C.c_void_p, _f64p, _f64p, _f64p, C.c_double, C.c_double,
                                          C.c_int32, _f64p, _f64p, _f64p]
        L.orc_wpr_adjoint_f64.restype = C.c_int
        L.orc_wpr_loss_f64.argtypes = [C.c_void_p, _f64p, _f64p, C.c_double, C.c_double, C.c_int32]
        L.orc_wpr_loss_f64.restype = C.c_double
        L.orc_from_entries.argtypes = [C.c_int32, C.c_int64, _i32p, _i32p, C.c_void_p, C.c_int32, C.c_uint32,
                                       C.POINTER(_OrcCSR)]
        L.orc_from_entries.restype = C.c_int
        L.orc_gen_rmat.argtypes = [C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                   C.c_int32, C.c_int32, C.POINTER(_OrcCSR)]
        L.orc_gen_rmat.restype = C.c_int
        L.orc_wpr_fd_f64.argtypes = [C.c_void_p, _f64p, _f64p, _f64p, C.c_double, _i32p, C.c_int32, C.c_double,
                                     C.c_double, C.c_int32, C.c_int32, _f64p]
        L.orc_wpr_fd_f64.restype = C.c_int
        _lib = L
    return _lib


@dataclass
class CSR:
    """Host CSR in the reference's csc_package shape (common.h:170-182)."""
    nv: int
    ne: int
    start_p: int
    tra: int
    csc_v: np.ndarray
    csc_e: np.ndarray
    csc_ev: np.ndarray

    def _struct(self):
        s = _OrcCSR()
        s.nv, s.ne, s.start_p, s.tra = self.nv, self.ne, self.start_p, self.tra
        s.csc_v = self.csc_v.ctypes.data_as(C.POINTER(C.c_int32))
        s.csc_e = self.csc_e.ctypes.data_as(C.POINTER(C.c_int32))
        s.csc_ev = self.csc_ev.ctypes.data_as(C.POINTER(C.c_int32))
        self._keep = s
        return C.byref(s)


def csr_from_arrays(row_ptr, col, wt=None, start_p=0) -> CSR:
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int32)
    col = np.ascontiguousarray(col, dtype=np.int32)
    if wt is None:
        wt = np.ones(len(col), dtype=np.int32)
    wt = np.ascontiguousarray(wt, dtype=np.int32)
    nv = len(row_ptr) - 1
    deg = np.diff(row_ptr)
    tra = int(nv > 1 and (deg[:-1] >= 128).any())
    return CSR(nv, len(col), start_p, tra, row_ptr, col, wt)


def _take(s) -> CSR:
    """Copy a C-allocated orc_csr into numpy arrays and free it."""
    nv, ne = s.nv, s.ne
    v = np.ctypeslib.as_array(s.csc_v, shape=(nv + 1,)).copy()
    e = np.ctypeslib.as_array(s.csc_e, shape=(max(ne, 1),))[:ne].copy()
    ev = np.ctypeslib.as_array(s.csc_ev, shape=(max(ne, 1),))[:ne].copy()
    out = CSR(nv, ne, s.start_p, s.tra, v, e, ev)
    lib().orc_csr_free(C.byref(s))
    return out


def load_mtx(path: str, source: int = 0, flags: int = LOAD_SYM, seed: int = 1) -> CSR:
    s = _OrcCSR()
    rc = lib().orc_load_mtx(path.encode(), source, flags, seed, C.byref(s))
    if rc != 0:
        raise OSError(rc, f"oracle loader failed with status {rc} on {path}")
    return _take(s)


def from_entries(nv_decl: int, src, dst, val=None, source: int = 0, flags: int = LOAD_SYM) -> CSR:
    """The loader pipeline on an in-memory entry list (0-based, file order)."""
    src = np.ascontiguousarray(src, dtype=np.int32)
    dst = np.ascontiguousarray(dst, dtype=np.int32)
    vp = None
    if val is not None:
        val = np.ascontiguousarray(val, dtype=np.int32)
        vp = val.ctypes.data_as(C.c_void_p)
    s = _OrcCSR()
    rc = lib().orc_from_entries(nv_decl, len(src), src, dst, vp, source, flags, C.byref(s))
    if rc != 0:
        raise ValueError(f"oracle loader failed with status {rc}")
    return _take(s)


def gen_rmat(scale: int, edge_factor: int = 16, a=0.57, b=0.19, c=0.19, seed: int = 1, wmin: int = 1,
             wmax: int = 64) -> CSR:
    """Symmetrised, deduplicated R-MAT graph (the benchmarks' synthetic input)."""
    s = _OrcCSR()
    rc = lib().orc_gen_rmat(scale, edge_factor, a, b, c, seed, wmin, wmax, C.byref(s))
    if rc != 0:
        raise ValueError(f"oracle R-MAT generator failed with status {rc}")
    return _take(s)


def pattern_weight(seed: int, entry: int) -> int:
    return int(lib().orc_pattern_weight(seed, entry))


def bfs(g: CSR, src: int) -> np.ndarray:
    out = np.empty(g.nv, dtype=np.int32)
    lib().orc_bfs(g._struct(), src, out)
    return out


def sssp(g: CSR, src: int, max_sweeps: int = 0):
    out = np.empty(g.nv, dtype=np.int32)
    sweeps = lib().orc_sssp(g._struct(), src, out, max_sweeps)
    return out, sweeps


def bc(g: CSR, src: int):
    lv = np.empty(g.nv, dtype=np.int32)
    sg = np.empty(g.nv, dtype=np.int32)
    dl = np.empty(g.nv, dtype=np.float32)
    lib().orc_bc(g._struct(), src, lv, sg, dl)
    return lv, sg, dl


def bc_f64(g: CSR, src: int):
    lv = np.empty(g.nv, dtype=np.int32)
    sg = np.empty(g.nv, dtype=np.float64)
    dl = np.empty(g.nv, dtype=np.float64)
    lib().orc_bc_f64(g._struct(), src, lv, sg, dl)
    return lv, sg, dl


def bc_ext(g: CSR, src: int):
    """Brandes with long-double path counts: (levels, log2 path counts, deltas)."""
    lv = np.empty(g.nv, dtype=np.int32)
    ls = np.empty(g.nv, dtype=np.float64)
    dl = np.empty(g.nv, dtype=np.float64)
    lib().orc_bc_ext(g._struct(), src, lv, ls, dl)
    return lv, ls, dl


def bc_multi_ext(g: CSR, sources) -> np.ndarray:
    s = np.ascontiguousarray(sources, dtype=np.int32)
    out = np.empty(g.nv, dtype=np.float64)
    lib().orc_bc_multi_ext(g._struct(), s, len(s), out)
    return out


def bc_multi_f64(g: CSR, sources) -> np.ndarray:
    s = np.ascontiguousarray(sources, dtype=np.int32)
    out = np.empty(g.nv, dtype=np.float64)
    lib().orc_bc_multi_f64(g._struct(), s, len(s), out)
    return out


def cc_minlabel(g: CSR) -> np.ndarray:
    out = np.empty(g.nv, dtype=np.int32)
    lib().orc_cc_minlabel(g._struct(), out)
    return out


def cc_relabel(labels: np.ndarray) -> np.ndarray:
    out = np.ascontiguousarray(labels, dtype=np.int32).copy()
    lib().orc_cc_relabel(len(out), out)
    return out


def pr_ref(g: CSR, mode: int, max_iter: int = 0):
    out = np.empty(g.nv, dtype=np.float32)
    it = lib().orc_pr_ref(g._struct(), mode, out, max_iter)
    return out, it


def pr_ref_f64(g: CSR, mode: int, max_iter: int = 0):
    out = np.empty(g.nv, dtype=np.float64)
    it = lib().orc_pr_ref_f64(g._struct(), mode, out, max_iter)
    return out, it


def pr_norm_f64(g: CSR, damping=0.85, tol=1e-6, max_iter=0):
    out = np.empty(g.nv, dtype=np.float64)
    it = lib().orc_pr_norm_f64(g._struct(), damping, tol, max_iter, out)
    return out, it


def ppr_f64(g: CSR, seed: int, damping=0.85, tol=1e-6, max_iter=0):
    out = np.empty(g.nv, dtype=np.float64)
    it = lib().orc_ppr_f64(g._struct(), seed, damping, tol, max_iter, out)
    return out, it


def wpr_f64(g: CSR, w, damping=0.85, tol=1e-12, max_iter=0):
    w = np.ascontiguousarray(w, dtype=np.float64)
    out = np.empty(g.nv, dtype=np.float64)
    it = lib().orc_wpr_f64(g._struct(), w, damping, tol, max_iter, out)
    return out, it


def wpr_adjoint_f64(g: CSR, w, x, gvec, damping=0.85, tol=1e-12, max_iter=0):
    w = np.ascontiguousarray(w, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    gvec = np.ascontiguousarray(gvec, dtype=np.float64)
    lam = np.empty(g.nv, dtype=np.float64)
    gw = np.empty(g.ne, dtype=np.float64)
    gp = np.empty(g.ne, dtype=np.float64)
    it = lib().orc_wpr_adjoint_f64(g._struct(), w, x, gvec, damping, tol, max_iter, lam, gw, gp)
    return lam, gw, gp, it


def wpr_fd_f64(g: CSR, w, x, gvec, entries, damping=0.85, eps=1e-3, rtol=1e-10, max_iter=2000, nthreads=0):
    """Central differences (L(w+eps) - L(w-eps)) / (2 eps) for the listed CSR
    entries, every loss from a complete FP64 solve (x = wpr_f64's solution)."""
    w = np.ascontiguousarray(w, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    gvec = np.ascontiguousarray(gvec, dtype=np.float64)
    entries = np.ascontiguousarray(entries, dtype=np.int32)
    out = np.empty(len(entries), dtype=np.float64)
    nt = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    it = lib().orc_wpr_fd_f64(g._struct(), w, x, gvec, damping, entries, len(entries), eps, rtol, max_iter, nt, out)
    if it < 0:
        raise MemoryError("oracle finite differences: out of memory")
    return out, it


def wpr_loss_f64(g: CSR, w, gvec, damping=0.85, tol=1e-13, max_iter=0) -> float:
    w = np.ascontiguousarray(w, dtype=np.float64)
    gvec = np.ascontiguousarray(gvec, dtype=np.float64)
    return float(lib().orc_wpr_loss_f64(g._struct(), w, gvec, damping, tol, max_iter))


# ---------------------------------------------------------------------------
# the reference's own loader / validator, compiled into oracle/_ref/
# ---------------------------------------------------------------------------
class RefTool:
    """Runs oracle/_ref/ref_<ALG> (the reference's generate_CSC + verifyResults)."""

    def __init__(self, alg: str):
        self.path = os.path.join(REF_DIR, f"ref_{alg}")

    @staticmethod
    def available(alg: str = "BFS") -> bool:
        return os.access(os.path.join(REF_DIR, f"ref_{alg}"), os.X_OK)

    def load(self, mtx: str, source: int, tmpdir: str) -> CSR:
        out = os.path.join(tmpdir, "ref_load.bin")
        subprocess.check_call([self.path, "load", mtx, str(source), out])
        a = np.fromfile(out, dtype=np.int32)
        nv, ne, sp, tra, has_ev = (int(x) for x in a[:5])
        p = 5
        v = a[p:p + nv + 1].copy(); p += nv + 1
        e = a[p:p + ne].copy(); p += ne
        ev = a[p:p + ne].copy() if has_ev else np.ones(ne, dtype=np.int32)
        return CSR(nv, ne, sp, tra, v, e, ev)

    def validate(self, mtx: str, source: int, arrays, tmpdir: str) -> str:
        out = os.path.join(tmpdir, "ref_result.bin")
        with open(out, "wb") as f:
            for a in arrays:
                f.write(np.ascontiguousarray(a).tobytes())
        r = subprocess.run([self.path, "validate", mtx, str(source), out],
                           capture_output=True, text=True, check=True)
        return r.stdout.strip()
