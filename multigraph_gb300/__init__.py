"""multigraph_gb300 -- GB300 frontier-processing engine (Python mirror of the C ABI).

The engine is ``libmg.so`` (hand-written sm_103a CUDA kernels behind the C ABI
declared in ``include/mg.h``).  This module binds it with ctypes and mirrors
the reference's host interface:

    generate_CSC(path, source)        -> HostGraph   (read_input.cu:11)
    generate_MultiGraph(host_graph)   -> Graph       (gen_structure.cu:2230)
    release_MultiGraph(graph)                        (release_structure.cu:4)
    Graph.bfs / sssp / bc / cc / pagerank            (the per-algorithm loops of
                                                      main.cu over process*.cu)

plus the additions without a reference counterpart: multi-source BC, batched
personalised PageRank, weighted PageRank and its adjoint, multi-graph batches
and the autotuner.  There is no CPU fallback: every compute call goes through
libmg.so, and building the package without it raises ImportError.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libmg.so")
BIN_DIR = os.path.join(_PKG, "bin")

MG_OK, MG_ERR_IO, MG_ERR_PARSE, MG_ERR_RANGE, MG_ERR_OOM, MG_ERR_CUDA, MG_ERR_ITER_LIMIT, MG_ERR_INVALID, \
    MG_ERR_UNSUPPORTED, MG_ERR_INTERNAL = range(10)
LOAD_SYM, LOAD_NSYM, LOAD_CC = 1, 2, 4
EXEC_GRAPH, EXEC_HOST = 0, 1
DIR_AUTO, DIR_PUSH, DIR_PULL = 0, 1, 2
PR_TOPOLOGY_REF, PR_DATA_REF, PR_TOPOLOGY, PR_DATA = 0, 1, 2, 3
PR_LAYOUT_GATHER, PR_LAYOUT_SEGMENTED, PR_LAYOUT_AUTO = 0, 1, 2
ALGO_BFS, ALGO_SSSP, ALGO_BC, ALGO_CC, ALGO_PR = range(5)
IUNUSED = 0x64646464


class MGError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where}: {_status_name(status)} ({message})")
        self.status = status


class Opts(C.Structure):
    _fields_ = [("exec", C.c_int32), ("direction", C.c_int32), ("max_iter", C.c_int32), ("alpha", C.c_int32),
                ("beta", C.c_int32), ("damping", C.c_float), ("tol", C.c_float), ("profile", C.c_int32),
                ("pr_layout", C.c_int32), ("reserved", C.c_int32 * 7)]


_OPT_FIELDS = frozenset(name for name, _ in Opts._fields_ if name != "reserved")


class KernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_int32), ("total_ms", C.c_double)]


class RunInfo(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("pull_iterations", C.c_int32), ("device_ms", C.c_double),
                ("residual", C.c_double), ("edges_scanned", C.c_int64), ("nkernels", C.c_int32),
                ("kernels", KernelTime * 16)]

    def kernel_times(self):
        return {self.kernels[i].name.decode(): (self.kernels[i].launches, self.kernels[i].total_ms)
                for i in range(self.nkernels)}


class CsrView(C.Structure):
    _fields_ = [("nv", C.c_int32), ("ne", C.c_int32), ("start_p", C.c_int32), ("tra", C.c_int32),
                ("csc_v", C.POINTER(C.c_int32)), ("csc_e", C.POINTER(C.c_int32)),
                ("csc_ev", C.POINTER(C.c_int32))]


def _load_lib():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run `python -m multigraph_gb300.build` (nvcc, sm_103a)")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, u32, u64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint32, C.c_uint64, C.c_float
    P = C.POINTER
    sig = {
        "mg_status_string": ([i32], C.c_char_p),
        "mg_last_error": ([], C.c_char_p),
        "mg_version": ([], C.c_char_p),
        "mg_load_mtx": ([C.c_char_p, i32, u32, u64, i32, P(vp)], i32),
        "mg_host_graph_from_entries": ([i32, i64, vp, vp, vp, i32, u32, u64, i32, P(vp)], i32),
        "mg_host_graph_from_csr": ([i32, i32, vp, vp, vp, i32, P(vp)], i32),
        "mg_host_graph_view": ([vp, P(CsrView)], i32),
        "mg_host_graph_pin": ([vp], i32),
        "mg_host_graph_stage_bytes": ([vp], i64),
        "mg_host_graph_free": ([vp], None),
        "mg_write_mtx": ([vp, C.c_char_p, i32], i32),
        "mg_save_csr": ([vp, C.c_char_p], i32),
        "mg_load_csr": ([C.c_char_p, P(vp)], i32),
        "mg_gen_rmat": ([i32, i32, C.c_double, C.c_double, C.c_double, u64, i32, i32, i32, P(vp)], i32),
        "mg_gen_lattice": ([i32, i32, C.c_double, u64, P(vp)], i32),
        "mg_graph_upload": ([vp, i32, P(vp)], i32),
        "mg_graph_reload": ([vp, vp], i32),
        "mg_graph_stage": ([vp, vp], i32),
        "mg_graph_commit": ([vp], i32),
        "mg_graph_free": ([vp], None),
        "mg_graph_info": ([vp, P(i32), P(i32)], i32),
        "mg_graph_stream": ([vp], vp),
        "mg_graph_set_float_weights": ([vp, vp], i32),
        "mg_opts_default": ([P(Opts)], None),
        "mg_result_device": ([vp, i32], vp),
        "mg_bfs": ([vp, i32, P(Opts), vp, P(RunInfo)], i32),
        "mg_sssp": ([vp, i32, P(Opts), vp, P(RunInfo)], i32),
        "mg_cc": ([vp, P(Opts), vp, P(RunInfo)], i32),
        "mg_bc": ([vp, i32, P(Opts), vp, vp, vp, P(RunInfo)], i32),
        "mg_bc_multi": ([vp, vp, i32, P(Opts), vp, P(RunInfo)], i32),
        "mg_pagerank": ([vp, i32, P(Opts), vp, P(RunInfo)], i32),
        "mg_ppr_batch": ([vp, vp, i32, P(Opts), vp, P(RunInfo)], i32),
        "mg_wpagerank": ([vp, P(Opts), vp, P(RunInfo)], i32),
        "mg_wpagerank_backward": ([vp, vp, P(Opts), vp, vp, P(RunInfo)], i32),
        "mg_batch_create": ([vp, i32, i32, P(vp)], i32),
        "mg_batch_free": ([vp], None),
        "mg_batch_bfs": ([vp, vp, P(Opts), vp, P(RunInfo)], i32),
        "mg_batch_cc": ([vp, P(Opts), vp, P(RunInfo)], i32),
        "mg_autotune": ([vp, i32, i32, C.c_char_p, P(Opts)], i32),
        "mg_pagerank_noalloc": ([vp, vp, i32, i32, f32, f32, i32, vp, vp, P(i32), P(C.c_double)], i32),
        "mg_selftest_segmented_layout": ([i32, i64, vp, vp, i32, P(i64)], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    return L


class _LazyLib:
    """libmg.so, loaded on first use (so the build module imports without it)."""
    _L = None

    def __getattr__(self, name):
        if _LazyLib._L is None:
            _LazyLib._L = _load_lib()
        return getattr(_LazyLib._L, name)


lib = _LazyLib()

# every symbol include/mg.h declares, in declaration order
EXPORTED = [
    "mg_status_string", "mg_last_error", "mg_version", "mg_load_mtx", "mg_host_graph_from_entries",
    "mg_host_graph_from_csr", "mg_host_graph_view", "mg_host_graph_pin", "mg_host_graph_stage_bytes",
    "mg_host_graph_free", "mg_write_mtx",
    "mg_save_csr", "mg_load_csr",
    "mg_gen_rmat", "mg_gen_lattice", "mg_graph_upload", "mg_graph_reload", "mg_graph_stage", "mg_graph_commit",
    "mg_graph_free", "mg_graph_info",
    "mg_graph_stream", "mg_graph_set_float_weights", "mg_opts_default", "mg_result_device", "mg_bfs", "mg_sssp",
    "mg_cc", "mg_bc", "mg_bc_multi", "mg_pagerank", "mg_ppr_batch", "mg_wpagerank", "mg_wpagerank_backward",
    "mg_batch_create", "mg_batch_free", "mg_batch_bfs", "mg_batch_cc", "mg_autotune", "mg_pagerank_noalloc",
    "mg_selftest_segmented_layout",
]
NOALLOC_MAX_VERTICES = 1 << 20


def pagerank_noalloc(d_row: int, d_col: int, nv: int, ne: int, d_rank: int, stream: int = 0,
                     damping: float = 0.85, tol: float = 1e-6, max_iter: int = 0):
    """mg_pagerank_noalloc on caller-owned device buffers (raw device pointers).

    For callers that cannot allocate device memory: libmg uses only a fixed
    internal device array (up to NOALLOC_MAX_VERTICES vertices).  Returns
    (iterations, residual)."""
    it = C.c_int32(0)
    res = C.c_double(0.0)
    _check(lib.mg_pagerank_noalloc(C.c_void_p(d_row), C.c_void_p(d_col), nv, ne, damping, tol, max_iter,
                                   C.c_void_p(d_rank), C.c_void_p(stream) if stream else None, C.byref(it),
                                   C.byref(res)), "mg_pagerank_noalloc")
    return it.value, res.value


def selftest_segmented_layout(row_ptr, col, threads: int = 4) -> int:
    """Host-only check of PageRank's segmented layout built from a CSR
    (mg_selftest_segmented_layout); returns the number of pieces, raises
    MGError on a violation."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    pieces = C.c_int64(0)
    _check(lib.mg_selftest_segmented_layout(len(rp) - 1, len(cl), rp.ctypes.data, cl.ctypes.data if len(cl) else None,
                                            threads, C.byref(pieces)), "mg_selftest_segmented_layout")
    return pieces.value


def _status_name(s: int) -> str:
    return lib.mg_status_string(s).decode()


def _check(status: int, where: str):
    if status != MG_OK:
        raise MGError(status, where, lib.mg_last_error().decode())


def _result(out, shape, dtype) -> Optional[np.ndarray]:
    """Host buffer for a run's result: `out` itself when it is an array of
    that shape and type (C-contiguous, writable: a caller reusing buffers,
    or page-locked ones, across runs), a new array when `out` is true,
    nothing (result left on the device) when it is false."""
    if isinstance(out, np.ndarray):
        if out.shape != tuple(shape) or out.dtype != np.dtype(dtype) or not out.flags.c_contiguous \
                or not out.flags.writeable:
            raise ValueError(f"out must be a writable C-contiguous {np.dtype(dtype)} array of shape {tuple(shape)}")
        return out
    return np.empty(shape, dtype) if out else None


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def version() -> str:
    return lib.mg_version().decode()


def default_opts(**kw) -> Opts:
    o = Opts()
    lib.mg_opts_default(C.byref(o))
    for k, v in kw.items():
        if k not in _OPT_FIELDS:
            raise TypeError(f"unknown mg_opts field {k!r}")
        setattr(o, k, v)
    return o


# ---------------------------------------------------------------------------
class HostGraph:
    """Host CSR owned by libmg (the reference's struct csc_package)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle

    @classmethod
    def load_mtx(cls, path: str, source: int = 0, flags: int = LOAD_SYM, weight_seed: int = 1,
                 nthreads: int = 0) -> "HostGraph":
        h = C.c_void_p()
        _check(lib.mg_load_mtx(path.encode(), source, flags, weight_seed, nthreads, C.byref(h)), "mg_load_mtx")
        return cls(h)

    @classmethod
    def from_entries(cls, nv_decl: int, src, dst, val=None, source: int = 0, flags: int = LOAD_SYM,
                     weight_seed: int = 1, nthreads: int = 0) -> "HostGraph":
        src = np.ascontiguousarray(src, dtype=np.int32)
        dst = np.ascontiguousarray(dst, dtype=np.int32)
        val = None if val is None else np.ascontiguousarray(val, dtype=np.int32)
        h = C.c_void_p()
        _check(lib.mg_host_graph_from_entries(nv_decl, len(src), _ptr(src), _ptr(dst), _ptr(val), source, flags,
                                              weight_seed, nthreads, C.byref(h)), "mg_host_graph_from_entries")
        return cls(h)

    @classmethod
    def from_csr(cls, row_ptr, col, wt=None, start_p: int = 0) -> "HostGraph":
        row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int32)
        col = np.ascontiguousarray(col, dtype=np.int32)
        wt = None if wt is None else np.ascontiguousarray(wt, dtype=np.int32)
        h = C.c_void_p()
        _check(lib.mg_host_graph_from_csr(len(row_ptr) - 1, len(col), _ptr(row_ptr), _ptr(col), _ptr(wt), start_p,
                                          C.byref(h)), "mg_host_graph_from_csr")
        return cls(h)

    @classmethod
    def rmat(cls, scale: int, edge_factor: int = 16, a=0.57, b=0.19, c=0.19, seed: int = 1, wmin: int = 1,
             wmax: int = 64, nthreads: int = 0) -> "HostGraph":
        h = C.c_void_p()
        _check(lib.mg_gen_rmat(scale, edge_factor, a, b, c, seed, wmin, wmax, nthreads, C.byref(h)), "mg_gen_rmat")
        return cls(h)

    @classmethod
    def lattice(cls, rows: int, cols: int, shortcut_frac: float = 0.05, seed: int = 1) -> "HostGraph":
        h = C.c_void_p()
        _check(lib.mg_gen_lattice(rows, cols, shortcut_frac, seed, C.byref(h)), "mg_gen_lattice")
        return cls(h)

    def view(self) -> CsrView:
        v = CsrView()
        _check(lib.mg_host_graph_view(self._h, C.byref(v)), "mg_host_graph_view")
        return v

    @property
    def nv(self) -> int:
        return self.view().nv

    @property
    def ne(self) -> int:
        return self.view().ne

    @property
    def start_p(self) -> int:
        return self.view().start_p

    def arrays(self):
        """(csc_v, csc_e, csc_ev) as numpy copies."""
        v = self.view()
        rp = np.ctypeslib.as_array(v.csc_v, shape=(v.nv + 1,)).copy()
        if v.ne:
            col = np.ctypeslib.as_array(v.csc_e, shape=(v.ne,)).copy()
            wt = np.ctypeslib.as_array(v.csc_ev, shape=(v.ne,)).copy()
        else:
            col = np.zeros(0, np.int32)
            wt = np.zeros(0, np.int32)
        return rp, col, wt

    def pin(self):
        _check(lib.mg_host_graph_pin(self._h), "mg_host_graph_pin")

    def stage_bytes(self) -> int:
        """Bytes Graph.stage copies to the device for this graph."""
        return int(lib.mg_host_graph_stage_bytes(self._h))

    def write_mtx(self, path: str, with_weights: bool = True):
        _check(lib.mg_write_mtx(self._h, path.encode(), int(with_weights)), "mg_write_mtx")

    def save_csr(self, path: str):
        """Binary CSR cache (mg_save_csr)."""
        _check(lib.mg_save_csr(self._h, path.encode()), "mg_save_csr")

    @classmethod
    def load_csr(cls, path: str) -> "HostGraph":
        h = C.c_void_p()
        _check(lib.mg_load_csr(path.encode(), C.byref(h)), "mg_load_csr")
        return cls(h)

    def free(self):
        if self._h:
            lib.mg_host_graph_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Graph:
    """Device-resident graph + engines (the reference's struct HYB)."""

    def __init__(self, host: HostGraph, device: int = 0):
        h = C.c_void_p()
        _check(lib.mg_graph_upload(host._h, device, C.byref(h)), "mg_graph_upload")
        self._h = h
        nv, ne = C.c_int32(), C.c_int32()
        lib.mg_graph_info(h, C.byref(nv), C.byref(ne))
        self.nv, self.ne = nv.value, ne.value

    def reload(self, host: HostGraph):
        _check(lib.mg_graph_reload(self._h, host._h), "mg_graph_reload")

    def stage(self, host: HostGraph):
        """Start copying `host` into the staging buffers (overlaps running work);
        keep `host` alive until commit()."""
        self._staged = host
        _check(lib.mg_graph_stage(self._h, host._h), "mg_graph_stage")

    def commit(self):
        """Rebuild the device CSR from the staged copy (after the runs before it)."""
        _check(lib.mg_graph_commit(self._h), "mg_graph_commit")
        self._staged = None

    def stream(self) -> int:
        return lib.mg_graph_stream(self._h) or 0

    def set_float_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert len(w) == self.ne
        _check(lib.mg_graph_set_float_weights(self._h, _ptr(w)), "mg_graph_set_float_weights")

    @staticmethod
    def _opts(opts, kw):
        o = opts if opts is not None else default_opts()
        for k, v in kw.items():
            if k not in _OPT_FIELDS:
                raise TypeError(f"unknown mg_opts field {k!r}")
            setattr(o, k, v)
        return o

    def bfs(self, source: int, opts: Opts = None, out: bool = True, **kw):
        o = self._opts(opts, kw)
        info = RunInfo()
        res = _result(out, (self.nv,), np.int32)
        _check(lib.mg_bfs(self._h, source, C.byref(o), _ptr(res), C.byref(info)), "mg_bfs")
        return res, info

    def sssp(self, source: int, opts: Opts = None, out: bool = True, **kw):
        o = self._opts(opts, kw)
        info = RunInfo()
        res = _result(out, (self.nv,), np.int32)
        _check(lib.mg_sssp(self._h, source, C.byref(o), _ptr(res), C.byref(info)), "mg_sssp")
        return res, info

    def cc(self, opts: Opts = None, out: bool = True, **kw):
        o = self._opts(opts, kw)
        info = RunInfo()
        res = _result(out, (self.nv,), np.int32)
        _check(lib.mg_cc(self._h, C.byref(o), _ptr(res), C.byref(info)), "mg_cc")
        return res, info

    def bc(self, source: int, opts: Opts = None, out: bool = True, **kw):
        o = self._opts(opts, kw)
        info = RunInfo()
        lv = np.empty(self.nv, np.int32) if out else None
        sg = np.empty(self.nv, np.float64) if out else None
        dl = np.empty(self.nv, np.float32) if out else None
        _check(lib.mg_bc(self._h, source, C.byref(o), _ptr(lv), _ptr(sg), _ptr(dl), C.byref(info)), "mg_bc")
        return (lv, sg, dl), info

    def bc_multi(self, sources: Sequence[int], opts: Opts = None, out: bool = True, **kw):
        o = self._opts(opts, kw)
        info = RunInfo()
        s = np.ascontiguousarray(sources, dtype=np.int32)
        res = _result(out, (self.nv,), np.float32)
        _check(lib.mg_bc_multi(self._h, _ptr(s), len(s), C.byref(o), _ptr(res), C.byref(info)), "mg_bc_multi")
        return res, info

    def pagerank(self, variant: int = PR_TOPOLOGY, opts: Opts = None, out: bool = True, **kw):
        o = self._opts(opts, kw)
        info = RunInfo()
        res = _result(out, (self.nv,), np.float32)
        _check(lib.mg_pagerank(self._h, variant, C.byref(o), _ptr(res), C.byref(info)), "mg_pagerank")
        return res, info

    def ppr_batch(self, seeds: Sequence[int], opts: Opts = None, out: bool = True, **kw):
        o = self._opts(opts, kw)
        info = RunInfo()
        s = np.ascontiguousarray(seeds, dtype=np.int32)
        res = _result(out, (len(s), self.nv), np.float32)
        _check(lib.mg_ppr_batch(self._h, _ptr(s), len(s), C.byref(o), _ptr(res), C.byref(info)), "mg_ppr_batch")
        return res, info

    def wpagerank(self, opts: Opts = None, out: bool = True, **kw):
        o = self._opts(opts, kw)
        info = RunInfo()
        res = _result(out, (self.nv,), np.float32)
        _check(lib.mg_wpagerank(self._h, C.byref(o), _ptr(res), C.byref(info)), "mg_wpagerank")
        return res, info

    def wpagerank_backward(self, gvec, opts: Opts = None, out: bool = True, **kw):
        o = self._opts(opts, kw)
        info = RunInfo()
        gv = np.ascontiguousarray(gvec, dtype=np.float32)
        grad = np.empty(self.ne, np.float32) if out else None
        lam = np.empty(self.nv, np.float32) if out else None
        _check(lib.mg_wpagerank_backward(self._h, _ptr(gv), C.byref(o), _ptr(grad), _ptr(lam), C.byref(info)),
               "mg_wpagerank_backward")
        return (grad, lam), info

    def autotune(self, algo: int, source: int = 0, cache_path: Optional[str] = None, opts: Opts = None) -> Opts:
        o = opts if opts is not None else default_opts()
        _check(lib.mg_autotune(self._h, algo, source, cache_path.encode() if cache_path else None, C.byref(o)),
               "mg_autotune")
        return o

    def free(self):
        if self._h:
            lib.mg_graph_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Batch:
    """Many graphs in one CSR arena; one launch sequence per algorithm for all."""

    def __init__(self, graphs: Sequence[HostGraph], device: int = 0):
        arr = (C.c_void_p * len(graphs))(*[g._h.value for g in graphs])
        h = C.c_void_p()
        _check(lib.mg_batch_create(arr, len(graphs), device, C.byref(h)), "mg_batch_create")
        self._h = h
        self.nvs = [g.nv for g in graphs]
        self.offsets = np.concatenate([[0], np.cumsum(self.nvs)]).astype(np.int64)

    def bfs(self, sources: Sequence[int], opts: Opts = None, **kw):
        o = Graph._opts(opts, kw)
        info = RunInfo()
        s = np.ascontiguousarray(sources, dtype=np.int32)
        res = np.empty(int(self.offsets[-1]), np.int32)
        _check(lib.mg_batch_bfs(self._h, _ptr(s), C.byref(o), _ptr(res), C.byref(info)), "mg_batch_bfs")
        return [res[self.offsets[i]:self.offsets[i + 1]] for i in range(len(self.nvs))], info

    def cc(self, opts: Opts = None, **kw):
        o = Graph._opts(opts, kw)
        info = RunInfo()
        res = np.empty(int(self.offsets[-1]), np.int32)
        _check(lib.mg_batch_cc(self._h, C.byref(o), _ptr(res), C.byref(info)), "mg_batch_cc")
        return [res[self.offsets[i]:self.offsets[i + 1]] for i in range(len(self.nvs))], info

    def free(self):
        if self._h:
            lib.mg_batch_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# --- the reference's host interface names -----------------------------------
def generate_CSC(path: str, source: int = 0, flags: int = LOAD_SYM, weight_seed: int = 1) -> HostGraph:
    """read_input.cu:11 -- MTX -> deduplicated, compacted CSR."""
    return HostGraph.load_mtx(path, source, flags, weight_seed)


def generate_MultiGraph(host: HostGraph, device: int = 0) -> Graph:
    """gen_structure.cu:2230 -- device layouts for the engines."""
    return Graph(host, device)


def release_MultiGraph(graph: Graph) -> None:
    """release_structure.cu:4."""
    graph.free()
