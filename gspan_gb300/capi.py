"""ctypes view of the C ABI in ``include/gspan_gb300.h``.

The mining itself runs in ``_lib/libgspan_gb300.so`` (CUDA, sm_103a); there is
no CPU fallback.  Importing this module loads the library and fails loudly if it
has not been built (``python -m gspan_gb300.build``).  The package's top level
(``gspan_gb300.Miner`` and the rest) imports this module on first use.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Iterable, Sequence

import numpy as np

from .datagen import CSR, load_bin  # noqa: F401  (re-exported)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgspan_gb300.so")
BIN_DIR = os.path.join(_HERE, "_lib")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"gspan_gb300: native library missing at {LIB_PATH}; build it with `python -m gspan_gb300.build` "
        "(there is no CPU fallback)")

_lib = ctypes.CDLL(LIB_PATH)

GSPAN_OK = 0
GSPAN_ERR_INVALID = 1
GSPAN_ERR_NOMEM = 3
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "LIMIT", 5: "DEVICE", 6: "ABORTED",
                7: "NO_DEVICE"}


class GspanError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        msg = f"{what}: {STATUS_NAMES.get(status, status)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


class Opts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("domain_mode", ctypes.c_int32),
                ("hash_threshold", ctypes.c_double), ("mem_fraction", ctypes.c_double),
                ("profile", ctypes.c_int32), ("path", ctypes.c_int32), ("mask_bias", ctypes.c_double),
                ("prune", ctypes.c_int32), ("fused_last", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [("seeds", ctypes.c_uint64), ("extended", ctypes.c_uint64), ("patterns", ctypes.c_uint64),
                ("support_keys", ctypes.c_uint64), ("hash_domains", ctypes.c_uint64),
                ("scanned_entries", ctypes.c_uint64), ("materialized_rows", ctypes.c_uint64),
                ("kernel_launches", ctypes.c_uint64), ("levels", ctypes.c_int32), ("mine_ms", ctypes.c_double),
                ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
                ("frontier_rows", ctypes.c_uint64),
                ("mask_parents", ctypes.c_uint64), ("candidate_parents", ctypes.c_uint64),
                ("expand_ms", ctypes.c_double), ("expand_launches", ctypes.c_uint64),
                ("expand_bytes", ctypes.c_double),
                ("rows_ms", ctypes.c_double), ("rows_launches", ctypes.c_uint64), ("rows_bytes", ctypes.c_double),
                ("sweep_ms", ctypes.c_double), ("sweep_bytes", ctypes.c_double),
                ("materialize_ms", ctypes.c_double), ("materialize_launches", ctypes.c_uint64),
                ("materialize_bytes", ctypes.c_double),
                ("seed_ms", ctypes.c_double), ("domain_ms", ctypes.c_double),
                ("canonical_checks", ctypes.c_uint64), ("canonical_ms", ctypes.c_double),
                ("pruned_vertices", ctypes.c_uint64), ("pruned_entries", ctypes.c_uint64),
                ("fused_rows", ctypes.c_uint64), ("sync_ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class PatternEdge(ctypes.Structure):
    _fields_ = [("frm", ctypes.c_int32), ("to", ctypes.c_int32), ("from_label", ctypes.c_int32),
                ("edge_label", ctypes.c_int32), ("to_label", ctypes.c_int32)]


EMIT_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(PatternEdge), ctypes.c_int32,
                           ctypes.c_int32)

_i32p = ctypes.POINTER(ctypes.c_int32)
_lib.gspan_opts_default.argtypes = [ctypes.POINTER(Opts)]
_lib.gspan_opts_default.restype = None
_lib.gspan_ctx_create.argtypes = [ctypes.POINTER(Opts), ctypes.POINTER(ctypes.c_void_p)]
_lib.gspan_ctx_create.restype = ctypes.c_int
_lib.gspan_ctx_destroy.argtypes = [ctypes.c_void_p]
_lib.gspan_ctx_destroy.restype = None
_lib.gspan_graph_upload.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
_lib.gspan_graph_upload.restype = ctypes.c_int
_lib.gspan_graph_free.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
_lib.gspan_graph_free.restype = ctypes.c_int
_lib.gspan_mine.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, EMIT_FN,
                            ctypes.c_void_p, ctypes.POINTER(Stats)]
_lib.gspan_mine.restype = ctypes.c_int
BATCH_EMIT_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(PatternEdge),
                                 ctypes.c_int32, ctypes.c_int32)
_lib.gspan_batch_upload.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.POINTER(ctypes.c_void_p)]
_lib.gspan_batch_upload.restype = ctypes.c_int
_lib.gspan_mine_batch.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                  BATCH_EMIT_FN, ctypes.c_void_p, ctypes.POINTER(Stats)]
_lib.gspan_mine_batch.restype = ctypes.c_int
_lib.gspan_graph_instances.argtypes = [ctypes.c_void_p]
_lib.gspan_graph_instances.restype = ctypes.c_int32
class JobInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("queued_ms", ctypes.c_double), ("run_ms", ctypes.c_double),
                ("latency_ms", ctypes.c_double), ("predicted_bytes", ctypes.c_double),
                ("retried_alone", ctypes.c_int32), ("stats", Stats)]


_lib.gspan_server_create.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.POINTER(ctypes.c_void_p)]
_lib.gspan_server_create.restype = ctypes.c_int
_lib.gspan_server_destroy.argtypes = [ctypes.c_void_p]
_lib.gspan_server_destroy.restype = None
_lib.gspan_server_add_graph.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]
_lib.gspan_server_add_graph.restype = ctypes.c_int
_lib.gspan_server_submit.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                     ctypes.POINTER(ctypes.c_int64)]
_lib.gspan_server_submit.restype = ctypes.c_int
_lib.gspan_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_int64, EMIT_FN, ctypes.c_void_p,
                                   ctypes.POINTER(JobInfo)]
_lib.gspan_server_wait.restype = ctypes.c_int
_lib.gspan_results_create.argtypes = []
_lib.gspan_results_create.restype = ctypes.c_void_p
_lib.gspan_results_destroy.argtypes = [ctypes.c_void_p]
_lib.gspan_results_destroy.restype = None
_lib.gspan_results_clear.argtypes = [ctypes.c_void_p]
_lib.gspan_results_clear.restype = None
_lib.gspan_results_patterns.argtypes = [ctypes.c_void_p]
_lib.gspan_results_patterns.restype = ctypes.c_int64
_lib.gspan_results_data.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]
_lib.gspan_results_data.restype = ctypes.POINTER(ctypes.c_int32)
# The collector's emit functions, passed to the miner as plain C pointers.
_RESULTS_EMIT = ctypes.cast(_lib.gspan_results_emit, EMIT_FN)
_RESULTS_BATCH_EMIT = ctypes.cast(_lib.gspan_results_batch_emit, BATCH_EMIT_FN)


class _Collector:
    """gspan_results: a run's patterns in one flat int32 buffer."""

    def __init__(self):
        self.h = _lib.gspan_results_create()
        if not self.h:
            raise MemoryError("gspan_results_create")

    def array(self) -> np.ndarray:
        n = ctypes.c_int64()
        ptr = _lib.gspan_results_data(self.h, ctypes.byref(n))
        if n.value == 0:
            return np.zeros(0, dtype=np.int32)
        return np.ctypeslib.as_array(ptr, shape=(n.value,)).copy()

    def close(self):
        if self.h:
            _lib.gspan_results_destroy(self.h)
            self.h = None


def decode_results(flat: np.ndarray, ninst: int = 1) -> list:
    """Flat collector words -> per instance [(code, support)], code a tuple
    of (from, to, from_label, edge_label, to_label) tuples."""
    out: list = [[] for _ in range(ninst)]
    words = flat.tolist()
    i, n = 0, len(words)
    while i < n:
        inst, length, sup = words[i], words[i + 1], words[i + 2]
        j = i + 3
        code = tuple(tuple(words[j + 5 * q: j + 5 * q + 5]) for q in range(length))
        out[inst].append((code, sup))
        i = j + 5 * length
    return out


_lib.gspan_graph_upload_text.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p),
                                         ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
_lib.gspan_graph_upload_text.restype = ctypes.c_int
_lib.gspan_autotune.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(Opts), ctypes.POINTER(ctypes.c_double)]
_lib.gspan_autotune.restype = ctypes.c_int
_lib.gspan_table_support.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p),
                                     ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p]
_lib.gspan_table_support.restype = ctypes.c_int
_lib.gspan_table_support_noalloc.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32,
                                             ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
_lib.gspan_table_support_noalloc.restype = ctypes.c_int
_lib.gspan_is_canonical.argtypes = [ctypes.POINTER(PatternEdge), ctypes.c_int32, _i32p]
_lib.gspan_is_canonical.restype = ctypes.c_int
_lib.gspan_status_string.argtypes = [ctypes.c_int]
_lib.gspan_status_string.restype = ctypes.c_char_p
_lib.gspan_last_error.argtypes = [ctypes.c_void_p]
_lib.gspan_last_error.restype = ctypes.c_char_p
_lib.gspan_max_pattern_edges.argtypes = []
_lib.gspan_max_pattern_edges.restype = ctypes.c_int32

# Every symbol include/gspan_gb300.h declares (checked by the tests).
ABI_SYMBOLS = ("gspan_opts_default", "gspan_ctx_create", "gspan_ctx_destroy", "gspan_graph_upload",
               "gspan_graph_free", "gspan_mine", "gspan_batch_upload", "gspan_mine_batch", "gspan_graph_instances",
               "gspan_table_support", "gspan_table_support_noalloc",
               "gspan_server_create", "gspan_server_destroy", "gspan_server_add_graph", "gspan_server_submit",
               "gspan_server_wait", "gspan_autotune", "gspan_graph_upload_text", "gspan_results_create", "gspan_results_destroy",
               "gspan_results_clear", "gspan_results_emit", "gspan_results_batch_emit", "gspan_results_patterns",
               "gspan_results_data", "gspan_is_canonical",
               "gspan_status_string", "gspan_last_error", "gspan_max_pattern_edges")

Code = tuple  # tuple of (from, to, from_label, edge_label, to_label)


def max_pattern_edges() -> int:
    return int(_lib.gspan_max_pattern_edges())


def is_canonical(code: Sequence[Sequence[int]]) -> bool:
    """The reference's minimum-DFS-code test (gspan.cu:586-606), host side."""
    arr = (PatternEdge * len(code))(*[PatternEdge(*map(int, e)) for e in code])
    out = ctypes.c_int32(0)
    rc = _lib.gspan_is_canonical(arr, len(code), ctypes.byref(out))
    if rc != GSPAN_OK:
        raise GspanError(rc, "gspan_is_canonical")
    return bool(out.value)


def format_pattern(code: Iterable[Sequence[int]], support: int) -> str:
    """One output line in the reference's format (gspan.cu:67-77)."""
    return "".join(f"({a} {b} {c} {d} {e})" for a, b, c, d, e in code) + f": {support}"


@dataclass
class DeviceGraph:
    handle: ctypes.c_void_p
    n: int
    m: int


class Miner:
    """One mining context on one GPU (a CUDA stream and the device memory it owns)."""

    def __init__(self, device: int = 0, domain_mode: int = 0, hash_threshold: float = 1.0,
                 profile: bool = False, mem_fraction: float = 0.85, path: int = 0, mask_bias: float = 1.0,
                 prune: bool = False, fused_last: int = 0):
        opts = Opts()
        _lib.gspan_opts_default(ctypes.byref(opts))
        opts.device = device
        opts.domain_mode = domain_mode
        opts.hash_threshold = hash_threshold
        opts.profile = 1 if profile else 0
        opts.mem_fraction = mem_fraction
        opts.path = path
        opts.mask_bias = mask_bias
        opts.prune = 1 if prune else 0
        opts.fused_last = fused_last
        self._ctx = ctypes.c_void_p()
        rc = _lib.gspan_ctx_create(ctypes.byref(opts), ctypes.byref(self._ctx))
        if rc != GSPAN_OK:
            raise GspanError(rc, "gspan_ctx_create")
        self._graphs: list[DeviceGraph] = []

    def _err(self, rc: int, what: str) -> GspanError:
        detail = _lib.gspan_last_error(self._ctx) if self._ctx else b""
        return GspanError(rc, what, (detail or b"").decode())

    def upload(self, g: CSR) -> DeviceGraph:
        off = np.ascontiguousarray(g.offsets, dtype=np.int32)
        vl = np.ascontiguousarray(g.vlabels, dtype=np.int32)
        ed = np.ascontiguousarray(g.edges, dtype=np.int32).reshape(-1, 3)
        return self.upload_arrays(off, vl, ed)

    def upload_arrays(self, offsets, vlabels, edges) -> DeviceGraph:
        """Host arrays (numpy, or anything exposing a contiguous int32 buffer
        through ``.ctypes.data`` or ``.data_ptr()``) in the reference's CSR layout."""
        def ptr(a):
            return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data
        n = int(vlabels.shape[0])
        m = int(edges.shape[0])
        h = ctypes.c_void_p()
        rc = _lib.gspan_graph_upload(self._ctx, n, m, ptr(offsets), ptr(vlabels) if n else None,
                                     ptr(edges) if m else None, ctypes.byref(h))
        if rc != GSPAN_OK:
            raise self._err(rc, "gspan_graph_upload")
        dg = DeviceGraph(h, n, m)
        self._graphs.append(dg)
        return dg

    def upload_text(self, text) -> DeviceGraph:
        """Builds the device store from gSpan text (bytes or str, the
        contents of a file that `convert` reads), parsed on the GPU."""
        if isinstance(text, str):
            text = text.encode()
        buf = ctypes.create_string_buffer(bytes(text), len(text)) if text else None
        h = ctypes.c_void_p()
        n = ctypes.c_int32()
        m = ctypes.c_int32()
        rc = _lib.gspan_graph_upload_text(self._ctx, buf, len(text), ctypes.byref(h), ctypes.byref(n), ctypes.byref(m))
        if rc != GSPAN_OK:
            raise self._err(rc, "gspan_graph_upload_text")
        dg = DeviceGraph(h, n.value, m.value)
        self._graphs.append(dg)
        return dg

    def free(self, dg: DeviceGraph) -> None:
        if dg in self._graphs:
            self._graphs.remove(dg)
            rc = _lib.gspan_graph_free(self._ctx, dg.handle)
            if rc != GSPAN_OK:
                raise self._err(rc, "gspan_graph_free")

    def mine(self, dg: DeviceGraph, k: int, min_support: int, raw: bool = False):
        """Returns (patterns, stats): patterns as [(code, support)] in the
        reference's pre-order, code a tuple of 5-tuples; raw=True returns the
        collector's flat int32 words instead (decode_results)."""
        col = _Collector()
        try:
            st = Stats()
            rc = _lib.gspan_mine(self._ctx, dg.handle, int(k), int(min_support), _RESULTS_EMIT, col.h,
                                 ctypes.byref(st))
            if rc != GSPAN_OK:
                raise self._err(rc, "gspan_mine")
            flat = col.array()
        finally:
            col.close()
        return (flat if raw else decode_results(flat, 1)[0]), st.as_dict()

    def upload_batch(self, graphs) -> DeviceGraph:
        """Uploads many independent graphs as one batch (gspan_batch_upload)."""
        arrs = [(np.ascontiguousarray(g.offsets, dtype=np.int32), np.ascontiguousarray(g.vlabels, dtype=np.int32),
                 np.ascontiguousarray(g.edges, dtype=np.int32).reshape(-1, 3)) for g in graphs]
        k = len(arrs)
        ns = np.array([a[1].shape[0] for a in arrs], dtype=np.int32)
        ms = np.array([a[2].shape[0] for a in arrs], dtype=np.int32)
        offs = (ctypes.c_void_p * k)(*[a[0].ctypes.data for a in arrs])
        vls = (ctypes.c_void_p * k)(*[a[1].ctypes.data if a[1].size else None for a in arrs])
        eds = (ctypes.c_void_p * k)(*[a[2].ctypes.data if a[2].size else None for a in arrs])
        h = ctypes.c_void_p()
        rc = _lib.gspan_batch_upload(self._ctx, k, ns.ctypes.data, ms.ctypes.data, offs, vls, eds, ctypes.byref(h))
        if rc != GSPAN_OK:
            raise self._err(rc, "gspan_batch_upload")
        dg = DeviceGraph(h, int(ns.sum()), int(ms.sum()))
        self._graphs.append(dg)
        return dg

    def mine_batch(self, dg: DeviceGraph, k: int, min_supports, raw: bool = False):
        """Returns (per-instance pattern lists, stats); each list as mine().
        raw=True returns the collector's flat words (decode_results)."""
        ninst = int(_lib.gspan_graph_instances(dg.handle))
        sups = np.ascontiguousarray(min_supports, dtype=np.int32)
        if sups.shape[0] != ninst:
            raise ValueError("one min_support per instance")
        col = _Collector()
        try:
            st = Stats()
            rc = _lib.gspan_mine_batch(self._ctx, dg.handle, int(k), sups.ctypes.data, _RESULTS_BATCH_EMIT, col.h,
                                       ctypes.byref(st))
            if rc != GSPAN_OK:
                raise self._err(rc, "gspan_mine_batch")
            flat = col.array()
        finally:
            col.close()
        return (flat if raw else decode_results(flat, ninst)), st.as_dict()

    TUNABLES = ("domain_mode", "hash_threshold", "mem_fraction", "path", "mask_bias", "fused_last")

    def autotune(self, dg: DeviceGraph, k: int, min_supports, candidates=None, ncand: int = 6, repeats: int = 2):
        """Times the job under each option set (dicts of TUNABLES; None: the
        built-in grid) and returns (the fastest set as Miner keyword arguments,
        median milliseconds per set).  Every set must give identical results."""
        ninst = int(_lib.gspan_graph_instances(dg.handle))
        sups = np.ascontiguousarray(np.atleast_1d(min_supports), dtype=np.int32)
        if sups.shape[0] != ninst:
            raise ValueError("one min_support per instance")
        cand_arr = None
        if candidates is not None:
            ncand = len(candidates)
            cand_arr = (Opts * ncand)()
            for o, c in zip(cand_arr, candidates):
                _lib.gspan_opts_default(ctypes.byref(o))
                for key, val in c.items():
                    if key not in self.TUNABLES:
                        raise ValueError(f"not a tunable: {key}")
                    setattr(o, key, val)
        best = Opts()
        ms = (ctypes.c_double * max(ncand, 1))()
        rc = _lib.gspan_autotune(self._ctx, dg.handle, int(k), sups.ctypes.data, cand_arr, int(ncand), int(repeats),
                                 ctypes.byref(best), ms)
        if rc != GSPAN_OK:
            raise self._err(rc, "gspan_autotune")
        n = ncand if candidates is not None else min(ncand, 6)
        return {key: getattr(best, key) for key in self.TUNABLES}, list(ms)[:n]

    def table_support(self, cols, nr_nodes: int):
        """MNI support of an embedding table on the device (the reference's
        support_gpu for a column table).  ``cols``: CUDA int32 tensors of equal
        length, one per pattern vertex.  Returns (domain sizes, support)."""
        import torch
        nrows = int(cols[0].numel()) if cols else 0
        ptrs = (ctypes.c_void_p * len(cols))(*[c.data_ptr() for c in cols])
        out = torch.empty(len(cols) + 1, dtype=torch.int32, device=cols[0].device if cols else "cuda")
        rc = _lib.gspan_table_support(self._ctx, int(nr_nodes), ptrs, len(cols), nrows, out.data_ptr())
        if rc != GSPAN_OK:
            raise self._err(rc, "gspan_table_support")
        host = out.cpu().tolist()
        return host[:-1], host[-1]

    def fsm(self, g: CSR, k: int, min_support: int):
        """Upload, mine, free: the reference's ``fsm`` as one call."""
        dg = self.upload(g)
        try:
            return self.mine(dg, k, min_support)
        finally:
            self.free(dg)

    def close(self) -> None:
        for dg in list(self._graphs):
            self.free(dg)
        if self._ctx:
            _lib.gspan_ctx_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving loop (gspan_server_*): resident graphs, jobs queued as they
    arrive, run on `slots` concurrent contexts with byte-budget admission."""

    def __init__(self, device: int = 0, slots: int = 4, budget_bytes: float = 0.0):
        self._s = ctypes.c_void_p()
        rc = _lib.gspan_server_create(device, slots, float(budget_bytes), ctypes.byref(self._s))
        if rc != GSPAN_OK:
            raise GspanError(rc, "gspan_server_create")

    def add_graph(self, g: CSR) -> int:
        off = np.ascontiguousarray(g.offsets, dtype=np.int32)
        vl = np.ascontiguousarray(g.vlabels, dtype=np.int32)
        ed = np.ascontiguousarray(g.edges, dtype=np.int32).reshape(-1, 3)
        gid = ctypes.c_int32()
        rc = _lib.gspan_server_add_graph(self._s, g.n, g.m, off.ctypes.data, vl.ctypes.data if g.n else None,
                                         ed.ctypes.data if g.m else None, ctypes.byref(gid))
        if rc != GSPAN_OK:
            raise GspanError(rc, "gspan_server_add_graph")
        return gid.value

    def submit(self, graph_id: int, k: int, min_support: int) -> int:
        jid = ctypes.c_int64()
        rc = _lib.gspan_server_submit(self._s, graph_id, int(k), int(min_support), ctypes.byref(jid))
        if rc != GSPAN_OK:
            raise GspanError(rc, "gspan_server_submit")
        return jid.value

    def wait(self, job_id: int):
        """Returns (patterns, info dict) of a finished job (blocks until done)."""
        col = _Collector()
        try:
            info = JobInfo()
            rc = _lib.gspan_server_wait(self._s, int(job_id), _RESULTS_EMIT, col.h, ctypes.byref(info))
            if rc != GSPAN_OK:
                raise GspanError(rc, "gspan_server_wait")
            flat = col.array()
        finally:
            col.close()
        d = {name: getattr(info, name) for name, _ in info._fields_ if name != "stats"}
        d["stats"] = info.stats.as_dict()
        return decode_results(flat, 1)[0], d

    def close(self) -> None:
        if self._s:
            _lib.gspan_server_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
