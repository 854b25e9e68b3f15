"""pico_gb300 -- GB300-native k-core decomposition engine.

Python mirror of the C ABI in include/kcore.h (libkcore.so, built in-tree by
pico_gb300/build.py).  Everything here is a thin ctypes binding: the graph
build and every decomposition run as hand-written sm_103a CUDA inside the
library; there is no CPU fallback.  If the library is missing the calls raise
KCoreError instead of computing anything on the host.

The reference (chriszhao13/pico) exposes no library: each method is a CUDA
executable.  ``pico_gb300.reference`` mirrors its driver-level interface
(``Graph(path)``, ``peelone_dyn(g)``, ``repSimulation``...) on top of this
module.
"""
from __future__ import annotations

import ctypes
import os
import re
from dataclasses import dataclass

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libkcore.so")
HEADER = os.path.join(os.path.dirname(_PKG), "include", "kcore.h")

# status codes (kcore.h)
KC_OK, KC_ERR_INVALID, KC_ERR_IO, KC_ERR_CUDA, KC_ERR_NOMEM, KC_ERR_CAPACITY, KC_ERR_TIMEOUT, \
    KC_ERR_UNSUPPORTED, KC_ERR_STATE = range(9)
STATUS_NAMES = {0: "KC_OK", 1: "KC_ERR_INVALID", 2: "KC_ERR_IO", 3: "KC_ERR_CUDA", 4: "KC_ERR_NOMEM",
                5: "KC_ERR_CAPACITY", 6: "KC_ERR_TIMEOUT", 7: "KC_ERR_UNSUPPORTED", 8: "KC_ERR_STATE"}

# methods (kcore.h): the reference's seven drivers plus AUTO
METHODS = {"HistoCore": 0, "CntCore": 1, "NbrCore": 2, "peelone": 3, "gppeel": 4, "peelone_dyn": 5,
           "peel_dyn": 6, "auto": 7}
_ALIASES = {"histo": 0, "cnt": 1, "nbr": 2, "gpp": 4, "peel": 5}

LOAD_COO, LOAD_CSR_DEDUP = 0, 1
EDGES_DEDUP, EDGES_SORT_ROWS = 1, 2


class KCoreError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(code, str(code)), msg))
        self.code = code


class kc_stats(ctypes.Structure):
    _fields_ = [("method", ctypes.c_uint32), ("iterations", ctypes.c_uint32), ("levels", ctypes.c_uint32),
                ("kmax", ctypes.c_uint32), ("kmin", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("n", ctypes.c_uint64), ("nnz", ctypes.c_uint64), ("ms", ctypes.c_double),
                ("build_ms", ctypes.c_double)]


class kc_update_stats(ctypes.Structure):
    _fields_ = [("inserted", ctypes.c_uint64), ("deleted", ctypes.c_uint64), ("rounds", ctypes.c_uint32),
                ("sweeps", ctypes.c_uint32), ("candidates", ctypes.c_uint64), ("recomputed", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("ms", ctypes.c_double)]


class kc_server_config(ctypes.Structure):
    _fields_ = [("decompose_slots", ctypes.c_uint32), ("max_batch_graphs", ctypes.c_uint32),
                ("max_batch_bytes", ctypes.c_uint64), ("hbm_reserve_bytes", ctypes.c_uint64)]


class kc_request_result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("kind", ctypes.c_uint32), ("n", ctypes.c_uint32),
                ("kmax", ctypes.c_uint32), ("digest", ctypes.c_uint64), ("latency_ms", ctypes.c_double),
                ("queue_ms", ctypes.c_double), ("update", kc_update_stats), ("has_core", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class kc_server_stats(ctypes.Structure):
    _fields_ = [("completed_updates", ctypes.c_uint64), ("completed_decompositions", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("p50_update_ms", ctypes.c_double), ("p99_update_ms", ctypes.c_double),
                ("p50_decompose_ms", ctypes.c_double), ("p99_decompose_ms", ctypes.c_double),
                ("elapsed_ms", ctypes.c_double), ("edges_decomposed", ctypes.c_uint64),
                ("edges_updated", ctypes.c_uint64), ("decompose_launches", ctypes.c_uint64),
                ("max_inflight", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class kc_level_trace(ctypes.Structure):
    _fields_ = [("t_start_ns", ctypes.c_uint64), ("level", ctypes.c_uint32), ("claimed", ctypes.c_uint32),
                ("scan_len", ctypes.c_uint32), ("spilled", ctypes.c_uint32), ("steals", ctypes.c_uint32),
                ("steal_fail", ctypes.c_uint32), ("t_work_end_ns", ctypes.c_uint64), ("rounds", ctypes.c_uint32),
                ("max_steal", ctypes.c_uint32), ("cta_ns", ctypes.c_uint64 * 4)]


@dataclass
class Stats:
    method: str
    iterations: int
    levels: int
    kmax: int
    kmin: int
    n: int
    nnz: int
    ms: float
    build_ms: float


_lib = None
_P = ctypes.c_void_p
_U32P = ctypes.POINTER(ctypes.c_uint32)
_I64P = ctypes.POINTER(ctypes.c_int64)
_U64P = ctypes.POINTER(ctypes.c_uint64)


def _sig(L, name, res, args):
    f = getattr(L, name)
    f.restype = res
    f.argtypes = args


def lib():
    """Load libkcore.so (raises KCoreError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise KCoreError(KC_ERR_STATE, "libkcore.so is not built (%s); run pico_gb300.build.build()" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    i, u32, u64, d = ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double
    PP = ctypes.POINTER(_P)
    _sig(L, "kc_abi_version", i, [])
    _sig(L, "kc_last_error", ctypes.c_char_p, [])
    _sig(L, "kc_device_count", i, [])
    _sig(L, "kc_graph_from_mtx", i, [ctypes.c_char_p, i, i, PP])
    _sig(L, "kc_parse_mtx", i, [ctypes.c_char_p, i, _U32P, _U64P, ctypes.POINTER(_U32P), ctypes.POINTER(_U32P)])
    _sig(L, "kc_host_free_edges", None, [_U32P, _U32P])
    _sig(L, "kc_graph_from_edges", i, [_P, _P, u64, u32, u32, i, PP])
    _sig(L, "kc_graph_from_edges_device", i, [_P, _P, u64, u32, u32, i, PP])
    _sig(L, "kc_graph_from_csr", i, [_P, _P, u32, i, PP])
    _sig(L, "kc_graph_from_csr_device", i, [_P, _P, u32, i, PP])
    _sig(L, "kc_graph_validate", i, [_P, _U64P])
    _sig(L, "kc_graph_free", i, [_P])
    _sig(L, "kc_graph_info", i, [_P, _U32P, _U64P, _U32P, _U64P])
    _sig(L, "kc_graph_device_csr", i, [_P, PP, PP])
    _sig(L, "kc_graph_copy_csr", i, [_P, _P, _P])
    _sig(L, "kc_graph_degrees", i, [_P, _P])
    _sig(L, "kc_graph_virtual_layout", i, [_P, u32, _P, _P, _P, _U64P])
    _sig(L, "kc_decompose", i, [_P, i, _P, i, ctypes.POINTER(kc_stats), _P])
    _sig(L, "kc_graph_device_core", i, [_P, PP])
    _sig(L, "kc_graph_last_timing", i, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)])
    _sig(L, "kc_graph_set_param", i, [_P, ctypes.c_char_p, ctypes.c_int64])
    _sig(L, "kc_graph_trace", i, [_P, ctypes.POINTER(kc_level_trace), u32, _U32P])
    _sig(L, "kc_host_alloc", i, [PP, ctypes.c_size_t])
    _sig(L, "kc_host_free", i, [_P])
    _sig(L, "kc_device_alloc", i, [PP, ctypes.c_size_t, i])
    _sig(L, "kc_device_free", i, [_P])
    _sig(L, "kc_memcpy", i, [_P, _P, ctypes.c_size_t, i])
    _sig(L, "kc_device_synchronize", i, [i])
    _sig(L, "kc_gen_rmat", i, [u32, u64, d, d, d, u64, _P, _P, _P])
    _sig(L, "kc_gen_er", i, [u32, u64, u64, _P, _P, _P])
    _sig(L, "kc_gen_planted", i, [u32, u32, d, u64, _P, _P, u64, _U64P, _P])
    _sig(L, "kc_gen_rmat_bounded", i, [u32, u64, d, d, d, u64, _P, _P, _P])
    _sig(L, "kc_gen_ba", i, [u32, u32, u64, _P, _P, _P])
    _sig(L, "kc_edges_offset", i, [_P, _P, u64, u32, _P])
    _sig(L, "kc_batch_create", i, [_P, _P, u32, PP])
    _sig(L, "kc_batch_set_param", i, [_P, ctypes.c_char_p, ctypes.c_int64])
    _sig(L, "kc_batch_get_param", i, [_P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64)])
    _sig(L, "kc_batch_autotune", i, [_P, ctypes.POINTER(ctypes.c_double)])
    _sig(L, "kc_batch_decompose", i, [_P, _P, i, ctypes.POINTER(kc_stats), _P])
    _sig(L, "kc_batch_free", i, [_P])
    _sig(L, "kc_batch_trace", i, [_P, _P, u32])
    _sig(L, "kc_graph_from_segment", i, [_P, u32, u32, PP])
    _sig(L, "kc_graph_save", i, [_P, ctypes.c_char_p])
    _sig(L, "kc_graph_load", i, [ctypes.c_char_p, i, PP])
    _sig(L, "kc_graph_from_edge_file", i, [ctypes.c_char_p, u32, i, PP])
    _sig(L, "kc_graph_kcore_subgraph", i, [_P, u32, PP, _P, i])
    _sig(L, "kc_graph_update", i, [_P, _P, _P, u64, _P, _P, u64, _P, i, ctypes.POINTER(kc_update_stats)])
    _sig(L, "kc_server_create", i, [_P, ctypes.POINTER(kc_server_config), PP])
    _sig(L, "kc_server_submit_update", i, [_P, _P, _P, u64, _P, _P, u64, i, _U64P])
    _sig(L, "kc_server_submit_decompose", i, [_P, _P, _P, u32, _U64P])
    _sig(L, "kc_server_wait", i, [_P, u64, ctypes.POINTER(kc_request_result), _P, u64])
    _sig(L, "kc_server_get_stats", i, [_P, ctypes.POINTER(kc_server_stats)])
    _sig(L, "kc_server_free", i, [_P])
    _sig(L, "kc_decompose_noalloc", i, [_P, _P, u32, _P, _P])
    _sig(L, "kc_graph_autotune", i, [_P, ctypes.POINTER(i), ctypes.POINTER(ctypes.c_double)])
    _lib = L
    return L


def check(rc):
    if rc != KC_OK:
        raise KCoreError(rc, lib().kc_last_error().decode(errors="replace"))


def header_symbols(path=HEADER):
    """Names of the functions declared in include/kcore.h."""
    txt = open(path).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(kc_\w+)\s*\(", txt)))


def method_id(method) -> int:
    if isinstance(method, int):
        return method
    if method in METHODS:
        return METHODS[method]
    m = method.lower()
    for k, v in METHODS.items():
        if k.lower() == m:
            return v
    if m in _ALIASES:
        return _ALIASES[m]
    raise ValueError("unknown method %r" % (method,))


def method_name(mid: int) -> str:
    for k, v in METHODS.items():
        if v == mid:
            return k
    return str(mid)


def device_count() -> int:
    return lib().kc_device_count()


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else ctypes.c_void_p(0)


class DeviceBuffer:
    """Device memory owned by Python (kc_device_alloc / kc_device_free)."""

    def __init__(self, nbytes, device=0):
        p = ctypes.c_void_p()
        check(lib().kc_device_alloc(ctypes.byref(p), max(int(nbytes), 1), device))
        self.ptr = p.value
        self.nbytes = int(nbytes)
        self.device = device

    def free(self):
        if self.ptr:
            lib().kc_device_free(ctypes.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def upload(self, arr):
        arr = np.ascontiguousarray(arr)
        assert arr.nbytes <= self.nbytes
        check(lib().kc_memcpy(ctypes.c_void_p(self.ptr), _ptr(arr), arr.nbytes, 1))

    def download(self, dtype, count):
        out = np.empty(count, dtype=dtype)
        if out.nbytes:
            check(lib().kc_memcpy(_ptr(out), ctypes.c_void_p(self.ptr), out.nbytes, 2))
        return out


class Graph:
    """A device-resident graph (owns a kc_graph handle)."""

    def __init__(self, handle, device=0):
        self._h = ctypes.c_void_p(handle)
        self.device = device

    def info(self):
        """(n, nnz, max degree, 32-wide virtual nodes), read from the library
        (they change when the graph is updated)."""
        n, nnz, md, vn = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint64()
        check(lib().kc_graph_info(self._h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(md), ctypes.byref(vn)))
        return n.value, nnz.value, md.value, vn.value

    @property
    def n(self):
        return self.info()[0]

    @property
    def nnz(self):
        return self.info()[1]

    @property
    def max_degree(self):
        return self.info()[2]

    @property
    def num_vnodes(self):
        return self.info()[3]

    # ---- construction ----
    @classmethod
    def from_mtx(cls, path, mode="coo", device=0):
        m = {"coo": LOAD_COO, "csr": LOAD_CSR_DEDUP, "dedup": LOAD_CSR_DEDUP}.get(mode, mode)
        h = ctypes.c_void_p()
        check(lib().kc_graph_from_mtx(os.fsencode(path), m, device, ctypes.byref(h)))
        return cls(h.value, device)

    @classmethod
    def from_edges(cls, src, dst, n, dedup=False, sort_rows=False, device=0):
        src = np.ascontiguousarray(src, dtype=np.uint32)
        dst = np.ascontiguousarray(dst, dtype=np.uint32)
        flags = (EDGES_DEDUP if dedup else 0) | (EDGES_SORT_ROWS if sort_rows else 0)
        h = ctypes.c_void_p()
        check(lib().kc_graph_from_edges(_ptr(src), _ptr(dst), src.size, int(n), flags, device, ctypes.byref(h)))
        return cls(h.value, device)

    @classmethod
    def from_edges_device(cls, d_src, d_dst, m, n, dedup=False, sort_rows=False, device=0):
        flags = (EDGES_DEDUP if dedup else 0) | (EDGES_SORT_ROWS if sort_rows else 0)
        h = ctypes.c_void_p()
        check(lib().kc_graph_from_edges_device(ctypes.c_void_p(d_src), ctypes.c_void_p(d_dst), int(m), int(n),
                                               flags, device, ctypes.byref(h)))
        return cls(h.value, device)

    @classmethod
    def from_csr(cls, rowptr, col, device=0):
        rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        col = np.ascontiguousarray(col, dtype=np.uint32)
        h = ctypes.c_void_p()
        check(lib().kc_graph_from_csr(_ptr(rowptr), _ptr(col), rowptr.size - 1, device, ctypes.byref(h)))
        return cls(h.value, device)

    @classmethod
    def from_csr_ptr(cls, rowptr_ptr, col_ptr, n, device=0):
        """Host pointers (e.g. pinned buffers) to a CSR; copies H2D inside the call."""
        h = ctypes.c_void_p()
        check(lib().kc_graph_from_csr(ctypes.c_void_p(rowptr_ptr), ctypes.c_void_p(col_ptr), int(n), device,
                                      ctypes.byref(h)))
        return cls(h.value, device)

    # ---- lifetime ----
    def free(self):
        if self._h is not None and self._h.value:
            lib().kc_graph_free(self._h)
        self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()

    @property
    def handle(self):
        return self._h

    # ---- queries ----
    def csr(self):
        n, nnz, _, _ = self.info()
        rowptr = np.empty(n + 1, dtype=np.int64)
        col = np.empty(max(nnz, 1), dtype=np.uint32)
        check(lib().kc_graph_copy_csr(self._h, _ptr(rowptr), _ptr(col)))
        return rowptr, col[:nnz]

    def degrees(self):
        d = np.empty(max(self.n, 1), dtype=np.uint32)
        check(lib().kc_graph_degrees(self._h, _ptr(d)))
        return d[:self.n]

    def device_csr(self):
        r, c = ctypes.c_void_p(), ctypes.c_void_p()
        check(lib().kc_graph_device_csr(self._h, ctypes.byref(r), ctypes.byref(c)))
        return r.value, c.value

    def validate(self):
        bad = ctypes.c_uint64()
        check(lib().kc_graph_validate(self._h, ctypes.byref(bad)))
        return bad.value

    def virtual_layout(self, part_size=64):
        """Reference virtual-graph layout (nodePointer, edgeList, parts[numParts, 2])."""
        np_ = ctypes.c_uint64()
        check(lib().kc_graph_virtual_layout(self._h, part_size, None, None, None, ctypes.byref(np_)))
        k = np_.value
        node_ptr = np.empty(max(self.n, 1), dtype=np.uint32)
        edge_list = np.empty(max(self.nnz + self.n, 1), dtype=np.uint32)
        parts = np.empty(max(2 * k, 2), dtype=np.uint32)
        check(lib().kc_graph_virtual_layout(self._h, part_size, _ptr(node_ptr), _ptr(edge_list), _ptr(parts),
                                            ctypes.byref(np_)))
        return node_ptr[:self.n], edge_list[:self.nnz + self.n], parts[:2 * k].reshape(k, 2)

    # ---- decomposition ----
    def decompose(self, method="peelone_dyn", out=None, stream=0):
        """Core numbers (uint32[n]) and Stats.  `out`: optional host array to fill."""
        mid = method_id(method)
        core = out if out is not None else np.empty(max(self.n, 1), dtype=np.uint32)
        st = kc_stats()
        check(lib().kc_decompose(self._h, mid, _ptr(core), 0, ctypes.byref(st), ctypes.c_void_p(stream)))
        return core[:self.n], _stats(st)

    def decompose_device(self, method="peelone_dyn", stream=0, stats=False):
        """Run on the device and leave the result there; returns Stats (if asked)."""
        st = kc_stats()
        check(lib().kc_decompose(self._h, method_id(method), None, 0, ctypes.byref(st) if stats else None,
                                 ctypes.c_void_p(stream)))
        return _stats(st) if stats else None

    def autotune(self):
        """Times the peel variants and the h-index iteration on this graph
        and keeps the fastest for method "auto"; returns (method name, ms)."""
        m = ctypes.c_int()
        ms = ctypes.c_double()
        check(lib().kc_graph_autotune(self._h, ctypes.byref(m), ctypes.byref(ms)))
        return method_name(m.value), ms.value

    def last_timing(self):
        """(total_ms, kernel_ms) of the last decomposition (CUDA events)."""
        a, b = ctypes.c_double(), ctypes.c_double()
        check(lib().kc_graph_last_timing(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def set_param(self, name, value):
        check(lib().kc_graph_set_param(self._h, name.encode(), int(value)))

    def trace(self):
        """Per-level trace of the last peel, or per-sweep trace of the last
        h-index decomposition (after set_param("trace", 1))."""
        cnt = ctypes.c_uint32()
        check(lib().kc_graph_trace(self._h, None, 0, ctypes.byref(cnt)))
        buf = (kc_level_trace * max(cnt.value, 1))()
        check(lib().kc_graph_trace(self._h, buf, cnt.value, ctypes.byref(cnt)))
        keys = [f[0] for f in kc_level_trace._fields_]
        return [{k: getattr(buf[i], k) for k in keys} for i in range(cnt.value)]

    def update(self, ins=None, dels=None, want_core=True):
        """Apply an edge batch (deletions first) keeping the core numbers
        exact.  ins / dels: (src, dst) arrays.  Returns (core or None, stats dict)."""
        e = np.zeros(0, dtype=np.uint32)
        is_, id_ = (np.ascontiguousarray(x, dtype=np.uint32) for x in (ins if ins is not None else (e, e)))
        ds_, dd_ = (np.ascontiguousarray(x, dtype=np.uint32) for x in (dels if dels is not None else (e, e)))
        core = np.empty(max(self.n, 1), dtype=np.uint32) if want_core else None
        st = kc_update_stats()
        check(lib().kc_graph_update(self._h, _ptr(is_), _ptr(id_), is_.size, _ptr(ds_), _ptr(dd_), ds_.size,
                                    _ptr(core) if want_core else None, 0, ctypes.byref(st)))
        stats = {k: getattr(st, k) for k, _ in kc_update_stats._fields_ if k != "reserved"}
        return (core[:self.n] if want_core else None), stats

    def save(self, path):
        """Binary snapshot (CSR, and the core numbers when a decomposition has completed)."""
        check(lib().kc_graph_save(self._h, os.fsencode(path)))

    @classmethod
    def load(cls, path, device=0):
        """Graph from a snapshot written by save(); its core numbers come back too."""
        h = ctypes.c_void_p()
        check(lib().kc_graph_load(os.fsencode(path), device, ctypes.byref(h)))
        return cls(h.value, device)

    @classmethod
    def from_edge_file(cls, path, dedup=False, sort_rows=False, device=0):
        """Graph from a binary file of little-endian uint32 (src, dst) pairs."""
        flags = (EDGES_DEDUP if dedup else 0) | (EDGES_SORT_ROWS if sort_rows else 0)
        h = ctypes.c_void_p()
        check(lib().kc_graph_from_edge_file(os.fsencode(path), flags, device, ctypes.byref(h)))
        return cls(h.value, device)

    def kcore_subgraph(self, k):
        """(Graph of the induced k-core, original ids uint32[n']) of the last decomposition."""
        core = self.core()
        cnt = int((core >= k).sum())
        ids = np.zeros(max(cnt, 1), dtype=np.uint32)
        h = ctypes.c_void_p()
        check(lib().kc_graph_kcore_subgraph(self._h, int(k), ctypes.byref(h), _ptr(ids), 0))
        return Graph(h.value, self.device), ids[:cnt]

    def core(self):
        """Core numbers of the last decomposition (host copy of the device result)."""
        p = self.device_core()
        out = np.empty(max(self.n, 1), dtype=np.uint32)
        if self.n:
            check(lib().kc_memcpy(_ptr(out), ctypes.c_void_p(p), 4 * self.n, 2))
        return out[:self.n]

    def segment(self, lo, hi):
        """Standalone graph of vertices [lo, hi) (ids rebased to 0)."""
        h = ctypes.c_void_p()
        check(lib().kc_graph_from_segment(self._h, int(lo), int(hi), ctypes.byref(h)))
        return Graph(h.value, self.device)

    def device_core(self):
        p = ctypes.c_void_p()
        check(lib().kc_graph_device_core(self._h, ctypes.byref(p)))
        return p.value


def _stats(st):
    return Stats(method=method_name(st.method), iterations=st.iterations, levels=st.levels, kmax=st.kmax,
                 kmin=st.kmin, n=st.n, nnz=st.nnz, ms=st.ms, build_ms=st.build_ms)


def parse_mtx(path, mode="coo"):
    """Host-only MatrixMarket parse: (n, src uint32[m], dst uint32[m])."""
    m_ = {"coo": LOAD_COO, "csr": LOAD_CSR_DEDUP, "dedup": LOAD_CSR_DEDUP}.get(mode, mode)
    n, m = ctypes.c_uint32(), ctypes.c_uint64()
    s, d = _U32P(), _U32P()
    check(lib().kc_parse_mtx(os.fsencode(path), m_, ctypes.byref(n), ctypes.byref(m), ctypes.byref(s),
                             ctypes.byref(d)))
    try:
        cnt = m.value
        src = np.ctypeslib.as_array(s, shape=(max(cnt, 1),))[:cnt].copy()
        dst = np.ctypeslib.as_array(d, shape=(max(cnt, 1),))[:cnt].copy()
    finally:
        lib().kc_host_free_edges(s, d)
    return n.value, src, dst


# ---- generators (device) ----
RMAT_ABC = (0.57, 0.19, 0.19)


def gen_rmat_edges(scale, num_edges, seed, abc=RMAT_ABC, device=0):
    """Raw R-MAT edge list on the device: (DeviceBuffer src, DeviceBuffer dst, m)."""
    s = DeviceBuffer(4 * num_edges, device)
    d = DeviceBuffer(4 * num_edges, device)
    check(lib().kc_gen_rmat(scale, num_edges, abc[0], abc[1], abc[2], seed, ctypes.c_void_p(s.ptr),
                            ctypes.c_void_p(d.ptr), None))
    check(lib().kc_device_synchronize(device))
    return s, d, num_edges


def gen_er_edges(n, m, seed, device=0):
    s = DeviceBuffer(4 * m, device)
    d = DeviceBuffer(4 * m, device)
    check(lib().kc_gen_er(n, m, seed, ctypes.c_void_p(s.ptr), ctypes.c_void_p(d.ptr), None))
    check(lib().kc_device_synchronize(device))
    return s, d, m


def gen_planted_edges(n, k, p, seed, device=0):
    cap = int(k * (k - 1) // 2 * min(1.0, p * 1.1 + 0.01)) + 1024
    s = DeviceBuffer(4 * cap, device)
    d = DeviceBuffer(4 * cap, device)
    m = ctypes.c_uint64()
    check(lib().kc_gen_planted(n, k, p, seed, ctypes.c_void_p(s.ptr), ctypes.c_void_p(d.ptr), cap,
                               ctypes.byref(m), None))
    check(lib().kc_device_synchronize(device))
    return s, d, m.value


def rmat_graph(scale, edge_factor, seed, abc=RMAT_ABC, device=0):
    """R-MAT graph: 2^scale ids, edge_factor*2^scale draws, deduplicated, symmetrised."""
    n = 1 << scale
    s, d, m = gen_rmat_edges(scale, edge_factor * n, seed, abc, device)
    g = Graph.from_edges_device(s.ptr, d.ptr, m, n, dedup=True, device=device)
    s.free()
    d.free()
    return g


def er_graph(n, m, seed, device=0):
    """Erdos-Renyi G(n, m): m distinct edges drawn without replacement."""
    s, d, mm = gen_er_edges(n, m, seed, device)
    g = Graph.from_edges_device(s.ptr, d.ptr, mm, n, dedup=True, device=device)
    s.free()
    d.free()
    return g


def rmat_planted_graph(scale, edge_factor, k, p, seed, abc=RMAT_ABC, device=0):
    """R-MAT graph plus a planted dense subgraph of k vertices at edge probability p."""
    n = 1 << scale
    m1 = edge_factor * n
    s1, d1, _ = gen_rmat_edges(scale, m1, seed, abc, device)
    s2, d2, m2 = gen_planted_edges(n, k, p, seed + 1, device)
    s = DeviceBuffer(4 * (m1 + m2), device)
    d = DeviceBuffer(4 * (m1 + m2), device)
    for dst_buf, a, b in ((s, s1, s2), (d, d1, d2)):
        check(lib().kc_memcpy(ctypes.c_void_p(dst_buf.ptr), ctypes.c_void_p(a.ptr), 4 * m1, 3))
        if m2:
            check(lib().kc_memcpy(ctypes.c_void_p(dst_buf.ptr + 4 * m1), ctypes.c_void_p(b.ptr), 4 * m2, 3))
    for b in (s1, d1, s2, d2):
        b.free()
    g = Graph.from_edges_device(s.ptr, d.ptr, m1 + m2, n, dedup=True, device=device)
    s.free()
    d.free()
    return g


class Batch:
    """Batched decomposition of the graphs packed in `graph` (segments vbase)."""

    def __init__(self, graph, vbase):
        self.graph = graph
        self.vbase = np.ascontiguousarray(vbase, dtype=np.uint32)
        h = ctypes.c_void_p()
        check(lib().kc_batch_create(graph.handle, _ptr(self.vbase), self.vbase.size - 1, ctypes.byref(h)))
        self._h = h

    @property
    def num_graphs(self):
        return self.vbase.size - 1

    def set_param(self, name, value):
        check(lib().kc_batch_set_param(self._h, name.encode(), int(value)))

    def get_param(self, name):
        v = ctypes.c_int64()
        check(lib().kc_batch_get_param(self._h, name.encode(), ctypes.byref(v)))
        return v.value

    def autotune(self):
        t = ctypes.c_double()
        check(lib().kc_batch_autotune(self._h, ctypes.byref(t)))
        return t.value

    def decompose(self, out=None, stream=0):
        core = out if out is not None else np.empty(max(self.graph.n, 1), dtype=np.uint32)
        st = kc_stats()
        check(lib().kc_batch_decompose(self._h, _ptr(core), 0, ctypes.byref(st), ctypes.c_void_p(stream)))
        return core[:self.graph.n], st.ms

    def decompose_device(self, stream=0):
        st = kc_stats()
        check(lib().kc_batch_decompose(self._h, None, 0, ctypes.byref(st), ctypes.c_void_p(stream)))
        return st.ms

    def trace(self):
        """(start_ns, end_ns, sm) per graph of the last decomposition (after set_param("trace", 1))."""
        out = np.zeros(3 * self.num_graphs, dtype=np.uint64)
        check(lib().kc_batch_trace(self._h, _ptr(out), out.size))
        return out.reshape(-1, 3)

    def free(self):
        if self._h is not None and self._h.value:
            lib().kc_batch_free(self._h)
        self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _struct_dict(st):
    out = {}
    for k, _ in st._fields_:
        if k == "reserved":
            continue
        v = getattr(st, k)
        out[k] = _struct_dict(v) if isinstance(v, ctypes.Structure) else v
    return out


class Server:
    """Continuous-batching request server around a resident graph."""

    def __init__(self, resident, decompose_slots=2, max_batch_graphs=64, max_batch_bytes=256 << 20,
                 hbm_reserve_bytes=1 << 30):
        self.resident = resident
        cfg = kc_server_config(decompose_slots, max_batch_graphs, max_batch_bytes, hbm_reserve_bytes)
        h = ctypes.c_void_p()
        check(lib().kc_server_create(resident.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._keep = {}

    def submit_update(self, ins=None, dels=None, want_core=False):
        e = np.zeros(0, dtype=np.uint32)
        is_, id_ = (np.ascontiguousarray(x, dtype=np.uint32) for x in (ins if ins is not None else (e, e)))
        ds_, dd_ = (np.ascontiguousarray(x, dtype=np.uint32) for x in (dels if dels is not None else (e, e)))
        t = ctypes.c_uint64()
        check(lib().kc_server_submit_update(self._h, _ptr(is_), _ptr(id_), is_.size, _ptr(ds_), _ptr(dd_), ds_.size,
                                            1 if want_core else 0, ctypes.byref(t)))
        return t.value

    def submit_decompose(self, rowptr, col):
        rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        col = np.ascontiguousarray(col, dtype=np.uint32)
        t = ctypes.c_uint64()
        check(lib().kc_server_submit_decompose(self._h, _ptr(rowptr), _ptr(col), rowptr.size - 1, ctypes.byref(t)))
        return t.value

    def wait(self, ticket, core_cap=0):
        res = kc_request_result()
        core = np.empty(max(core_cap, 1), dtype=np.uint32) if core_cap else None
        rc = lib().kc_server_wait(self._h, ticket, ctypes.byref(res), _ptr(core) if core_cap else None, core_cap)
        d = _struct_dict(res)
        if core is not None and res.has_core:
            d["core"] = core[:res.n]
        if rc != KC_OK:
            raise KCoreError(rc, lib().kc_last_error().decode(errors="replace"))
        return d

    def stats(self):
        st = kc_server_stats()
        check(lib().kc_server_get_stats(self._h, ctypes.byref(st)))
        return _struct_dict(st)

    def close(self):
        if self._h is not None and self._h.value:
            check(lib().kc_server_free(self._h))
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
