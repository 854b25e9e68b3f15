"""TEST INFRASTRUCTURE ONLY -- the k-core oracle.

CPU restatement of chriszhao13/pico's k-core path, used to check the CUDA
engine in ``pico_gb300``.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this package; the product never does.

* ``kcore_oracle.c`` (built here into ``oracle/_build/liboracle.so``) holds the
  serial Batagelj-Zaversnik peel and restatements of the reference's
  decomposition drivers and graph builders; each function cites the reference
  file:line it follows.
* ``load_coo_reference`` / ``load_csr_reference`` below restate the two
  MatrixMarket loaders in pure Python (small files only).
* ``build_ref.sh`` compiles the reference's own loader / virtual-graph host
  code from its sources into ``oracle/_ref/`` when the reference checkout is
  present; ``tests/golden/make_golden.py`` uses those binaries to pin the
  restatements with committed golden files.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
_SRC = os.path.join(HERE, "kcore_oracle.c")

_lib = None
_lock = threading.Lock()


def build(force: bool = False) -> str:
    """Compile kcore_oracle.c with gcc into oracle/_build/liboracle.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(_SRC)):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-pthread", "-shared", "-fPIC", _SRC, "-o", tmp])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_ref() -> bool:
    """Build the reference-side dump tools (oracle/_ref) when the reference is present."""
    script = os.path.join(HERE, "build_ref.sh")
    subprocess.check_call(["bash", script])
    return os.path.exists(os.path.join(HERE, "_ref", "ref_dump_coo"))


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            u32p = ctypes.POINTER(ctypes.c_uint32)
            i64p = ctypes.POINTER(ctypes.c_int64)
            u64p = ctypes.POINTER(ctypes.c_uint64)
            L.orc_bz.argtypes = [ctypes.c_uint32, i64p, u32p, u32p]
            L.orc_bz.restype = ctypes.c_int64
            L.orc_hindex_jacobi.argtypes = [ctypes.c_uint32, i64p, u32p, u32p, u32p]
            L.orc_peel_rounds.argtypes = [ctypes.c_uint32, i64p, u32p, u32p, u32p, u32p]
            L.orc_gpp.argtypes = [ctypes.c_uint32, i64p, u32p, u32p, u32p]
            L.orc_peel_dyn.argtypes = [ctypes.c_uint32, i64p, u32p, u32p, u32p]
            L.orc_make_ugraph.argtypes = [ctypes.c_uint32, ctypes.c_uint64, u32p, u32p, ctypes.c_uint32,
                                          u32p, u32p, u32p, u64p]
            L.orc_csr_dedup.argtypes = [ctypes.c_uint32, ctypes.c_uint64, u32p, u32p, i64p, u32p]
            L.orc_csr_dedup.restype = ctypes.c_int64
            L.orc_check_local.argtypes = [ctypes.c_uint32, i64p, u32p, u32p]
            L.orc_check_local.restype = ctypes.c_uint64
            L.orc_csr_dedup_mt.argtypes = [ctypes.c_uint32, ctypes.c_uint64, u32p, u32p, i64p, u32p, ctypes.c_int]
            L.orc_csr_dedup_mt.restype = ctypes.c_int64
            L.orc_gen_rmat_mt.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                          ctypes.c_uint64, ctypes.c_uint64, u32p, u32p, ctypes.c_int]
            L.orc_gen_rmat_mt.restype = None
            _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def _csr(rowptr, col):
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.uint32)
    if col.size == 0:
        col = np.zeros(1, dtype=np.uint32)
    return rowptr, col, rowptr.size - 1


def bz(rowptr, col):
    """Core numbers by serial Batagelj-Zaversnik; returns (core uint32[n], kmax)."""
    rowptr, col, n = _csr(rowptr, col)
    core = np.zeros(max(n, 1), dtype=np.uint32)
    k = lib().orc_bz(n, _p(rowptr, ctypes.c_int64), _p(col, ctypes.c_uint32), _p(core, ctypes.c_uint32))
    if k < 0:
        raise MemoryError("orc_bz")
    return core[:n], int(k)


def hindex_jacobi(rowptr, col):
    """(core, iterations) of the synchronous h-index iteration (index2core drivers)."""
    rowptr, col, n = _csr(rowptr, col)
    core = np.zeros(max(n, 1), dtype=np.uint32)
    it = ctypes.c_uint32(0)
    rc = lib().orc_hindex_jacobi(n, _p(rowptr, ctypes.c_int64), _p(col, ctypes.c_uint32),
                                 _p(core, ctypes.c_uint32), ctypes.byref(it))
    if rc:
        raise MemoryError("orc_hindex_jacobi")
    return core[:n], it.value


def peel_rounds(rowptr, col):
    """(core, rounds, kmax) of the peelone level-synchronous peel."""
    rowptr, col, n = _csr(rowptr, col)
    core = np.zeros(max(n, 1), dtype=np.uint32)
    r = ctypes.c_uint32(0)
    km = ctypes.c_uint32(0)
    rc = lib().orc_peel_rounds(n, _p(rowptr, ctypes.c_int64), _p(col, ctypes.c_uint32),
                               _p(core, ctypes.c_uint32), ctypes.byref(r), ctypes.byref(km))
    if rc:
        raise MemoryError("orc_peel_rounds")
    return core[:n], r.value, km.value


def gpp(rowptr, col):
    """(final_core, rounds) of the GPP scan/scatter peel (degree-0 vertices get 1)."""
    rowptr, col, n = _csr(rowptr, col)
    core = np.zeros(max(n, 1), dtype=np.uint32)
    r = ctypes.c_uint32(0)
    rc = lib().orc_gpp(n, _p(rowptr, ctypes.c_int64), _p(col, ctypes.c_uint32),
                       _p(core, ctypes.c_uint32), ctypes.byref(r))
    if rc:
        raise MemoryError("orc_gpp")
    return core[:n], r.value


def peel_dyn(rowptr, col):
    """(core, levels) of the peelone_dyn select/queue peel."""
    rowptr, col, n = _csr(rowptr, col)
    core = np.zeros(max(n, 1), dtype=np.uint32)
    lv = ctypes.c_uint32(0)
    rc = lib().orc_peel_dyn(n, _p(rowptr, ctypes.c_int64), _p(col, ctypes.c_uint32),
                            _p(core, ctypes.c_uint32), ctypes.byref(lv))
    if rc:
        raise MemoryError("orc_peel_dyn")
    return core[:n], lv.value


def check_local(rowptr, col, core):
    rowptr, col, n = _csr(rowptr, col)
    core = np.ascontiguousarray(core, dtype=np.uint32)
    return int(lib().orc_check_local(n, _p(rowptr, ctypes.c_int64), _p(col, ctypes.c_uint32),
                                     _p(core, ctypes.c_uint32)))


def make_ugraph(n, src, dst, part_size=64):
    """Reference virtual-graph layout: (nodePointer, edgeList, parts[numParts,2])."""
    src = np.ascontiguousarray(src, dtype=np.uint32)
    dst = np.ascontiguousarray(dst, dtype=np.uint32)
    m = src.size
    deg = np.bincount(np.concatenate([src, dst]).astype(np.int64), minlength=n)[:n] if m else np.zeros(n, np.int64)
    np_total = int(((deg + part_size - 1) // part_size).sum())
    node_ptr = np.zeros(max(n, 1), dtype=np.uint32)
    edge_list = np.zeros(max(2 * m + n, 1), dtype=np.uint32)
    parts = np.zeros(max(2 * np_total, 2), dtype=np.uint32)
    out_np = ctypes.c_uint64(0)
    s = src if m else np.zeros(1, np.uint32)
    d = dst if m else np.zeros(1, np.uint32)
    rc = lib().orc_make_ugraph(n, m, _p(s, ctypes.c_uint32), _p(d, ctypes.c_uint32), part_size,
                               _p(node_ptr, ctypes.c_uint32), _p(edge_list, ctypes.c_uint32),
                               _p(parts, ctypes.c_uint32), ctypes.byref(out_np))
    if rc:
        raise MemoryError("orc_make_ugraph")
    k = out_np.value
    return node_ptr[:n], edge_list[:2 * m + n], parts[:2 * k].reshape(k, 2)


def csr_dedup(n, src, dst, threads=1):
    """Sorted de-duplicated CSR (rowptr int64[n+1], col uint32[nnz]) of an
    edge list; threads > 1 builds it on that many host threads (same result)."""
    src = np.ascontiguousarray(src, dtype=np.uint32)
    dst = np.ascontiguousarray(dst, dtype=np.uint32)
    m = src.size
    rowptr = np.zeros(n + 1, dtype=np.int64)
    col = np.empty(max(2 * m, 1), dtype=np.uint32)
    s = src if m else np.zeros(1, np.uint32)
    d = dst if m else np.zeros(1, np.uint32)
    if threads > 1:
        k = lib().orc_csr_dedup_mt(n, m, _p(s, ctypes.c_uint32), _p(d, ctypes.c_uint32),
                                   _p(rowptr, ctypes.c_int64), _p(col, ctypes.c_uint32), int(threads))
    else:
        k = lib().orc_csr_dedup(n, m, _p(s, ctypes.c_uint32), _p(d, ctypes.c_uint32),
                                _p(rowptr, ctypes.c_int64), _p(col, ctypes.c_uint32))
    if k < 0:
        raise MemoryError("orc_csr_dedup")
    return rowptr, col[:k]


def csr_multi(n, src, dst):
    """CSR that keeps every line of an edge list (both directions, no dedup,
    self-loops dropped), each row in input order: the adjacency the COO loader
    and MakeUGraph produce (virtual_graph.cpp:142-163)."""
    src = np.asarray(src, dtype=np.int64)
    dst = np.asarray(dst, dtype=np.int64)
    keep = src != dst
    src, dst = src[keep], dst[keep]
    m = src.size
    rows = np.empty(2 * m, dtype=np.int64)
    cols = np.empty(2 * m, dtype=np.int64)
    rows[0::2], cols[0::2] = src, dst
    rows[1::2], cols[1::2] = dst, src
    order = np.argsort(rows, kind="stable")
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows, minlength=n)[:n], out=rowptr[1:])
    return rowptr, cols[order].astype(np.uint32)


# --------------------------------------------------------------------------
# Pure-Python restatements of the two MatrixMarket loaders (small files only).

def _tokens(line):
    out = []
    for tok in line.split():
        try:
            out.append(int(tok))
        except ValueError:
            break
    return out


def load_coo_reference(path):
    """Restates Graph::ReadGraph (index2core/shared/graph.cpp:17-95) and the id
    shift of VirtualGraph::VirtualGraph (virtual_graph.cpp:16-23).

    Skips exactly two lines, reads `u v` per line, drops self-loops, keeps
    duplicates.  n = max id, plus one when id 0 occurs; without id 0 every id is
    shifted down by one.  Only well-formed input is restated: a line without two
    integers raises ValueError (the reference would silently re-append the
    previous edge through its reused `newEdge`).
    Returns (n, src, dst, has_zero)."""
    src, dst = [], []
    mx = 0
    has_zero = False
    with open(path, "r") as f:
        lines = f.read().split("\n")
    if lines and lines[-1] == "":
        lines = lines[:-1]
    for line in lines[2:]:
        t = _tokens(line)
        if len(t) < 2:
            raise ValueError("malformed edge line: %r" % line)
        s, e = t[0], t[1]
        if s == e:
            continue
        src.append(s)
        dst.append(e)
        if s == 0 or e == 0:
            has_zero = True
        mx = max(mx, s, e)
    n = mx + 1 if has_zero else mx
    src = np.array(src, dtype=np.int64)
    dst = np.array(dst, dtype=np.int64)
    if not has_zero:
        src -= 1
        dst -= 1
    return n, src.astype(np.uint32), dst.astype(np.uint32), has_zero


def load_csr_reference(path):
    """Restates Graph::readFile (peel/src/graph.cpp:58-133): skip one line,
    read the size line, then `s t [w]` per line with ids shifted from 1-based,
    self-loops dropped, V = max id + 1, neighbours de-duplicated and sorted.
    Only well-formed 1-based input is restated: a line without two integers or
    with id 0 raises ValueError.  Returns (V, rowptr int64[V+1], col uint32[E])."""
    src, dst = [], []
    V = 0
    with open(path, "r") as f:
        lines = f.read().split("\n")
    if lines and lines[-1] == "":
        lines = lines[:-1]
    for line in lines[2:]:
        t = _tokens(line)
        if len(t) < 2 or t[0] < 1 or t[1] < 1:
            raise ValueError("malformed edge line: %r" % line)
        s, e = t[0] - 1, t[1] - 1
        if s == e:
            continue
        V = max(V, s, e)
        src.append(s)
        dst.append(e)
    V += 1
    rowptr, col = csr_dedup(V, np.array(src, dtype=np.uint32), np.array(dst, dtype=np.uint32))
    return V, rowptr, col
