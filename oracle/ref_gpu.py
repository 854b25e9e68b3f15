"""TEST INFRASTRUCTURE ONLY -- the reference's own GPU drivers as a second oracle.

The seven decomposition drivers of chriszhao13/pico (index2core/HistoCore.cu,
CntCore.cu, NbrCore.cu, peel/peelone.cu, peel/gppeel.cu and the two peel/src
methods peel_dyn / peelone_dyn) are compiled for sm_103a from their own
sources, unmodified, with ``ref_gpu/kcref_shim.h`` pre-included (it pads every
device allocation and captures the core array; see that header), and run as
separate processes on a MatrixMarket file.  ``oracle/build_ref.sh`` copies the
sources (read-only) into the git-ignored ``oracle/_ref/src`` in the
development container; this module compiles them wherever nvcc is present
(the GPU machine has no reference checkout) into ``oracle/_ref/gpu``.

Only tests and the benchmark's reference section use this module, and only
as a checker or a timed baseline.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "_ref", "src")
BIN = os.path.join(HERE, "_ref", "gpu")
SHIM = os.path.join(HERE, "ref_gpu", "kcref_shim.h")
DYN_MAIN = os.path.join(HERE, "ref_gpu", "ref_dyn_main.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# driver -> (source folder under _ref/src, main source, loader semantics)
INDEX2CORE = ("HistoCore", "CntCore", "NbrCore")
PEEL_VG = ("peelone", "gppeel")
DYN = ("peel_dyn", "peelone_dyn")
DRIVERS = INDEX2CORE + PEEL_VG + DYN


def sources_present() -> bool:
    return os.path.isfile(os.path.join(SRC, "index2core", "HistoCore.cu")) and \
        os.path.isfile(os.path.join(SRC, "peel", "src", "peelone-dyn.cc"))


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    return None


def _targets():
    sh_i = [os.path.join(SRC, "index2core", "shared", f) for f in
            ("Timer.cpp", "argument.cpp", "graph.cpp", "util.cpp", "virtual_graph.cpp")]
    sh_p = [os.path.join(SRC, "peel", "shared", f) for f in
            ("Timer.cpp", "argument.cpp", "graph.cpp", "util.cpp", "virtual_graph.cpp")]
    t = {}
    for d in INDEX2CORE:
        t[d] = [os.path.join(SRC, "index2core", d + ".cu")] + sh_i
    for d in PEEL_VG:
        t[d] = [os.path.join(SRC, "peel", d + ".cu")] + sh_p
    t["ref_dyn"] = [DYN_MAIN, os.path.join(SRC, "peel", "src", "graph.cpp"),
                    os.path.join(SRC, "peel", "src", "gpu_memory_allocation.cu")]
    return t


def _stale(out, deps):
    return not os.path.exists(out) or any(os.path.getmtime(d) > os.path.getmtime(out) for d in deps)


def build() -> bool:
    """Compile the drivers (incrementally); False when sources or nvcc are absent."""
    nv = _nvcc()
    if not sources_present() or nv is None:
        return False
    os.makedirs(BIN, exist_ok=True)

    def one(item):
        name, srcs = item
        out = os.path.join(BIN, name)
        if not _stale(out, srcs + [SHIM]):
            return None
        cmd = [nv, "-O3", "-std=c++14", "-w"] + ARCH + ["--pre-include", SHIM]
        if name == "ref_dyn":
            cmd += ["-I" + os.path.join(SRC, "peel"), "-Xcompiler", "-fopenmp"]
        cmd += srcs + ["-o", out + ".tmp"]
        if name == "ref_dyn":
            cmd += ["-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return "%s: %s\n%s" % (name, " ".join(cmd), r.stderr[-3000:])
        os.replace(out + ".tmp", out)
        return None

    with cf.ThreadPoolExecutor(6) as ex:
        errs = [e for e in ex.map(one, _targets().items()) if e]
    if errs:
        raise RuntimeError("reference GPU driver build failed:\n" + "\n".join(errs))
    return True


class RefResult:
    def __init__(self, core, ms, iterations, kmax, stdout):
        self.core = core
        self.ms = ms
        self.iterations = iterations
        self.kmax = kmax
        self.stdout = stdout


def run(driver, mtx_path, n, timeout=600) -> RefResult:
    """Runs one reference driver on a MatrixMarket file in a fresh working
    folder; returns its core array (n values) and its printed time.  `n` is
    the vertex count the driver's loader gives (COO semantics for the five
    virtual-graph drivers, max id for the two peel/src ones)."""
    if driver not in DRIVERS:
        raise ValueError(driver)
    mtx_path = os.path.abspath(mtx_path)
    with tempfile.TemporaryDirectory() as td:
        os.makedirs(os.path.join(td, "output"))
        dump = os.path.join(td, "core.bin")
        env = dict(os.environ)
        if driver in DYN:
            cmd = [os.path.join(BIN, "ref_dyn"), mtx_path, driver, dump]
        else:
            cmd = [os.path.join(BIN, driver), mtx_path]
            env["KCREF_DUMP"] = dump
            env["KCREF_DUMP_BYTES"] = str(4 * n)
        r = subprocess.run(cmd, cwd=td, env=env, capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError("%s exited %d: %s %s" % (driver, r.returncode, r.stdout[-1000:], r.stderr[-1000:]))
        out = r.stdout
        if n == 0:
            core = np.zeros(0, np.uint32)
        else:
            core = np.fromfile(dump, dtype=np.uint32)
        if core.size != n:
            raise RuntimeError("%s: core array of %d values, expected %d" % (driver, core.size, n))
    ms = it = km = None
    m = re.search(r"Processing finished in ([0-9.eE+-]+) \(ms\)", out) or re.search(r"^ms: (\d+)", out, re.M)
    if m:
        ms = float(m.group(1))
    m = re.search(r"Number of iterations = (\d+)", out)
    if m:
        it = int(m.group(1))
    m = re.search(r"Max K = (\d+)", out) or re.search(r"^kmax: (\d+)", out, re.M)
    if m:
        km = int(m.group(1))
    return RefResult(core, ms, it, km, out)
