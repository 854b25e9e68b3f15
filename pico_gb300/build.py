"""Build libkcore.so (and the CLI drivers) in-tree with nvcc for sm_103a.

Every translation unit under pico_gb300/csrc is compiled in parallel into
pico_gb300/_build/obj/, then linked into pico_gb300/_build/libkcore.so.  The
CLI drivers under pico_gb300/cli link against that library.  Nothing is
installed outside the package folder.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
CLI = os.path.join(PKG, "cli")
BUILD = os.path.join(PKG, "_build")
OBJ = os.path.join(BUILD, "obj")
BIN = os.path.join(BUILD, "bin")
LIB = os.path.join(BUILD, "libkcore.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "-I" + INCLUDE]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose=False):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + _headers()):
        return obj, None
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj + ".tmp"]
    if src.endswith(".cpp"):
        cmd = [nvcc()] + NVCC_FLAGS + ["-x", "c++", "-c", src, "-o", obj + ".tmp"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj, (r.stderr if verbose else None)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile every CUDA/C++ source and link libkcore.so; returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    objs = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for obj, msg in ex.map(lambda s: _compile(s, verbose), srcs):
            if msg and msg.startswith("compile failed"):
                raise RuntimeError(msg)
            if msg and verbose:
                sys.stderr.write(msg)
            objs.append(obj)
    if _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(tmp, LIB)
    _build_cli()
    return LIB


def _build_cli():
    srcs = sorted(glob.glob(os.path.join(CLI, "*.cpp")))
    common = [s for s in srcs if os.path.basename(s).startswith("_")]
    mains = [s for s in srcs if s not in common]
    for src in mains:
        name = os.path.splitext(os.path.basename(src))[0]
        out = os.path.join(BIN, name)
        if not _stale(out, [src, LIB] + common + _headers()):
            continue
        cmd = ["g++", "-O2", "-std=c++17", "-I" + INCLUDE, src] + common + \
            ["-L" + BUILD, "-lkcore", "-Wl,-rpath,$ORIGIN/..", "-o", out + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("CLI build failed: %s\n%s" % (" ".join(cmd), r.stderr))
        os.replace(out + ".tmp", out)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
