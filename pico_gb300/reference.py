"""The reference's host interface for the peel drivers, kept name for name.

The reference's ``peel/main.cu`` holds a ``Graph`` loaded from a MatrixMarket
file (``peel/inc/graph.h:5-21``, loader ``peel/src/graph.cpp:58-133``) and
times ``int peel_dyn(Graph&)`` / ``int peelone_dyn(Graph&)``
(``peel/src/peel-dyn.cc:133-182``, ``peel/src/peelone-dyn.cc:120-168``) with
``repSimulation`` (``peel/main.cu:28-49``). This module keeps that shape over
``libkcore``: the functions take a ``Graph``, run one decomposition on the GPU,
set ``g.kmax`` and return whole milliseconds. The graph stays resident on the
device between calls, so repeated runs time only the decomposition, as the
reference's do after its own upload.

Errors raise ``pico_gb300.KCoreError`` instead of exiting the process.
"""
from __future__ import annotations

import math

import numpy as np

from . import Graph as _EngineGraph
from . import KCoreError  # noqa: F401  (re-exported for callers)

__all__ = [
    "Graph", "peel_dyn", "peelone_dyn", "peelone", "gppeel", "histo_core", "cnt_core",
    "nbr_core", "rep_simulation", "std_degrees", "print_max",
]


class Graph:
    """``Graph(input_file)`` of ``peel/inc/graph.h``: the de-duplicated CSR
    loader (1-based ids, ``V`` = max id, sorted unique neighbours).

    ``V`` vertices, ``E`` CSR entries (both directions of each edge, as the
    reference counts them), ``degrees`` the host degree array, ``kmax`` the
    largest core number of the last run (``peel-dyn.cc:176``), ``dmax`` the
    maximum degree. ``neighbors`` / ``neighbors_offset`` are host copies of the
    CSR made on first access. ``core`` holds the core numbers of the last run.
    """

    def __init__(self, input_file: str, device: int = 0):
        self._g = _EngineGraph.from_mtx(input_file, mode="csr", device=device)
        self.V = self._g.n
        self.E = self._g.nnz
        self.degrees = self._g.degrees()
        self.dmax = int(self.degrees.max()) if self.V else 0
        self.AVG_DEGREE = self.E // self.V if self.V else 0
        self.kmax = 0
        self.core = None
        self._csr = None

    @property
    def engine(self) -> _EngineGraph:
        return self._g

    @property
    def neighbors_offset(self) -> np.ndarray:
        if self._csr is None:
            self._csr = self._g.csr()
        return self._csr[0]

    @property
    def neighbors(self) -> np.ndarray:
        if self._csr is None:
            self._csr = self._g.csr()
        return self._csr[1]

    def write_kcore_to_disk(self, path: str) -> None:
        """``Graph::writeKCoreToDisk`` (``peel/src/graph.cpp:135-148``): a JSON
        dictionary ``{ "i": core, ... }`` over vertices of non-zero degree,
        written to ``path`` (the reference prefixes ``./output/pkc-kcore-``)."""
        if self.core is None:
            raise RuntimeError("no decomposition has run on this graph")
        items = [f'"{i}": {int(self.core[i])}' for i in np.flatnonzero(self.degrees)]
        with open(path, "w") as f:
            f.write("{ " + ", \n".join(items) + " }" if items else "{  }")

    def free(self) -> None:
        self._g.free()


def _run(g: Graph, method: str) -> int:
    core, st = g.engine.decompose(method)
    g.core = core
    g.kmax = st.kmax
    return int(st.ms)


def peel_dyn(g: Graph) -> int:
    """``int peel_dyn(Graph&)`` (``peel/src/peel-dyn.cc:133-182``)."""
    return _run(g, "peel_dyn")


def peelone_dyn(g: Graph) -> int:
    """``int peelone_dyn(Graph&)`` (``peel/src/peelone-dyn.cc:120-168``)."""
    return _run(g, "peelone_dyn")


def peelone(g: Graph) -> int:
    """The peelone driver's timed loop (``peel/peelone.cu:157-186``)."""
    return _run(g, "peelone")


def gppeel(g: Graph) -> int:
    """The gppeel driver's timed loop (``peel/gppeel.cu:186-228``); degree-0
    vertices report core 1 as the reference's do."""
    return _run(g, "gppeel")


def histo_core(g: Graph) -> int:
    """HistoCore's timed loop (``index2core/HistoCore.cu:292-341``)."""
    return _run(g, "histo")


def cnt_core(g: Graph) -> int:
    """CntCore's timed loop (``index2core/CntCore.cu:344-417``)."""
    return _run(g, "cnt")


def nbr_core(g: Graph) -> int:
    """NbrCore's timed loop (``index2core/NbrCore.cu:244-297``)."""
    return _run(g, "nbr")


def rep_simulation(kern, g: Graph, rep: int = 10, out=print) -> float:
    """``repSimulation`` (``peel/main.cu:28-49``): run ``kern(g)`` ``rep``
    times, print each time, drop the fastest and slowest from the average,
    print and return it."""
    if rep < 3:
        raise ValueError("rep must be at least 3")
    times = [int(kern(g)) for _ in range(rep)]
    avg = (sum(times) - max(times) - min(times)) / (rep - 2)
    out(" ".join(f"{t}ms" for t in times) + f"  ave: {avg:g}")
    return avg


def std_degrees(g: Graph) -> float:
    """``STDdegrees`` (``peel/main.cu:51-63``): population standard deviation."""
    d = g.degrees.astype(np.float64)
    return math.sqrt(float(((d - d.mean()) ** 2).sum()) / g.V) if g.V else 0.0


def print_max(values) -> int:
    """``PrintMax`` (``peel/main.cu:10-26``): the maximum of the array."""
    return int(np.max(values)) if len(values) else 0
