"""Every decomposition method against the reference's own GPU drivers.

The seven drivers of the reference (HistoCore, CntCore, NbrCore, peelone,
gppeel, peel_dyn, peelone_dyn) are compiled for sm_103a from their own
sources (oracle/ref_gpu.py; the sources are copied next to the tree by
oracle/build_ref.sh in the development container) and run on the same
MatrixMarket files as the engine.  Each engine method's core array must equal
the matching driver's output bit for bit (gppeel's core 1 for degree-0
vertices included), and each driver's output must equal Batagelj-Zaversnik.
The drivers' own "Number of iterations" lines also pin the oracle's
restatements of their synchronous schedules.

Inputs: the ten golden files, Erdos-Renyi G(65,536, 1,048,576) and an R-MAT
scale-16 graph.  The peel/src drivers keep fixed per-block queues of 10^6
entries with a device assert on overflow; every input here has far fewer
vertices than that, so no queue can overflow."""
import os

import numpy as np
import pytest

import oracle
import pico_gb300 as pg
from oracle import ref_gpu

pytestmark = pytest.mark.gpu

COO_DRIVERS = ["HistoCore", "CntCore", "NbrCore", "peelone", "gppeel"]
CSR_DRIVERS = ["peel_dyn", "peelone_dyn"]
CASES = ["example", "zero_based_dups", "dups_selfloops", "sparse_ids", "hub150", "er300", "rmat9",
         "clique40_path", "no_edges", "only_selfloops"]


@pytest.fixture(scope="module")
def drivers():
    if not ref_gpu.sources_present():
        pytest.skip("reference GPU driver sources absent (oracle/build_ref.sh copies them from the checkout)")
    assert ref_gpu.build()


def write_mtx(path, rowptr, col):
    """1-based MatrixMarket file with each undirected edge of a CSR once."""
    n = rowptr.size - 1
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(rowptr))
    up = src < col
    e = np.stack([src[up] + 1, col[up].astype(np.int64) + 1], axis=1)
    with open(path, "w") as f:
        f.write("%%%%MatrixMarket matrix coordinate pattern symmetric\n%d %d %d\n" % (n, n, e.shape[0]))
        np.savetxt(f, e, fmt="%d")


def compare(path, n_coo, n_csr, iterations=None):
    """Runs every driver and engine method on one file; returns the drivers'
    printed iteration counts."""
    its = {}
    g = pg.Graph.from_mtx(path, "coo")
    assert g.n == n_coo
    rp, col = g.csr()
    bz, _ = oracle.bz(rp, col)
    for d in COO_DRIVERS:
        r = ref_gpu.run(d, path, n_coo)
        want = np.where(np.diff(rp) == 0, 1, bz).astype(np.uint32) if d == "gppeel" else bz
        assert np.array_equal(r.core, want), "reference %s differs from Batagelj-Zaversnik" % d
        got, _ = g.decompose(d)
        bad = np.flatnonzero(got != r.core)
        assert bad.size == 0, "%s: %d vertices differ from the reference driver, first %d: %d vs %d" % (
            d, bad.size, bad[0], got[bad[0]], r.core[bad[0]])
        its[d] = r.iterations
    g.free()
    if n_csr is not None:
        g = pg.Graph.from_mtx(path, "csr")
        assert g.n == n_csr
        rp2, col2 = g.csr()
        bz2, _ = oracle.bz(rp2, col2)
        for d in CSR_DRIVERS:
            r = ref_gpu.run(d, path, n_csr)
            assert np.array_equal(r.core, bz2), "reference %s differs from Batagelj-Zaversnik" % d
            got, _ = g.decompose(d)
            assert np.array_equal(got, r.core), d
        g.free()
    return its, (rp, col)


@pytest.mark.parametrize("name", CASES)
def test_golden_inputs_equal_reference_drivers(drivers, golden, mtx_file, name):
    case = golden[name]
    path = mtx_file(case["text"])
    n_csr = case["csr"]["V"] if "csr" in case else None
    compare(path, case["coo"]["n"], n_csr)


def synthetic(tmp_path, kind):
    g = pg.er_graph(65536, 1048576, seed=1) if kind == "er65536" else pg.rmat_graph(16, 16, seed=8)
    rp, col = g.csr()
    g.free()
    path = os.path.join(str(tmp_path), kind + ".mtx")
    write_mtx(path, rp, col)
    # ids of isolated vertices above the largest used id are not part of
    # the file's graph (both loaders size it by the largest id)
    used = np.flatnonzero(np.diff(rp) > 0)
    n = int(used[-1]) + 1 if used.size else 0
    return path, n


@pytest.mark.parametrize("kind", ["er65536", "rmat16"])
def test_synthetic_graphs_equal_reference_drivers(drivers, tmp_path, kind):
    path, n = synthetic(tmp_path, kind)
    its, (rp, col) = compare(path, n, n)
    # the drivers' printed iteration counts are those of the oracle's
    # restated synchronous schedules
    want_h = oracle.hindex_jacobi(rp, col)[1]
    assert its["HistoCore"] == want_h and its["CntCore"] == want_h and its["NbrCore"] == want_h, (its, want_h)
    assert its["peelone"] == oracle.peel_rounds(rp, col)[1], its
    assert its["gppeel"] == oracle.gpp(rp, col)[1], its
