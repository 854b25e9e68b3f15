"""Batched decomposition of many graphs (segmented CSR) against the oracle."""
import numpy as np
import pytest

import oracle
import pico_gb300 as pg
from oracle import gen as gen_ref
from pico_gb300 import workloads

pytestmark = pytest.mark.gpu


def test_ba_and_bounded_rmat_generators_match_host():
    s, d, m = pg.DeviceBuffer(4 * 5000), pg.DeviceBuffer(4 * 5000), 5000
    pg.check(pg.lib().kc_gen_ba(1000, 5, 77, pg.ctypes.c_void_p(s.ptr), pg.ctypes.c_void_p(d.ptr), None))
    pg.check(pg.lib().kc_device_synchronize(0))
    es, ed = gen_ref.ba(1000, 5, 77)
    assert np.array_equal(s.download(np.uint32, m), es) and np.array_equal(d.download(np.uint32, m), ed)
    pg.check(pg.lib().kc_gen_rmat_bounded(1500, 5000, 0.57, 0.19, 0.19, 5, pg.ctypes.c_void_p(s.ptr),
                                          pg.ctypes.c_void_p(d.ptr), None))
    pg.check(pg.lib().kc_device_synchronize(0))
    es, ed = gen_ref.rmat_bounded(1500, 5000, 5)
    assert np.array_equal(s.download(np.uint32, m), es) and np.array_equal(d.download(np.uint32, m), ed)


def small_mix(G=300, seed=9):
    return workloads.batch_mix(G, seed, log_n=(1.0, 3.7))


@pytest.mark.parametrize("cuda_graph", [0, 1])
def test_batch_matches_bz_small_mix(cuda_graph):
    g, vbase, p = small_mix()
    rp, col = g.csr()
    core, _ = oracle.bz(rp, col)
    b = pg.Batch(g, vbase)
    b.set_param("batch.cuda_graph", cuda_graph)
    for _ in range(2):
        got, ms = b.decompose()
        assert np.array_equal(got, core)
    # every size class, including the global-memory path
    for small_n, chunk in ((32, 128), (100000, 4096), (1024, 256)):
        b.set_param("batch.small_n", small_n)
        b.set_param("batch.chunk", chunk)
        got, _ = b.decompose()
        assert np.array_equal(got, core), (small_n, chunk)
    b.free()


def test_batch_segments_equal_single_graph_runs():
    g, vbase, p = small_mix(40, seed=3)
    b = pg.Batch(g, vbase)
    got, _ = b.decompose()
    for i in range(40):
        h = g.segment(vbase[i], vbase[i + 1])
        c, _ = h.decompose("peelone_dyn")
        assert np.array_equal(c, got[vbase[i]:vbase[i + 1]]), i
        h.free()


def test_batch_rejects_cross_segment_edges():
    g = pg.Graph.from_edges([0, 1, 2], [1, 2, 3], 4)
    with pytest.raises(pg.KCoreError) as e:
        pg.Batch(g, [0, 2, 4])
    assert e.value.code == pg.KC_ERR_INVALID


def test_autotune_keeps_results_exact():
    g, vbase, p = small_mix(200, seed=5)
    rp, col = g.csr()
    core, _ = oracle.bz(rp, col)
    b = pg.Batch(g, vbase)
    t = b.autotune()
    assert t > 0
    got, _ = b.decompose()
    assert np.array_equal(got, core)


def test_config4_batch_mix_4096():
    """4096 graphs, n log-uniform in [1e2, 1e5], ER / R-MAT / BA: the batched
    result is bit-exact against Batagelj-Zaversnik on the packed CSR."""
    g, vbase, p = workloads.batch_mix(4096, seed=4)
    assert vbase.size == 4097
    b = pg.Batch(g, vbase)
    got, ms = b.decompose()
    rp, col = g.csr()
    core, _ = oracle.bz(rp, col)
    assert np.array_equal(got, core)


@pytest.mark.parametrize("large_threads", [256, 1024])
def test_large_graphs_in_global_memory(large_threads):
    """Graphs above batch.small_n with their degrees in global memory (many
    CTAs per SM) give the same core numbers as the shared-memory class."""
    g, vbase, _ = workloads.batch_mix(96, seed=11)
    b = pg.Batch(g, vbase)
    b.set_param("batch.small_n", 2048)
    want, _ = b.decompose()
    b.set_param("batch.large_shared", 0)
    b.set_param("batch.large_threads", large_threads)
    got, _ = b.decompose()
    assert b.get_param("batch.large_shared") == 0
    assert np.array_equal(got, want)
    rp, col = g.csr()
    assert np.array_equal(got, oracle.bz(rp, col)[0])
    b.free()
    g.free()


def test_batch_size_classes_at_their_edges():
    """Graphs that land in every size class: a star whose centre has degree
    above 65,534 (uint32 degrees), a graph too large for shared memory (global
    class), tiny graphs (1 and 2 vertices, an isolated vertex) and a clique;
    the packed result equals Batagelj-Zaversnik graph by graph."""
    parts = []
    # star with 70,000 leaves: maxdeg above the uint16 range
    leaves = np.arange(1, 70001, dtype=np.uint32)
    parts.append((70001, np.zeros(leaves.size, np.uint32), leaves))
    # 120,000-vertex random graph: above the shared-memory capacity
    rng = np.random.default_rng(3)
    parts.append((120000, rng.integers(0, 120000, 400000).astype(np.uint32),
                  rng.integers(0, 120000, 400000).astype(np.uint32)))
    parts.append((1, np.zeros(0, np.uint32), np.zeros(0, np.uint32)))  # one isolated vertex
    parts.append((2, np.array([0], np.uint32), np.array([1], np.uint32)))
    a, b = np.triu_indices(60, 1)
    parts.append((60, a.astype(np.uint32), b.astype(np.uint32)))
    vbase = [0]
    src, dst = [], []
    for n, s, d in parts:
        src.append(s + vbase[-1])
        dst.append(d + vbase[-1])
        vbase.append(vbase[-1] + n)
    src = np.concatenate(src)
    dst = np.concatenate(dst)
    g = pg.Graph.from_edges(src, dst, vbase[-1], dedup=True)
    bt = pg.Batch(g, np.array(vbase, dtype=np.uint32))
    got, _ = bt.decompose()
    rp, col = g.csr()
    assert np.array_equal(got, oracle.bz(rp, col)[0])
    bt.free()
    g.free()
