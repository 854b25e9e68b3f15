"""kc_decompose_noalloc: the allocation-free entry point for callers that
cannot allocate device memory on their path (a framework that owns all device
memory through its own pool, or a loop where cudaMalloc's device
synchronisation is not acceptable).  It must give exactly the core numbers of
Batagelj-Zaversnik and of kc_decompose, call after call, through the C ABI,
and turn every input it cannot take into an error status.  This file is
collected last so that a failure here cannot hide the other tests."""
import ctypes

import numpy as np
import pytest

import oracle
import pico_gb300 as pg

pytestmark = pytest.mark.gpu


def call(rp_ptr, col_ptr, n, out):
    return pg.lib().kc_decompose_noalloc(ctypes.c_void_p(rp_ptr), ctypes.c_void_p(col_ptr), n,
                                         ctypes.c_void_p(out.ptr), None)


def noalloc(g, out):
    rp, col = g.device_csr()
    return call(rp, col, g.n, out)


def graphs():
    yield pg.rmat_graph(14, 8, seed=61)
    # 50,000 vertices: the largest graph the entry point takes, and the
    # largest shared-memory footprint of its kernel
    yield pg.er_graph(50000, 400000, seed=62)
    k = 200
    a, b = np.triu_indices(k, 1)
    s = np.concatenate([a, np.zeros(3000)]).astype(np.uint32)
    d = np.concatenate([b, np.arange(k, k + 3000)]).astype(np.uint32)
    yield pg.Graph.from_edges(s, d, k + 3000, dedup=True)


def test_noalloc_matches_bz_and_decompose_twice_in_a_row():
    for g in graphs():
        rp, col = g.csr()
        want, _ = oracle.bz(rp, col)
        engine, _ = g.decompose("peelone_dyn")
        assert np.array_equal(engine, want)
        out = pg.DeviceBuffer(4 * g.n)
        for _ in range(2):  # the shared scratch keeps the previous call's contents
            pg.check(noalloc(g, out))
            got = out.download(np.uint32, g.n)
            assert np.array_equal(got, want)
        out.free()
        g.free()


def test_noalloc_rejects_graphs_beyond_its_limits():
    g = pg.er_graph(60000, 100000, seed=63)  # above the vertex limit
    out = pg.DeviceBuffer(4 * g.n)
    assert noalloc(g, out) == pg.KC_ERR_CAPACITY
    assert b"exceed the limit" in pg.lib().kc_last_error()
    g.free()
    # within the vertex limit, above the 4,194,304-entry limit
    g = pg.er_graph(40000, 2200000, seed=64)
    assert g.nnz > (1 << 22)
    assert noalloc(g, out) == pg.KC_ERR_CAPACITY
    assert b"entries exceed the limit" in pg.lib().kc_last_error()
    g.free()
    out.free()


def test_noalloc_rejects_bad_ids_and_offsets_without_faulting():
    out = pg.DeviceBuffer(64)
    rp = pg.DeviceBuffer(64)
    col = pg.DeviceBuffer(64)
    # column id equal to n
    rp.upload(np.array([0, 1, 2], np.int64))
    col.upload(np.array([1, 2], np.uint32))
    assert call(rp.ptr, col.ptr, 2, out) == pg.KC_ERR_INVALID
    # decreasing row offsets
    rp.upload(np.array([0, 2, 1, 2], np.int64))
    col.upload(np.array([1, 0], np.uint32))
    assert call(rp.ptr, col.ptr, 3, out) == pg.KC_ERR_INVALID
    # the context is still usable: a valid triangle afterwards
    rp.upload(np.array([0, 2, 4, 6], np.int64))
    col.upload(np.array([1, 2, 0, 2, 0, 1], np.uint32))
    pg.check(call(rp.ptr, col.ptr, 3, out))
    assert out.download(np.uint32, 3).tolist() == [2, 2, 2]
    for b in (out, rp, col):
        b.free()


def test_noalloc_empty_and_edgeless_graphs():
    out = pg.DeviceBuffer(64)
    rp = pg.DeviceBuffer(64)
    rp.upload(np.zeros(6, np.int64))
    pg.check(call(rp.ptr, None, 0, out))  # no vertices
    # five isolated vertices, no column array at all
    out.upload(np.full(5, 7, np.uint32))
    pg.check(call(rp.ptr, None, 5, out))
    assert out.download(np.uint32, 5).tolist() == [0] * 5
    out.free()
    rp.free()


def test_noalloc_between_batch_runs_keeps_the_batch_launchable():
    """A planned batch whose graph needs the batched kernel's largest
    shared-memory class (uint32 degrees: a multigraph star with centre degree
    80,000), then an allocation-free call on a small graph, then the batch
    again: the batch still launches and both results stay exact."""
    leaves = np.repeat(np.arange(1, 2001, dtype=np.uint32), 40)  # parallel edges kept
    g = pg.Graph.from_edges(np.zeros(leaves.size, np.uint32), leaves, 2001)
    assert g.max_degree == 80000
    rp, col = g.csr()
    want, _ = oracle.bz(rp, col)
    b = pg.Batch(g, np.array([0, 2001], np.uint32))
    got, _ = b.decompose()
    assert np.array_equal(got, want)
    small = pg.rmat_graph(10, 8, seed=65)
    srp, scol = small.csr()
    out = pg.DeviceBuffer(4 * small.n)
    pg.check(noalloc(small, out))
    assert np.array_equal(out.download(np.uint32, small.n), oracle.bz(srp, scol)[0])
    got, _ = b.decompose()
    assert np.array_equal(got, want)
    out.free()
    small.free()
    b.free()
    g.free()
