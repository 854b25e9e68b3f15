"""kc_decompose_noalloc: the allocation-free entry point for callers that
cannot allocate device memory on their path (a framework that owns all device
memory through its own pool, or a loop where cudaMalloc's device
synchronisation is not acceptable).  It must give exactly the core numbers of
kc_decompose, call after call, through the C ABI.  This file is collected
last so that a failure here cannot hide the other tests."""
import ctypes

import numpy as np
import pytest

import pico_gb300 as pg

pytestmark = pytest.mark.gpu


def noalloc(g, out):
    rp, col = g.device_csr()
    return pg.lib().kc_decompose_noalloc(ctypes.c_void_p(rp), ctypes.c_void_p(col), g.n,
                                         ctypes.c_void_p(out.ptr), None)


def graphs():
    yield pg.rmat_graph(14, 8, seed=61)
    yield pg.er_graph(50000, 400000, seed=62)
    k = 200
    a, b = np.triu_indices(k, 1)
    s = np.concatenate([a, np.zeros(3000)]).astype(np.uint32)
    d = np.concatenate([b, np.arange(k, k + 3000)]).astype(np.uint32)
    yield pg.Graph.from_edges(s, d, k + 3000, dedup=True)


def test_noalloc_matches_decompose_twice_in_a_row():
    for g in graphs():
        want, _ = g.decompose("peelone_dyn")
        out = pg.DeviceBuffer(4 * g.n)
        for _ in range(2):  # the shared scratch keeps the previous call's contents
            pg.check(noalloc(g, out))
            got = out.download(np.uint32, g.n)
            assert np.array_equal(got, want)
        out.free()
        g.free()


def test_noalloc_rejects_graphs_beyond_its_limit():
    g = pg.er_graph(60000, 100000, seed=63)
    out = pg.DeviceBuffer(4 * g.n)
    rc = noalloc(g, out)
    assert rc == pg.KC_ERR_CAPACITY
    assert b"exceed the limit" in pg.lib().kc_last_error()
