"""The peel's work-accounting protocol under extreme tunables: everything
spilled to the shared queues, one item per steal, 1..64 queues, tiny and large
row chunks, one CTA per SM, both CTA sizes and both unroll depths, with and
without warp-aggregated decrements.  Every setting must give the exact core
numbers."""
import numpy as np
import pytest

import oracle
import pico_gb300 as pg

pytestmark = pytest.mark.gpu

SETTINGS = [
    {},
    {"peel.queues": 1},
    {"peel.queues": 64, "peel.steal": 1},
    {"peel.spill": 0, "peel.steal": 3},
    {"peel.spill": 0, "peel.queues": 7, "peel.chunk": 256},
    {"peel.spill": 3072, "peel.steal": 64, "peel.chunk": 65536},
    {"peel.ctas_per_sm": 1, "peel.queues": 32},
    {"peel.chunk": 256, "peel.steal": 5, "peel.queues": 3},
    {"peel.unroll": 8},
    {"peel.threads": 256},
    {"peel.threads": 256, "peel.unroll": 8, "peel.spill": 0, "peel.steal": 2},
    {"peel.threads": 256, "peel.ctas_per_sm": 1, "peel.queues": 16},
    {"peel.balanced": 1},
    {"peel.balanced": 1, "peel.round_entries": 256, "peel.spill": 0, "peel.steal": 1},
    {"peel.balanced": 1, "peel.round_entries": 1 << 20, "peel.unroll": 8},
    {"peel.balanced": 1, "peel.threads": 256, "peel.chunk": 65536, "peel.queues": 5},
    {"peel.balanced": 0, "peel.chunk": 256},
    {"peel.balanced": 0, "peel.unroll": 8, "peel.spill": 0, "peel.steal": 2},
    {"peel.scan_unroll": 8},
    {"peel.scan_unroll": 8, "peel.balanced": 1, "peel.chunk": 512, "peel.round_entries": 16384},
    {"peel.scan_unroll": 8, "peel.threads": 256, "peel.unroll": 8, "peel.spill": 0},
    {"peel.aggregate": 1},
    {"peel.aggregate": 1, "peel.balanced": 0, "peel.unroll": 8, "peel.spill": 0, "peel.steal": 2},
    {"peel.aggregate": 1, "peel.threads": 256, "peel.chunk": 256, "peel.round_entries": 256},
    {"peel.aggregate": 0},
]


def graphs():
    yield "rmat16", pg.rmat_graph(16, 16, seed=11)
    rng = np.random.default_rng(4)
    n = 50000
    s = np.concatenate([np.arange(n - 1), rng.integers(0, n, 20000)]).astype(np.uint32)
    d = np.concatenate([np.arange(1, n), rng.integers(0, n, 20000)]).astype(np.uint32)
    yield "path+random", pg.Graph.from_edges(s, d, n, dedup=True)
    k = 400
    a, b = np.triu_indices(k, 1)
    hub = np.arange(k, 30000, dtype=np.uint32)
    s = np.concatenate([a, np.zeros(hub.size)]).astype(np.uint32)
    d = np.concatenate([b, hub]).astype(np.uint32)
    yield "clique+star", pg.Graph.from_edges(s, d, 30000, dedup=True)


@pytest.mark.parametrize("setting", SETTINGS, ids=lambda p: ",".join("%s=%d" % kv for kv in p.items()) or "default")
def test_peel_exact_under_tunables(setting):
    for name, g in graphs():
        rp, col = g.csr()
        core, _ = oracle.bz(rp, col)
        for k, v in setting.items():
            g.set_param(k, v)
        for method in ("peelone_dyn", "gppeel"):
            got, st = g.decompose(method)
            want = np.where(np.diff(rp) == 0, 1, core) if method == "gppeel" else core
            assert np.array_equal(got, want), (name, method, setting)
        g.free()


def test_trace_records_levels():
    g = pg.rmat_graph(15, 8, seed=5)
    g.set_param("trace", 1)
    core, st = g.decompose("peelone_dyn")
    tr = g.trace()
    assert len(tr) == st.iterations
    assert sum(r["claimed"] for r in tr) == g.n
    levels = [r["level"] for r in tr]
    assert levels == sorted(levels) and levels[0] == 0
    assert len({r["level"] for r in tr if r["claimed"]}) == st.levels == np.unique(core).size


def test_trace_records_hindex_sweeps():
    """After an h-index decomposition the trace holds one record per sweep:
    sweep 0 examines every vertex (short rows by warps; by CTAs the rows
    above 8,192 entries, or above 512 without the degree-ordered copy of the
    long rows), the last sweep lowers nothing, and the estimates lowered add
    up to at least the total drop from degree to core number in steps of one
    vertex each."""
    g = pg.rmat_graph(16, 16, seed=7)
    rp, col = g.csr()
    deg = np.diff(rp)
    want, _ = oracle.bz(rp, col)
    g.set_param("trace", 1)
    for order, cta_rows in ((0, 512), (1, 8192)):
        g.set_param("hindex.order", order)
        core, st = g.decompose("histo")
        assert np.array_equal(core, want)
        tr = g.trace()
        assert len(tr) == st.iterations >= 2
        assert [r["level"] for r in tr] == list(range(len(tr)))
        assert tr[0]["spilled"] == int((deg > cta_rows).sum()) and tr[0]["scan_len"] == g.n
    assert tr[-1]["claimed"] == 0
    lowered = sum(r["claimed"] for r in tr)
    assert lowered >= int((core < deg).sum())
    assert all(r["steals"] <= r["claimed"] for r in tr)
    assert all(r["t_work_end_ns"] >= r["t_start_ns"] for r in tr)
    g.set_param("trace", 0)
    g.decompose("histo")
    assert g.trace() == []
    g.free()


@pytest.mark.parametrize("warp_rows", [512, 2048, 1 << 30])
def test_hindex_warp_rows(warp_rows):
    """Rows above 512 entries re-examined by one warp (windowed histogram
    below the estimate) or by a whole CTA: the same core numbers as
    Batagelj-Zaversnik, on R-MAT graphs with hubs and on a graph whose hub
    loses most of its support (a 700-clique whose vertices also hold long
    pendant stars, joined to a 1,500-leaf hub)."""
    g = pg.rmat_graph(16, 16, seed=11)
    rp, col = g.csr()
    want, _ = oracle.bz(rp, col)
    g.set_param("hindex.warp_rows", warp_rows)
    for method in ("histo", "cnt", "nbr"):
        got, _ = g.decompose(method)
        assert np.array_equal(got, want), method
    g.free()
    a, b = np.triu_indices(700, 1)
    src = [a, np.zeros(1500, np.int64)]
    dst = [b, 700 + np.arange(1500)]
    src.append(np.zeros(600, np.int64))  # the hub also touches the clique
    dst.append(np.arange(1, 601))
    n = 2200 + 700 * 20
    src.append(np.repeat(np.arange(700), 20))  # 20 leaves per clique vertex
    dst.append(2200 + np.arange(700 * 20))
    h = pg.Graph.from_edges(np.concatenate(src).astype(np.uint32), np.concatenate(dst).astype(np.uint32), n,
                            dedup=True)
    h.set_param("hindex.warp_rows", warp_rows)
    rp, col = h.csr()
    want, _ = oracle.bz(rp, col)
    got, _ = h.decompose("histo")
    assert np.array_equal(got, want)
    h.free()


def _hub_graphs():
    """Graphs whose long rows span many degree buckets: an R-MAT graph; a
    400-clique plus a 29,600-leaf star (a hub above 4,096, so the CTA path
    narrows its value range in sweep 0); a hub over 600 star centres of 600
    leaves each (the centres start high and fall to 1, so the hub's estimate
    falls by more than one histogram window); a hub joined to vertices of
    degree 2^0 .. 2^13 and to a 300-clique."""
    yield "rmat16", pg.rmat_graph(16, 16, seed=11)
    k = 400
    a, b = np.triu_indices(k, 1)
    hub = np.arange(k, 30000, dtype=np.uint32)
    yield "clique+star", pg.Graph.from_edges(np.concatenate([a, np.zeros(hub.size)]).astype(np.uint32),
                                             np.concatenate([b, hub]).astype(np.uint32), 30000, dedup=True)
    c = 600
    centres = 1 + np.arange(c)
    leaves = 1 + c + np.arange(c * c)
    s = np.concatenate([np.zeros(c), np.repeat(centres, c)])
    d = np.concatenate([centres, leaves])
    yield "star-of-stars", pg.Graph.from_edges(s.astype(np.uint32), d.astype(np.uint32), 1 + c + c * c, dedup=True)
    src, dst, nxt = [], [], 1
    for e in range(14):  # neighbour nxt of the hub gets 2^e - 1 leaves of its own
        src.append([0])
        dst.append([nxt])
        leaves = (1 << e) - 1
        src.append(np.full(leaves, nxt))
        dst.append(nxt + 1 + np.arange(leaves))
        nxt += 1 + leaves
    a, b = np.triu_indices(300, 1)
    src += [a + nxt, np.zeros(300)]
    dst += [b + nxt, nxt + np.arange(300)]
    n = nxt + 300
    yield "buckets", pg.Graph.from_edges(np.concatenate(src).astype(np.uint32), np.concatenate(dst).astype(np.uint32),
                                         n, dedup=True)


@pytest.mark.parametrize("order,order_min,warp_rows", [(1, 128, 8192), (1, 128, 512), (1, 128, 1 << 30),
                                                       (1, 300, 8192), (1, 9000, 512), (0, 128, 8192)])
def test_hindex_ordered_rows(order, order_min, warp_rows):
    """Long rows read from the copy ordered by neighbour degree (prefix reads
    in the support test, the bucket-by-bucket histogram and the notification
    window), for the warp and CTA paths and with the copy limited to longer
    rows or off: the same core numbers as Batagelj-Zaversnik, twice in a row
    on the same graph."""
    for name, g in _hub_graphs():
        rp, col = g.csr()
        want, _ = oracle.bz(rp, col)
        g.set_param("hindex.order", order)
        g.set_param("hindex.order_min", order_min)
        g.set_param("hindex.warp_rows", warp_rows)
        for method in ("histo", "nbr"):
            got, _ = g.decompose(method)
            assert np.array_equal(got, want), (name, method)
        g.free()


def test_hindex_order_min_range():
    g = pg.rmat_graph(10, 8, seed=1)
    for bad in (0, 127, (1 << 30) + 1):
        with pytest.raises(pg.KCoreError):
            g.set_param("hindex.order_min", bad)
    g.set_param("hindex.order_min", 128)
    g.free()
