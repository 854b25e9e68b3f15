"""Parity of the CUDA engine with the oracle (bit-exact integer results),
through the C ABI.  Runs on the GB300."""
import numpy as np
import pytest

from oracle import gen as gen_ref
import oracle
import pico_gb300 as pg

pytestmark = pytest.mark.gpu

ALL = ["HistoCore", "CntCore", "NbrCore", "peelone", "gppeel", "peelone_dyn", "peel_dyn"]
CASES = ["example", "zero_based_dups", "dups_selfloops", "sparse_ids", "hub150", "er300", "rmat9",
         "clique40_path", "no_edges", "only_selfloops"]


def expected(method, core, rowptr):
    """The reference's output for `method` given the true core numbers."""
    if method == "gppeel":
        return np.where(np.diff(rowptr) == 0, 1, core).astype(np.uint32)
    return core


def check_all_methods(g, rowptr, col, methods=ALL):
    core, kmax = oracle.bz(rowptr, col)
    for m in methods:
        got, st = g.decompose(m)
        exp = expected(m, core, rowptr)
        assert got.shape == exp.shape
        bad = np.flatnonzero(got != exp)
        assert bad.size == 0, "%s: %d mismatches, first v=%d got %d want %d" % (
            m, bad.size, bad[0], got[bad[0]], exp[bad[0]])
        if g.n:
            assert st.kmax == int(exp.max())
            assert st.kmin == min(10, int(exp.min()))
    return core


def test_example_known_answer(golden, mtx_file):
    path = mtx_file(golden["example"]["text"])
    for mode in ("coo", "csr"):
        g = pg.Graph.from_mtx(path, mode)
        for m in ALL:
            core, st = g.decompose(m)
            assert core.tolist() == [2, 2, 2, 2, 2]
            assert st.kmax == 2 and st.kmin == 2
        g.free()


@pytest.mark.parametrize("name", CASES)
def test_golden_inputs_all_methods(golden, mtx_file, name):
    case = golden[name]
    path = mtx_file(case["text"])
    g = pg.Graph.from_mtx(path, "coo")
    coo = case["coo"]
    assert g.n == coo["n"] and g.nnz == 2 * coo["m"]
    rp, col = g.csr()
    core = check_all_methods(g, rp, col)
    assert core.tolist() == case["core_bz_coo"]
    if g.n:
        # the reference's virtual-graph layout, built on the device
        node_ptr, edge_list, parts = g.virtual_layout(64)
        assert node_ptr.tolist() == coo["node_pointer"]
        assert edge_list.tolist() == coo["edge_list"]
        assert parts.tolist() == coo["parts"]
    g.free()
    if "csr" in case:
        g = pg.Graph.from_mtx(path, "csr")
        rp, col = g.csr()
        assert g.n == case["csr"]["V"]
        assert rp.tolist() == case["csr"]["offsets"] and col.tolist() == case["csr"]["neighbors"]
        core = check_all_methods(g, rp, col)
        assert core.tolist() == case["core_bz_csr"]
        g.free()


def random_edges(rng, n, m):
    return rng.integers(0, n, size=m).astype(np.uint32), rng.integers(0, n, size=m).astype(np.uint32)


@pytest.mark.parametrize("seed", range(6))
def test_random_graphs_all_methods(seed):
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(50, 20000))
    m = int(rng.integers(n, 20 * n))
    s, d = random_edges(rng, n, m)
    g = pg.Graph.from_edges(s, d, n, dedup=True)
    rp, col = g.csr()
    erp, ecol = oracle.csr_dedup(n, s, d)
    assert np.array_equal(rp, erp) and np.array_equal(col, ecol)
    check_all_methods(g, rp, col)
    assert g.validate() == 0


def test_multigraph_keeps_parallel_edges_in_edge_order():
    rng = np.random.default_rng(5)
    n, m = 3000, 40000
    s, d = random_edges(rng, 300, m)  # many repeats
    g = pg.Graph.from_edges(s, d, n)
    rp, col = g.csr()
    erp, ecol = oracle.csr_multi(n, s, d)
    assert np.array_equal(rp, erp) and np.array_equal(col, ecol)
    check_all_methods(g, rp, col)


def test_sort_rows_without_dedup():
    rng = np.random.default_rng(6)
    s, d = random_edges(rng, 500, 20000)
    g = pg.Graph.from_edges(s, d, 500, sort_rows=True)
    rp, col = g.csr()
    erp, ecol = oracle.csr_multi(500, s, d)
    assert np.array_equal(rp, erp)
    for v in range(500):
        assert np.array_equal(col[rp[v]:rp[v + 1]], np.sort(ecol[erp[v]:erp[v + 1]]))


def test_structured_graphs():
    # star (one hub above the chunk size), long path (deep cascade within a
    # level), clique, disjoint union with isolated ids
    cases = []
    hub = 50000
    cases.append((hub + 1, np.zeros(hub, np.uint32), np.arange(1, hub + 1, dtype=np.uint32)))
    L = 200000
    cases.append((L, np.arange(L - 1, dtype=np.uint32), np.arange(1, L, dtype=np.uint32)))
    k = 300
    a, b = np.triu_indices(k, 1)
    cases.append((k, a.astype(np.uint32), b.astype(np.uint32)))
    s = np.concatenate([a, a + 1000, [5000]]).astype(np.uint32)
    d = np.concatenate([b, b + 1000, [5001]]).astype(np.uint32)
    cases.append((6000, s, d))
    for n, s, d in cases:
        g = pg.Graph.from_edges(s, d, n, dedup=True)
        rp, col = g.csr()
        check_all_methods(g, rp, col)
        g.free()


def test_hub_rows_large_sort_and_stable_order():
    # rows far above 4096 entries take the radix path of the row sort
    rng = np.random.default_rng(9)
    n = 70000
    s = np.concatenate([np.zeros(60000), rng.integers(0, n, 30000)]).astype(np.uint32)
    d = np.concatenate([rng.integers(1, n, 60000), rng.integers(0, n, 30000)]).astype(np.uint32)
    g = pg.Graph.from_edges(s, d, n, dedup=True)
    rp, col = g.csr()
    erp, ecol = oracle.csr_dedup(n, s, d)
    assert np.array_equal(rp, erp) and np.array_equal(col, ecol)
    g2 = pg.Graph.from_edges(s, d, n)
    rp2, col2 = g2.csr()
    erp2, ecol2 = oracle.csr_multi(n, s, d)
    assert np.array_equal(rp2, erp2) and np.array_equal(col2, ecol2)
    check_all_methods(g, rp, col, ["peelone_dyn", "NbrCore"])


def test_generators_match_host_restatement():
    s, d, m = pg.gen_rmat_edges(12, 20000, seed=42)
    es, ed = gen_ref.rmat(12, 20000, 42)
    assert np.array_equal(s.download(np.uint32, m), es) and np.array_equal(d.download(np.uint32, m), ed)
    s, d, m = pg.gen_er_edges(1000, 30000, seed=7)
    es, ed = gen_ref.er(1000, 30000, 7)
    gs, gd = s.download(np.uint32, m), d.download(np.uint32, m)
    assert np.array_equal(gs, es) and np.array_equal(gd, ed)
    assert (gs < gd).all() and np.unique(gs.astype(np.int64) * 1000 + gd).size == m  # without replacement
    s, d, m = pg.gen_planted_edges(100000, 60, 0.6, seed=3)
    es, ed = gen_ref.planted(100000, 60, 0.6, 3)
    assert m == es.size
    assert np.array_equal(s.download(np.uint32, m), es) and np.array_equal(d.download(np.uint32, m), ed)


def test_repeated_decompositions_and_device_output():
    g = pg.rmat_graph(14, 8, seed=1)
    rp, col = g.csr()
    core, _ = oracle.bz(rp, col)
    for _ in range(3):
        for m in ("peelone_dyn", "NbrCore", "gppeel"):
            got, _ = g.decompose(m)
            assert np.array_equal(got, expected(m, core, rp))
    g.decompose_device("peel_dyn")
    buf = pg.DeviceBuffer(4 * g.n)
    pg.check(pg.lib().kc_memcpy(pg.ctypes.c_void_p(buf.ptr), pg.ctypes.c_void_p(g.device_core()), 4 * g.n, 3))
    assert np.array_equal(buf.download(np.uint32, g.n), core)


def test_invalid_inputs_fail_with_status():
    with pytest.raises(pg.KCoreError) as e:
        pg.Graph.from_edges([0, 5], [1, 2], 3)
    assert e.value.code == pg.KC_ERR_INVALID
    g = pg.Graph.from_edges([0], [1], 2)
    with pytest.raises(pg.KCoreError) as e:
        pg.check(pg.lib().kc_decompose(g.handle, 99, None, 0, None, None))
    assert e.value.code == pg.KC_ERR_INVALID


def test_config1_er_65536_1m():
    g = pg.er_graph(65536, 1048576, seed=1)
    assert g.n == 65536 and g.nnz == 2 * 1048576
    rp, col = g.csr()
    check_all_methods(g, rp, col, ALL + ["auto"])
    assert g.validate() == 0


def test_config2_rmat22_ef16():
    g = pg.rmat_graph(22, 16, seed=2)
    rp, col = g.csr()
    assert g.n == 1 << 22 and g.validate() == 0
    core, kmax = oracle.bz(rp, col)
    # every method at full size (they share kernels, which is what this guards)
    for m in ALL + ["auto"]:
        got, st = g.decompose(m)
        want = expected(m, core, rp)
        assert np.array_equal(got, want), m
        assert st.kmax == kmax
    # the h-index sweeps race lowered estimates against pending-bit updates;
    # repeated runs vary the interleaving
    for _ in range(12):
        got, _ = g.decompose("histo")
        assert np.array_equal(got, core)


def test_config3_rmat25_planted_core():
    """R-MAT scale 25, edge factor 16, plus a planted 4000-vertex subgraph at
    p = 0.6: bit-exact against Batagelj-Zaversnik at full size."""
    g = pg.rmat_planted_graph(25, 16, 4000, 0.6, seed=3)
    assert g.n == 1 << 25 and g.nnz > 1_000_000_000
    got, st = g.decompose("peelone_dyn")
    rp, col = g.csr()
    core, kmax = oracle.bz(rp, col)
    assert np.array_equal(got, core)
    assert st.kmax == kmax and kmax >= 2000  # the planted core dominates
    for m in ALL:
        got, st = g.decompose(m)
        assert np.array_equal(got, expected(m, core, rp)), m
        assert st.kmax == kmax
    for _ in range(6):
        got_h, _ = g.decompose("NbrCore")
        assert np.array_equal(got_h, core)


def test_relabelling_and_local_core_property():
    """Relabelling the vertices permutes the core numbers, and the result
    passes the local k-core check (each vertex of core k has at least k
    neighbours of core >= k and is not in the (k+1)-core)."""
    rng = np.random.default_rng(17)
    g = pg.rmat_graph(15, 16, seed=9)
    rp, col = g.csr()
    n = g.n
    core, _ = g.decompose("peelone_dyn")
    assert oracle.check_local(rp, col, core) == 0
    perm = rng.permutation(n).astype(np.uint32)
    src = np.repeat(np.arange(n, dtype=np.uint32), np.diff(rp))
    h = pg.Graph.from_edges(perm[src], perm[col], n, dedup=True)
    for method in ("peelone_dyn", "histo", "gppeel"):
        c2, _ = h.decompose(method)
        want = np.where(np.diff(rp) == 0, 1, core) if method == "gppeel" else core
        assert np.array_equal(c2[perm], want), method
    g.free()
    h.free()


def test_hub_row_above_2_pow_24():
    """A hub whose row holds more than 2^24 entries (17 M leaves), joined to
    a 64-clique: every method against Batagelj-Zaversnik (cores 63 on the
    clique, 1 elsewhere)."""
    leaves = (1 << 24) + 1000
    a, b = np.triu_indices(64, 1)
    s = np.concatenate([np.zeros(leaves, np.uint32), a.astype(np.uint32) + 1 + leaves])
    d = np.concatenate([np.arange(1, leaves + 1, dtype=np.uint32), b.astype(np.uint32) + 1 + leaves])
    s = np.concatenate([s, np.zeros(64, np.uint32)])  # the hub also touches every clique vertex
    d = np.concatenate([d, np.arange(leaves + 1, leaves + 65, dtype=np.uint32)])
    n = leaves + 65
    g = pg.Graph.from_edges(s, d, n, dedup=True)
    rp, col = g.csr()
    assert int(np.diff(rp)[0]) == leaves + 64
    core, kmax = oracle.bz(rp, col)
    assert kmax == 64  # the hub joins the clique's core: 65 vertices of degree >= 64
    for method in ("peelone_dyn", "peel_dyn", "peelone", "gppeel", "histo", "cnt", "nbr"):
        got, st = g.decompose(method)
        assert np.array_equal(got, core), method
        assert st.kmax == kmax, method
    g.free()


def test_auto_method_is_tuned_per_graph_and_exact():
    """KC_AUTO: the first call times the peel variants and the h-index
    iteration on the graph and keeps the fastest; every call, first and
    later, gives the Batagelj-Zaversnik core numbers, and later calls run
    the method the tuner chose."""
    graphs = [pg.rmat_graph(16, 16, seed=3), pg.er_graph(20000, 200000, seed=4)]
    for g in graphs:
        rp, col = g.csr()
        want, _ = oracle.bz(rp, col)
        got, st = g.decompose("auto")
        assert np.array_equal(got, want)
        name, ms = g.autotune()
        assert name in pg.METHODS and name != "auto" and ms > 0
        got, st = g.decompose("auto")
        assert np.array_equal(got, want) and st.method == name
        g.free()
