"""The oracle itself, pinned before it is trusted: against the reference's
known answer (example.txt), against golden arrays produced by the reference's
own loader / virtual-graph code, against networkx, and the restated drivers
against Batagelj-Zaversnik on random graphs."""
import numpy as np
import pytest

import oracle


def test_example_known_answer(golden, mtx_file):
    case = golden["example"]
    n, s, d, has_zero = oracle.load_coo_reference(mtx_file(case["text"]))
    rp, col = oracle.csr_multi(n, s, d)
    core, kmax = oracle.bz(rp, col)
    assert core.tolist() == case["known_answer"] == [2, 2, 2, 2, 2]
    assert kmax == 2


@pytest.mark.parametrize("name", ["example", "zero_based_dups", "dups_selfloops", "sparse_ids", "hub150",
                                  "er300", "rmat9", "clique40_path", "no_edges", "only_selfloops"])
def test_loader_restatements_match_reference(golden, mtx_file, name):
    case = golden[name]
    path = mtx_file(case["text"])
    n, s, d, has_zero = oracle.load_coo_reference(path)
    coo = case["coo"]
    assert n == coo["n"] and len(s) == coo["m"] and has_zero == coo["has_zero"]
    assert s.tolist() == coo["src"] and d.tolist() == coo["dst"]
    node_ptr, edge_list, parts = oracle.make_ugraph(n, s, d, 64)
    assert node_ptr.tolist() == coo["node_pointer"]
    assert edge_list.tolist() == coo["edge_list"]
    assert parts.tolist() == coo["parts"]
    if "csr" in case:
        V, rp, col = oracle.load_csr_reference(path)
        csr = case["csr"]
        assert V == csr["V"]
        assert rp.tolist() == csr["offsets"] and col.tolist() == csr["neighbors"]
        assert np.diff(rp).tolist() == csr["degrees"]


@pytest.mark.parametrize("name", ["example", "dups_selfloops", "sparse_ids", "hub150", "er300", "rmat9",
                                  "clique40_path", "no_edges"])
def test_bz_matches_networkx_and_restated_drivers(golden, name):
    case = golden[name]
    if "csr" not in case:
        pytest.skip("0-based input: the CSR loader does not apply")
    rp = np.array(case["csr"]["offsets"], dtype=np.int64)
    col = np.array(case["csr"]["neighbors"], dtype=np.uint32)
    core, kmax = oracle.bz(rp, col)
    assert core.tolist() == case["core_networkx_csr"] == case["core_bz_csr"]
    assert oracle.hindex_jacobi(rp, col)[0].tolist() == core.tolist()
    assert oracle.peel_rounds(rp, col)[0].tolist() == core.tolist()
    assert oracle.peel_dyn(rp, col)[0].tolist() == core.tolist()
    gpp = oracle.gpp(rp, col)[0]
    expect = np.where(np.diff(rp) == 0, 1, core)
    assert gpp.tolist() == expect.tolist()
    assert oracle.check_local(rp, col, core) == 0


def test_multigraph_coo_semantics(golden):
    # the COO loader keeps duplicate lines: parallel edges count in degrees
    for name in ("zero_based_dups", "dups_selfloops", "rmat9"):
        case = golden[name]
        coo = case["coo"]
        rp, col = oracle.csr_multi(coo["n"], coo["src"], coo["dst"])
        core, _ = oracle.bz(rp, col)
        assert core.tolist() == case["core_bz_coo"]
        assert oracle.hindex_jacobi(rp, col)[0].tolist() == core.tolist()
        assert oracle.peel_dyn(rp, col)[0].tolist() == core.tolist()
        assert np.diff(rp).tolist() == coo["out_degree"]


def _random_graph(rng, n, m):
    s = rng.integers(0, n, size=m)
    d = rng.integers(0, n, size=m)
    return oracle.csr_dedup(n, s.astype(np.uint32), d.astype(np.uint32))


@pytest.mark.parametrize("seed", range(12))
def test_restated_drivers_agree_on_random_graphs(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 400))
    m = int(rng.integers(0, 6 * n))
    rp, col = _random_graph(rng, n, m)
    core, _ = oracle.bz(rp, col)
    assert oracle.hindex_jacobi(rp, col)[0].tolist() == core.tolist()
    assert oracle.peel_rounds(rp, col)[0].tolist() == core.tolist()
    assert oracle.peel_dyn(rp, col)[0].tolist() == core.tolist()
    assert oracle.check_local(rp, col, core) == 0


def test_networkx_cross_check_random():
    nx = pytest.importorskip("networkx")
    rng = np.random.default_rng(7)
    for _ in range(5):
        n = int(rng.integers(5, 300))
        rp, col = _random_graph(rng, n, 4 * n)
        g = nx.Graph()
        g.add_nodes_from(range(n))
        for v in range(n):
            for u in col[rp[v]:rp[v + 1]]:
                g.add_edge(v, int(u))
        cn = nx.core_number(g)
        assert oracle.bz(rp, col)[0].tolist() == [cn[v] for v in range(n)]


def test_check_local_detects_errors():
    rng = np.random.default_rng(3)
    rp, col = _random_graph(rng, 200, 1500)
    core, _ = oracle.bz(rp, col)
    bad = core.copy()
    v = int(np.argmax(core))
    bad[v] += 1  # planted mistake, in the oracle's input, on the CPU
    assert oracle.check_local(rp, col, bad) > 0


def test_hindex_iteration_counts_match_reference_trajectory(golden):
    # example.txt: Jacobi sweeps change {0,4}, then {1,2}, then nothing -> 3
    case = golden["example"]
    rp = np.array(case["csr"]["offsets"], dtype=np.int64)
    col = np.array(case["csr"]["neighbors"], dtype=np.uint32)
    assert oracle.hindex_jacobi(rp, col)[1] == 3
    assert oracle.peel_dyn(rp, col)[1] == 3  # levels 0, 1, 2


def test_rmat_restatements_agree():
    from oracle import gen
    s1, d1 = gen.rmat_numpy(16, 5000, 9)
    s2, d2 = gen.rmat(16, (1 << 20) + 7, 9)
    assert np.array_equal(s1, s2[:5000]) and np.array_equal(d1, d2[:5000])


def test_threaded_host_builders_equal_serial():
    """The multi-threaded R-MAT generator and CSR build (used to build the
    billion-entry graphs of the CPU benchmark arm) give exactly the serial
    results, including rows long enough for the radix path and self-loops."""
    from oracle import gen
    s1, d1 = gen.rmat(16, (1 << 20) + 12345, 7)
    s4, d4 = gen.rmat(16, (1 << 20) + 12345, 7, threads=4)
    assert np.array_equal(s1, s4) and np.array_equal(d1, d4)
    rp1, c1 = oracle.csr_dedup(1 << 16, s1, d1)
    for t in (2, 5):
        rp, c = oracle.csr_dedup(1 << 16, s1, d1, threads=t)
        assert np.array_equal(rp, rp1) and np.array_equal(c, c1)
    rp0, c0 = oracle.csr_dedup(5, np.array([], np.uint32), np.array([], np.uint32), threads=3)
    assert rp0.tolist() == [0] * 6 and c0.size == 0
