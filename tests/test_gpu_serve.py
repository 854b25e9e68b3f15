"""The request server: continuous batching, admission by device memory, and
results that are the same whether a request runs alone or in the mix."""
import numpy as np
import pytest

import oracle
import pico_gb300 as pg
from pico_gb300 import workloads

pytestmark = pytest.mark.gpu


def base_graph():
    return pg.rmat_graph(14, 8, seed=33)


def stream(num=40, seed=8):
    g = base_graph()
    rp, col = g.csr()
    g.free()
    return workloads.serve_stream(rp, col, num, seed=seed, rate_hz=1e4, batch_log=(2.0, 3.5),
                                  graph_log_n=(1.5, 3.5))


def test_results_same_alone_and_in_the_mix():
    reqs = stream()
    # in the mix: everything submitted at once, lanes overlap and pack requests
    g1 = base_graph()
    s1 = pg.Server(g1, decompose_slots=3, max_batch_graphs=8)
    mixed = workloads.run_stream(s1, reqs, realtime=False)
    st = s1.stats()
    s1.close()
    # alone: one request at a time on a fresh copy of the resident graph
    g2 = base_graph()
    s2 = pg.Server(g2, decompose_slots=1, max_batch_graphs=1)
    alone = [workloads.run_stream(s2, [r], realtime=False)[0] for r in reqs]
    s2.close()
    assert [r["digest"] for r in mixed] == [r["digest"] for r in alone]
    assert [r["kmax"] for r in mixed] == [r["kmax"] for r in alone]
    assert st["completed_updates"] + st["completed_decompositions"] == len(reqs)
    # the resident graphs ended in the same state, with exact cores
    rp1, col1 = g1.csr()
    rp2, col2 = g2.csr()
    assert np.array_equal(rp1, rp2) and np.array_equal(col1, col2)
    core, _ = g1.decompose("peelone_dyn")
    assert np.array_equal(core, oracle.bz(rp1, col1)[0])


def test_decompose_results_exact_and_packed():
    reqs = [r for r in stream(60, seed=3) if r["kind"] == "decompose"]
    g = base_graph()
    s = pg.Server(g, decompose_slots=1, max_batch_graphs=16)
    tickets = [s.submit_decompose(r["rowptr"], r["col"]) for r in reqs]
    for r, tk in zip(reqs, tickets):
        res = s.wait(tk, core_cap=r["rowptr"].size - 1)
        core, _ = oracle.bz(r["rowptr"], r["col"])
        assert np.array_equal(res["core"], core)
    st = s.stats()
    s.close()
    assert st["completed_decompositions"] == len(reqs)
    assert st["decompose_launches"] < len(reqs)  # waiting requests were packed together


def test_update_with_core_snapshot():
    g = base_graph()
    rp, col = g.csr()
    s = pg.Server(g)
    reqs = [r for r in workloads.serve_stream(rp, col, 10, seed=4, update_frac=1.0, batch_log=(2, 3))]
    res = workloads.run_stream(s, reqs, realtime=False, want_core=True)
    s.close()
    assert all(r["status"] == 0 and r["kind"] == 0 for r in res)
    rp2, col2 = g.csr()
    core, _ = oracle.bz(rp2, col2)
    last = res[-1]
    assert last["kmax"] == int(core.max())


def test_admission_rejects_what_cannot_fit():
    g = base_graph()
    s = pg.Server(g, hbm_reserve_bytes=1 << 50)
    rp, col = workloads.graph_csr_host(workloads.KIND_ER, 200, 800, 1)
    tk = s.submit_decompose(rp, col)
    with pytest.raises(pg.KCoreError) as e:
        s.wait(tk)
    assert e.value.code == pg.KC_ERR_NOMEM
    assert s.stats()["failed"] == 1
    s.close()
