"""Exact core maintenance under edge batches (kc_graph_update): after every
batch the CSR equals the expected edge set and the core numbers equal
Batagelj-Zaversnik on the updated graph."""
import numpy as np
import pytest

import oracle
import pico_gb300 as pg

pytestmark = pytest.mark.gpu


def edge_keys(rp, col):
    n = rp.size - 1
    src = np.repeat(np.arange(n, dtype=np.uint64), np.diff(rp))
    dst = col.astype(np.uint64)
    m = src < dst
    return np.sort((src[m] << np.uint64(32)) | dst[m])


def random_batch(rng, keys, n, n_ins, n_del):
    dk = rng.choice(keys, size=min(n_del, keys.size), replace=False) if n_del else np.zeros(0, np.uint64)
    a = rng.integers(0, n, size=n_ins).astype(np.uint64)
    b = rng.integers(0, n, size=n_ins).astype(np.uint64)
    return (a.astype(np.uint32), b.astype(np.uint32)), ((dk >> np.uint64(32)).astype(np.uint32),
                                                         (dk & np.uint64(0xffffffff)).astype(np.uint32))


def expected_keys(keys, ins, dels):
    dk = np.minimum(dels[0], dels[1]).astype(np.uint64) << np.uint64(32) | np.maximum(dels[0], dels[1]).astype(np.uint64)
    keep = keys[~np.isin(keys, dk)]
    a, b = ins
    ok = a != b
    ik = np.minimum(a, b)[ok].astype(np.uint64) << np.uint64(32) | np.maximum(a, b)[ok].astype(np.uint64)
    return np.union1d(keep, ik)


@pytest.mark.parametrize("incremental_max", [1 << 30, 0])
def test_update_batches_exact(incremental_max):
    rng = np.random.default_rng(12)
    g = pg.rmat_graph(14, 8, seed=21)
    g.set_param("update.incremental_max", incremental_max)
    n = g.n
    g.decompose("peelone_dyn")
    for step, (ni, nd) in enumerate([(0, 300), (300, 0), (500, 500), (2000, 1500), (1, 1), (0, 0), (40, 4000)]):
        rp, col = g.csr()
        keys = edge_keys(rp, col)
        ins, dels = random_batch(rng, keys, n, ni, nd)
        want_keys = expected_keys(keys, ins, dels)
        core, st = g.update(ins, dels)
        rp2, col2 = g.csr()
        assert np.array_equal(edge_keys(rp2, col2), want_keys), step
        assert all((np.diff(col2[rp2[v]:rp2[v + 1]].astype(np.int64)) > 0).all() for v in range(0, n, 97))
        ref, _ = oracle.bz(rp2, col2)
        assert np.array_equal(core, ref), (step, st)
        assert st["recomputed"] == (0 if incremental_max else 1) or (ni + nd == 0)
    # the graph keeps working as a normal graph
    got, _ = g.decompose("NbrCore")
    assert np.array_equal(got, ref)


def test_insertions_raising_cores_through_subcores():
    # a path of triangles: inserting chords raises whole chains of cores
    n = 3000
    s = np.arange(n - 1, dtype=np.uint32)
    d = s + 1
    g = pg.Graph.from_edges(s, d, n, dedup=True)
    g.decompose("peelone_dyn")
    rng = np.random.default_rng(2)
    for _ in range(4):
        a = rng.integers(0, n - 2, 400).astype(np.uint32)
        core, st = g.update((a, a + 2), None)
        rp, col = g.csr()
        assert np.array_equal(core, oracle.bz(rp, col)[0])
        assert st["rounds"] >= 1


def test_delete_and_reinsert_same_edge_keeps_it():
    g = pg.Graph.from_edges([0, 1, 2, 0], [1, 2, 0, 3], 4, dedup=True)
    g.decompose("peelone_dyn")
    core, st = g.update(([0], [1]), ([1], [0]))
    rp, col = g.csr()
    assert 1 in col[rp[0]:rp[1]].tolist()
    assert core.tolist() == [2, 2, 2, 1]


def test_update_rejects_bad_ids_and_multigraphs():
    g = pg.Graph.from_edges([0, 1], [1, 2], 3, dedup=True)
    with pytest.raises(pg.KCoreError) as e:
        g.update(([0], [7]), None)
    assert e.value.code == pg.KC_ERR_INVALID
    h = pg.Graph.from_edges([0, 0, 1], [1, 1, 2], 3)  # parallel edge kept
    with pytest.raises(pg.KCoreError) as e:
        h.update(([0], [2]), None)
    assert e.value.code == pg.KC_ERR_UNSUPPORTED
