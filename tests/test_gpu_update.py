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
    g.set_param("update.deletion_incremental_max", incremental_max)
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
    # the full path (ids checked on the device) rejects them too and leaves
    # the graph as it was
    g.set_param("update.incremental_max", 0)
    g.set_param("update.deletion_incremental_max", 0)
    for ins, dels in ((([0], [7]), None), (None, ([0], [9])), (([0], [2]), ([5], [1]))):
        with pytest.raises(pg.KCoreError) as e:
            g.update(ins, dels)
        assert e.value.code == pg.KC_ERR_INVALID
    rp, col = g.csr()
    assert list(rp) == [0, 1, 3, 4] and list(col) == [1, 0, 2, 1]
    core, st = g.update(([0], [2]), None)
    assert list(core) == [2, 2, 2] and st["recomputed"] == 1
    h = pg.Graph.from_edges([0, 0, 1], [1, 1, 2], 3)  # parallel edge kept
    with pytest.raises(pg.KCoreError) as e:
        h.update(([0], [2]), None)
    assert e.value.code == pg.KC_ERR_UNSUPPORTED


def c5_batch(rng, keys, n, size):
    """One edge-update batch of the dynamic-serving configuration: `size`
    edges, half insertions (uniform vertex pairs that are neither self-loops
    nor current edges) and half deletions (drawn uniformly, without
    replacement, from the current edge set)."""
    ni = size // 2
    nd = size - ni
    dpos = np.unique(rng.integers(0, keys.size, size=2 * nd))
    rng.shuffle(dpos)
    dk = keys[dpos[:nd]]
    ins = np.zeros(0, np.uint64)
    while ins.size < ni:
        a = rng.integers(0, n, size=2 * ni, dtype=np.uint64)
        b = rng.integers(0, n, size=2 * ni, dtype=np.uint64)
        k = (np.minimum(a, b) << np.uint64(32)) | np.maximum(a, b)
        k = k[a != b]
        p = np.searchsorted(keys, k)
        k = k[~((p < keys.size) & (keys[np.minimum(p, keys.size - 1)] == k))]
        ins = np.unique(np.concatenate([ins, k]))
    ins = rng.permutation(ins)[:ni]
    split = lambda kk: ((kk >> np.uint64(32)).astype(np.uint32), (kk & np.uint64(0xffffffff)).astype(np.uint32))
    return split(ins), split(dk), ins, dk


def row_keys(rp, col):
    """Keys (u << 32 | v, u < v) of a CSR with sorted rows, in row order."""
    n = rp.size - 1
    src = np.repeat(np.arange(n, dtype=np.uint64), np.diff(rp))
    m = src < col
    return (src[m] << np.uint64(32)) | col[m].astype(np.uint64)


@pytest.mark.parametrize("mode", ["default", "incremental"])
def test_c5_rmat22_update_batches_exact(mode):
    """The dynamic-serving configuration: an R-MAT scale-22 base graph
    (edge factor 16, seed 2) receives update batches of floor(10^U(3,6))
    edges, 50/50 insert/delete.  After every batch the CSR holds exactly the
    expected edge set and the core numbers equal Batagelj-Zaversnik on the
    updated graph.  "incremental" raises update.incremental_max so that
    batches of 10^3-10^4 edges take the incremental path."""
    rng = np.random.default_rng(55 if mode == "default" else 56)
    g = pg.rmat_graph(22, 16, 2)
    n = g.n
    if mode == "incremental":
        g.set_param("update.incremental_max", 20000)
        sizes = np.floor(10.0 ** rng.uniform(3.0, 4.0, 4)).astype(np.int64)
    else:
        sizes = np.floor(10.0 ** rng.uniform(3.0, 6.0, 5)).astype(np.int64)
    g.decompose("peelone_dyn")
    rp, col = g.csr()
    keys = row_keys(rp, col)
    for step, size in enumerate(sizes):
        ins, dels, ik, dk = c5_batch(rng, keys, n, int(size))
        core, st = g.update(ins, dels)
        assert st["inserted"] == ik.size and st["deleted"] == dk.size, (step, st)
        # default threshold (512 edges): every batch of 10^3 or more edges is a
        # rewrite plus a full decomposition
        assert st["recomputed"] == (0 if mode == "incremental" else 1), (step, size, st)
        rp, col = g.csr()
        new_keys = row_keys(rp, col)
        assert (new_keys[1:] > new_keys[:-1]).all()  # rows sorted, no repeated neighbours
        assert new_keys.size == keys.size + ik.size - dk.size
        p = np.searchsorted(new_keys, ik)
        assert (new_keys[np.minimum(p, new_keys.size - 1)] == ik).all()
        p = np.searchsorted(new_keys, dk)
        assert not ((p < new_keys.size) & (new_keys[np.minimum(p, new_keys.size - 1)] == dk)).any()
        want, _ = oracle.bz(rp, col)
        bad = np.flatnonzero(core != want)
        assert bad.size == 0, (step, int(size), bad.size, st)
        keys = new_keys
    g.free()


def test_incremental_deletions_below_old_core():
    """A deletion batch can leave a vertex with fewer edges than its old core
    number, the upper bound the incremental path starts from: two vertices of
    a 700-clique (core 699) keep 49 and 19 of their edges, so their rows take
    the short-row paths of the h-index with estimates far above the row
    length.  Also 30% of an R-MAT graph's edges deleted in one incremental
    batch.  Both exact against Batagelj-Zaversnik on the updated graph."""
    k = 700
    a, b = np.triu_indices(k, 1)
    g = pg.Graph.from_edges(a.astype(np.uint32), b.astype(np.uint32), k, dedup=True)
    g.decompose("peelone_dyn")
    g.set_param("update.incremental_max", 1 << 30)
    ds = np.concatenate([np.zeros(650), np.ones(680)]).astype(np.uint32)
    dd = np.concatenate([np.arange(50, 700), np.arange(20, 700)]).astype(np.uint32)
    core, st = g.update(dels=(ds, dd))
    assert st["recomputed"] == 0
    rp, col = g.csr()
    assert rp[1] - rp[0] == 49 and rp[2] - rp[1] == 19
    want, _ = oracle.bz(rp, col)
    assert np.array_equal(core, want)
    g.free()

    g = pg.rmat_graph(14, 16, seed=21)
    rp, col = g.csr()
    src = np.repeat(np.arange(g.n, dtype=np.uint32), np.diff(rp))
    upper = src < col
    es, ed = src[upper], col[upper]
    pick = np.random.default_rng(5).choice(es.size, size=int(0.3 * es.size), replace=False)
    g.decompose("peelone_dyn")
    g.set_param("update.incremental_max", 1 << 30)
    core, st = g.update(dels=(es[pick], ed[pick]))
    assert st["recomputed"] == 0
    rp, col = g.csr()
    want, _ = oracle.bz(rp, col)
    assert np.array_equal(core, want)
    g.free()


def test_deletion_batches_incremental_by_default():
    """Batches of deletions only take the incremental path up to
    update.deletion_incremental_max edges (default 500,000), mixed batches
    only up to update.incremental_max (512); both exact."""
    rng = np.random.default_rng(8)
    g = pg.rmat_graph(15, 16, seed=4)
    g.decompose("peelone_dyn")
    rp, col = g.csr()
    keys = edge_keys(rp, col)
    ins, dels = random_batch(rng, keys, g.n, 0, 20000)
    core, st = g.update(ins, dels)
    assert st["recomputed"] == 0 and st["deleted"] == 20000
    rp, col = g.csr()
    assert np.array_equal(core, oracle.bz(rp, col)[0])
    keys = edge_keys(rp, col)
    ins, dels = random_batch(rng, keys, g.n, 1000, 1000)
    core, st = g.update(ins, dels)
    assert st["recomputed"] == 1
    rp, col = g.csr()
    assert np.array_equal(core, oracle.bz(rp, col)[0])
    g.set_param("update.deletion_incremental_max", 100)
    keys = edge_keys(rp, col)
    ins, dels = random_batch(rng, keys, g.n, 0, 1000)
    core, st = g.update(ins, dels)
    assert st["recomputed"] == 1
    g.free()
