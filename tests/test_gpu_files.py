"""Graph files and result extraction: binary snapshots (checked by a content
hash), binary edge-list input, and the induced k-core subgraph."""
import numpy as np
import pytest

import oracle
import pico_gb300 as pg

pytestmark = pytest.mark.gpu


def test_snapshot_round_trip_with_cores(tmp_path):
    g = pg.rmat_graph(14, 8, seed=9)
    core, _ = g.decompose("peelone_dyn")
    p = tmp_path / "g.kcs"
    g.save(str(p))
    h = pg.Graph.load(str(p))
    rp, col = g.csr()
    rp2, col2 = h.csr()
    assert np.array_equal(rp, rp2) and np.array_equal(col, col2)
    assert np.array_equal(h.core(), core)  # restored without a new decomposition
    assert np.array_equal(h.decompose("histo")[0], core)
    g.free()
    h.free()


def test_snapshot_without_cores(tmp_path):
    g = pg.er_graph(3000, 20000, seed=2)
    p = tmp_path / "g.kcs"
    g.save(str(p))
    h = pg.Graph.load(str(p))
    with pytest.raises(pg.KCoreError) as e:
        h.device_core()
    assert e.value.code == pg.KC_ERR_STATE
    assert np.array_equal(h.decompose()[0], oracle.bz(*g.csr())[0])
    g.free()
    h.free()


def test_snapshot_rejects_damaged_files(tmp_path):
    g = pg.er_graph(2000, 9000, seed=3)
    g.decompose()
    p = tmp_path / "g.kcs"
    g.save(str(p))
    data = bytearray(p.read_bytes())
    flipped = tmp_path / "flipped.kcs"
    bad = bytearray(data)
    bad[len(bad) // 2] ^= 0x10
    flipped.write_bytes(bytes(bad))
    short = tmp_path / "short.kcs"
    short.write_bytes(bytes(data[:-4]))
    other = tmp_path / "other.kcs"
    other.write_bytes(b"%%MatrixMarket\n" + bytes(100))
    for path in (flipped, short, other, tmp_path / "missing.kcs"):
        with pytest.raises(pg.KCoreError) as e:
            pg.Graph.load(str(path))
        assert e.value.code == pg.KC_ERR_IO, path
    g.free()


def test_edge_file_matches_edge_arrays(tmp_path):
    rng = np.random.default_rng(12)
    n = 20000
    s = rng.integers(0, n, 150000).astype(np.uint32)
    d = rng.integers(0, n, 150000).astype(np.uint32)
    d[-1] = n - 1  # the largest id sets n
    p = tmp_path / "edges.bin"
    np.stack([s, d], axis=1).astype("<u4").tofile(p)
    a = pg.Graph.from_edge_file(str(p), dedup=True)
    b = pg.Graph.from_edges(s, d, n, dedup=True)
    assert a.n == n
    ra, ca = a.csr()
    rb, cb = b.csr()
    assert np.array_equal(ra, rb) and np.array_equal(ca, cb)
    assert np.array_equal(a.decompose()[0], oracle.bz(ra, ca)[0])
    empty = tmp_path / "empty.bin"
    empty.write_bytes(b"")
    e = pg.Graph.from_edge_file(str(empty))
    assert e.n == 0 and e.nnz == 0
    odd = tmp_path / "odd.bin"
    odd.write_bytes(bytes(12))
    with pytest.raises(pg.KCoreError):
        pg.Graph.from_edge_file(str(odd))
    a.free()
    b.free()
    e.free()


def induced(rp, col, keep):
    n = rp.size - 1
    newid = np.cumsum(keep) - 1
    rows = []
    for v in np.flatnonzero(keep):
        nb = col[rp[v]:rp[v + 1]]
        rows.append(newid[nb[keep[nb]]].astype(np.uint32))
    nrp = np.zeros(len(rows) + 1, dtype=np.int64)
    np.cumsum([r.size for r in rows], out=nrp[1:])
    return nrp, (np.concatenate(rows) if rows else np.zeros(0, np.uint32)), np.flatnonzero(keep).astype(np.uint32)


@pytest.mark.parametrize("k", [0, 1, 3, 8, 1000])
def test_kcore_subgraph(k):
    g = pg.rmat_graph(13, 8, seed=4)
    core, st = g.decompose("peelone_dyn")
    sub, ids = g.kcore_subgraph(k)
    rp, col = g.csr()
    nrp, ncol, nids = induced(rp, col, core >= k)
    assert sub.n == nids.size and np.array_equal(ids, nids)
    srp, scol = sub.csr()
    assert np.array_equal(srp, nrp) and np.array_equal(scol, ncol)
    if sub.n:
        # the k-core keeps the core numbers of its vertices
        sc, _ = sub.decompose("peelone_dyn")
        assert np.array_equal(sc, core[ids])
        assert int(sc.min()) >= k
    sub.free()
    g.free()


def test_kcore_subgraph_needs_a_decomposition():
    g = pg.er_graph(500, 2000, seed=1)
    with pytest.raises(pg.KCoreError) as e:
        g.kcore_subgraph(2)
    assert e.value.code == pg.KC_ERR_STATE
    g.free()
