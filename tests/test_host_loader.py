"""The product's host MatrixMarket loader (libkcore.so, no GPU needed) against
the golden arrays of the reference's own loaders."""
import numpy as np
import pytest

import pico_gb300 as pg

CASES = ["example", "zero_based_dups", "dups_selfloops", "sparse_ids", "hub150", "er300", "rmat9",
         "clique40_path", "no_edges", "only_selfloops"]


@pytest.mark.parametrize("name", CASES)
def test_coo_loader_matches_readgraph(golden, mtx_file, name):
    case = golden[name]
    n, s, d = pg.parse_mtx(mtx_file(case["text"]), "coo")
    coo = case["coo"]
    assert n == coo["n"]
    assert s.tolist() == coo["src"] and d.tolist() == coo["dst"]


@pytest.mark.parametrize("name", [c for c in CASES if c != "zero_based_dups"])
def test_csr_loader_vertex_count_matches_readfile(golden, mtx_file, name):
    case = golden[name]
    n, s, d = pg.parse_mtx(mtx_file(case["text"]), "csr")
    assert n == case["csr"]["V"]
    assert (s < n).all() and (d < n).all() and (s != d).all()


def test_comment_lines_and_blank_lines(mtx_file):
    text = "%%MatrixMarket matrix coordinate integer symmetric\n% a comment\n%another\n4 4 3\n\n1 2\n2 3 7\n3 4\n"
    n, s, d = pg.parse_mtx(mtx_file(text), "coo")
    # the size line "4 4 3" is a self-loop and is dropped, as in the reference
    assert n == 4 and s.tolist() == [0, 1, 2] and d.tolist() == [1, 2, 3]


def test_malformed_line_is_an_error(mtx_file):
    text = "%%MatrixMarket matrix coordinate integer symmetric\n3 3 2\n1 2\n1 x\n"
    with pytest.raises(pg.KCoreError) as e:
        pg.parse_mtx(mtx_file(text), "coo")
    assert e.value.code == pg.KC_ERR_INVALID and ":4:" in str(e.value)


def test_missing_file_is_io_error(tmp_path):
    with pytest.raises(pg.KCoreError) as e:
        pg.parse_mtx(str(tmp_path / "nope.mtx"), "coo")
    assert e.value.code == pg.KC_ERR_IO


def test_csr_mode_rejects_zero_id(golden, mtx_file):
    with pytest.raises(pg.KCoreError) as e:
        pg.parse_mtx(mtx_file(golden["zero_based_dups"]["text"]), "csr")
    assert e.value.code == pg.KC_ERR_INVALID


def test_large_parallel_parse_keeps_file_order(mtx_file):
    rng = np.random.default_rng(11)
    m = 400_000
    s = rng.integers(1, 50_000, size=m)
    d = rng.integers(1, 50_000, size=m)
    lines = ["%%MatrixMarket matrix coordinate integer symmetric", "50000 50000 %d" % m]
    lines += ["%d %d 1" % (a, b) for a, b in zip(s, d)]
    n, ps, pd = pg.parse_mtx(mtx_file("\n".join(lines) + "\n"), "coo")
    keep = s != d
    assert n == max(s.max(), d.max())
    assert ps.tolist() == (s[keep] - 1).tolist() and pd.tolist() == (d[keep] - 1).tolist()
