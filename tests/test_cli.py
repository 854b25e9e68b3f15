"""CLI drivers keep the reference binaries' command-line contract and report
lines; the Python mirror keeps ``int method(Graph&)`` of ``peel/main.cu``."""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
from pico_gb300 import build as pb

H2C = ("HistoCore", "CntCore", "NbrCore", "peelone", "gppeel")


def _bin(name):
    p = os.path.join(pb.BIN, name)
    if not os.access(p, os.X_OK):
        pytest.skip("CLI %s not built" % name)
    return p


@pytest.mark.parametrize("name", H2C)
def test_help_on_wrong_argc(name):
    # argument::Parse: anything but exactly one argument prints help, exits 0
    for argv in ([], ["a.mtx", "b.mtx"]):
        r = subprocess.run([_bin(name)] + argv, capture_output=True, text=True, timeout=60)
        assert r.returncode == 0
        assert "Required arguments:" in r.stdout and "[--input]" in r.stdout


def test_peel_main_usage():
    r = subprocess.run([_bin("peelone_dyn")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 255
    assert r.stdout.strip() == "./kcore file deviceID Repeattime"


def test_missing_file_fails_without_crash(tmp_path):
    r = subprocess.run([_bin("HistoCore"), str(tmp_path / "none.mtx")], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1 and "load:" in r.stderr


def _graph_text(seed=3, n=400, m=3000):
    rng = np.random.default_rng(seed)
    s = rng.integers(1, n + 1, m)
    d = rng.integers(1, n + 1, m)
    # a 12-clique so kmax is not tiny
    cl = [(a, b) for a in range(1, 13) for b in range(a + 1, 13)]
    lines = ["%%MatrixMarket matrix coordinate pattern symmetric", f"{n} {n} {m + len(cl)}"]
    lines += [f"{a} {b}" for a, b in zip(s, d)] + [f"{a} {b}" for a, b in cl]
    return "\n".join(lines) + "\n"


@pytest.mark.gpu
@pytest.mark.parametrize("name", H2C)
def test_cli_report_matches_bz(name, mtx_file, tmp_path):
    path = mtx_file(_graph_text())
    out = tmp_path / "res.txt"
    env = dict(os.environ, KCORE_OUTPUT=str(out))
    r = subprocess.run([_bin(name), path], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    n, src, dst = oracle.load_coo_reference(path)[:3]
    rowptr, col = oracle.csr_multi(n, src, dst)
    ref = oracle.bz(rowptr, col)[0]
    if name == "gppeel":
        deg = np.diff(rowptr)
        ref = np.where(deg == 0, 1, ref)
    assert f"Number of nodes = {n}" in r.stdout
    assert re.search(r"Number of iterations = \d+", r.stdout)
    assert re.search(r"Processing finished in [0-9.e+-]+ \(ms\)\.", r.stdout)
    assert f" Max K = {int(ref.max())}\n" in r.stdout
    assert f" Min K = {min(10, int(ref.min()))}\n" in r.stdout
    got = np.loadtxt(out, dtype=np.int64).reshape(-1, 2)
    assert np.array_equal(got[:, 0], np.arange(n))
    assert np.array_equal(got[:, 1], ref)


@pytest.mark.gpu
def test_peel_main_report(mtx_file):
    path = mtx_file(_graph_text(seed=5))
    r = subprocess.run([_bin("peelone_dyn"), path], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    V, rowptr, col = oracle.load_csr_reference(path)[:3]
    ref = oracle.bz(rowptr, col)[0]
    deg = np.diff(rowptr)
    assert f"V: {V}\n" in r.stdout
    assert f"E: {len(col) // 2}\n" in r.stdout
    assert f" Maxdegree = {int(deg.max())}\n" in r.stdout
    std = float(r.stdout.split("STD: \n")[1].split("\n")[0])
    assert std == pytest.approx(float(np.std(deg)), rel=1e-5)
    for tag in ("ICDE23_peel: ", "Our_Paper_peel: "):
        line = r.stdout.split(tag)[1].split("\n")[0]
        assert len(re.findall(r"\d+ms ", line)) == 10 and " ave: " in line
    assert r.stdout.count(f"Kmax: {int(ref.max())}\n") == 2


@pytest.mark.gpu
def test_python_reference_mirror(mtx_file, tmp_path):
    import json
    from pico_gb300 import reference as R
    path = mtx_file(_graph_text(seed=7))
    g = R.Graph(path)
    V, rowptr, col = oracle.load_csr_reference(path)[:3]
    ref = oracle.bz(rowptr, col)[0]
    assert (g.V, g.E, g.dmax) == (V, len(col), int(np.diff(rowptr).max()))
    assert np.array_equal(g.neighbors_offset, rowptr) and np.array_equal(g.neighbors, col)
    for kern in (R.peel_dyn, R.peelone_dyn, R.peelone, R.gppeel, R.histo_core, R.cnt_core, R.nbr_core):
        g.kmax = 0
        t = kern(g)
        assert isinstance(t, int) and t >= 0
        assert g.kmax == int(ref.max())
    lines = []
    avg = R.rep_simulation(R.peelone_dyn, g, out=lines.append)
    assert avg >= 0 and lines[0].count("ms ") == 10
    assert np.array_equal(g.core, ref)
    assert R.std_degrees(g) == pytest.approx(float(np.std(np.diff(rowptr))))
    out = tmp_path / "kcore.json"
    g.write_kcore_to_disk(str(out))
    d = json.loads(out.read_text())
    nz = np.flatnonzero(np.diff(rowptr))
    assert d == {str(i): int(ref[i]) for i in nz}
    g.free()
