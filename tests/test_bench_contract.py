"""The JSON line of `bench.py --impl reference` (the reference's CPU path on
the host cores): one line with the keys the benchmark contract names, on the
small Erdos-Renyi workload so that it runs in seconds without a GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "er65536", "--steps", "2", "--warmup", "3"], capture_output=True, text=True, timeout=600,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 2 and d["warmup"] == 3
    assert d["value"] > 0 and d["unit"] == "M edges/s" and d["higher_is_better"] is True
    assert d["vs_baseline"] is None and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_serving_exactness_replay_detects_a_wrong_result():
    """bench.serve_exact replays the update stream on the host edge set and
    compares each served digest with Batagelj-Zaversnik; one wrong digest
    makes the whole check fail."""
    import numpy as np

    import oracle
    sys.path.insert(0, ROOT)
    import bench
    from pico_gb300 import workloads
    rng = np.random.default_rng(1)
    n = 2000
    rp, col = oracle.csr_dedup(n, rng.integers(0, n, 20000).astype(np.uint32),
                               rng.integers(0, n, 20000).astype(np.uint32))
    cur = workloads.edge_keys(rp, col)
    split = lambda k: ((k >> np.uint64(32)).astype(np.uint32), (k & np.uint64(0xffffffff)).astype(np.uint32))
    reqs, res = [], []
    for _ in range(3):
        dk = rng.choice(cur, 50, replace=False)
        a = rng.integers(0, n, 60).astype(np.uint64)
        b = rng.integers(0, n, 60).astype(np.uint64)
        ik = (np.minimum(a, b) << np.uint64(32)) | np.maximum(a, b)
        reqs.append(dict(kind="update", ins=split(ik), dels=split(dk)))
        cur = np.union1d(np.setdiff1d(cur, dk), ik[a != b])
        r2, c2 = oracle.csr_dedup(n, *split(cur))
        res.append(dict(digest=bench.core_digest(oracle.bz(r2, c2)[0])))
    reqs.append(dict(kind="decompose", rowptr=rp, col=col))
    res.append(dict(digest=bench.core_digest(oracle.bz(rp, col)[0])))
    assert bench.serve_exact(rp, col, reqs, res) == (True, 4)
    res[1]["digest"] += 1
    assert bench.serve_exact(rp, col, reqs, res) == (False, 4)


def test_param_option_and_e2e_defaults():
    """--param NAME=VALUE (decimal or 0x) reaches the tunables of the main
    graph; the end-to-end section defaults to three steps in flight with the
    peel on one CTA per SM."""
    import argparse

    import pytest
    sys.path.insert(0, ROOT)
    import bench
    assert bench._param("hindex.order=0") == ("hindex.order", 0)
    assert bench._param("peel.chunk=0x800") == ("peel.chunk", 2048)
    for bad in ("hindex.order", "=3", "x=y"):
        with pytest.raises((argparse.ArgumentTypeError, ValueError)):
            bench._param(bad)
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                         timeout=120, cwd=ROOT)
    assert out.returncode == 0 and "--param NAME=VALUE" in out.stdout
    src = open(os.path.join(ROOT, "bench.py")).read()
    assert '"--e2e-depth", type=int, default=3' in src and '"--e2e-ctas-per-sm", type=int, default=1' in src
