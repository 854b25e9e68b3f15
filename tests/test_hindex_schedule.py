"""The re-examination rule of the h-index kernel, simulated on the host in
serial orders: a vertex whose estimate drops from cap to h notifies exactly
the neighbours u with h < c[u] <= cap (the ones it stopped supporting) and
re-examines itself in the next sweep; the support test runs first; sweeps go
on while any vertex is queued.  Whatever the order of the evaluations inside
a sweep, the estimates end at the Batagelj-Zaversnik core numbers.  (The
kernel's concurrent interleavings are covered by the GPU tests; this checks
the rule itself.)"""
import numpy as np
import pytest

import oracle


def h_index(vals):
    v = np.sort(np.asarray(vals))[::-1]
    k = 0
    while k < v.size and v[k] >= k + 1:
        k += 1
    return k


def simulate(rp, col, rng):
    n = rp.size - 1
    c = np.diff(rp).astype(np.int64)
    queued = np.zeros(n, bool)
    cur = list(range(n))
    sweeps = 0
    while cur:
        sweeps += 1
        nxt = []
        rng.shuffle(cur)
        for v in cur:
            queued[v] = False
            cap = c[v]
            if cap == 0:
                continue
            nb = col[rp[v]:rp[v + 1]]
            vals = c[nb]
            if int((vals >= cap).sum()) >= cap:
                continue  # support intact
            h = h_index(np.minimum(vals, cap))
            assert h < cap
            c[v] = h
            for u in list(nb[(vals > h) & (vals <= cap)]) + [v]:  # window, then self
                if not queued[u]:
                    queued[u] = True
                    nxt.append(int(u))
        cur = nxt
        assert sweeps <= 2 * (col.size + 1) + 4
    return c, sweeps


@pytest.mark.parametrize("seed", range(6))
def test_window_rule_reaches_the_cores_in_any_serial_order(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(20, 400))
    m = int(rng.integers(n, 8 * n))
    s = rng.integers(0, n, m).astype(np.uint32)
    d = rng.integers(0, n, m).astype(np.uint32)
    # a dense block, so that deep cores and long cascades occur
    k = int(rng.integers(5, 30))
    a, b = np.triu_indices(k, 1)
    keep = rng.random(a.size) < 0.7
    s = np.concatenate([s, a[keep].astype(np.uint32)])
    d = np.concatenate([d, b[keep].astype(np.uint32)])
    rp, col = oracle.csr_dedup(n, s, d)
    want, _ = oracle.bz(rp, col)
    for trial in range(3):
        got, _ = simulate(rp, col, np.random.default_rng(100 * seed + trial))
        assert np.array_equal(got, want)


def test_window_rule_on_a_path_and_a_star():
    for n, s, d in ((200, np.arange(199), np.arange(1, 200)), (300, np.zeros(299, int), np.arange(1, 300))):
        rp, col = oracle.csr_dedup(n, s.astype(np.uint32), d.astype(np.uint32))
        want, _ = oracle.bz(rp, col)
        got, _ = simulate(rp, col, np.random.default_rng(1))
        assert np.array_equal(got, want)


def simulate_stale(rp, col, rng, self_requeue=True):
    """Like simulate(), but every estimate a vertex reads (for its support
    test, its histogram and its notification window) may be the value at the
    start of the sweep instead of the current one, as a concurrent read that
    raced an update may be.  Values only fall, so a stale read is never below
    the current value.  As in the kernel, a vertex is queued for the next
    sweep in a flag of that sweep's parity, so a notification is never
    dropped because its target is still pending in the current sweep (whose
    evaluation could read the notifier's old value)."""
    n = rp.size - 1
    c = np.diff(rp).astype(np.int64)
    inq = [np.zeros(n, bool), np.zeros(n, bool)]
    cur = list(range(n))
    sweeps = 0
    while cur:
        p = sweeps & 1
        sweeps += 1
        start = c.copy()
        nxt = []
        rng.shuffle(cur)
        for v in cur:
            inq[p][v] = False
            cap = c[v]
            if cap == 0:
                continue
            nb = col[rp[v]:rp[v + 1]]
            stale = rng.random(nb.size) < 0.5
            vals = np.where(stale, start[nb], c[nb])
            if int((vals >= cap).sum()) >= cap:
                continue
            h = h_index(np.minimum(vals, cap))
            c[v] = h
            note = list(nb[(vals > h) & (vals <= cap)])
            if self_requeue:
                note.append(v)
            for u in note:
                if not inq[p ^ 1][u]:
                    inq[p ^ 1][u] = True
                    nxt.append(int(u))
        cur = nxt
        assert sweeps <= 4 * (col.size + 1) + 8
    return c


@pytest.mark.parametrize("seed", range(6))
def test_window_rule_with_stale_reads(seed):
    """With reads that may lag by a sweep, the self-requeue keeps the result
    exact."""
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(20, 300))
    m = int(rng.integers(n, 6 * n))
    s = rng.integers(0, n, m).astype(np.uint32)
    d = rng.integers(0, n, m).astype(np.uint32)
    k = int(rng.integers(5, 25))
    a, b = np.triu_indices(k, 1)
    s = np.concatenate([s, a.astype(np.uint32)])
    d = np.concatenate([d, b.astype(np.uint32)])
    rp, col = oracle.csr_dedup(n, s, d)
    want, _ = oracle.bz(rp, col)
    for trial in range(3):
        got = simulate_stale(rp, col, np.random.default_rng(7 * seed + trial))
        assert np.array_equal(got, want)


def test_self_requeue_is_needed_with_stale_reads():
    """Without the self-requeue some of the same stale-read runs end above the
    core numbers: a neighbour whose window test read this vertex's old value
    skips it, while this vertex counted the neighbour at its old value."""
    wrong = 0
    for seed in range(20):
        rng = np.random.default_rng(5000 + seed)
        n = int(rng.integers(20, 300))
        m = int(rng.integers(n, 6 * n))
        s = rng.integers(0, n, m).astype(np.uint32)
        d = rng.integers(0, n, m).astype(np.uint32)
        k = int(rng.integers(5, 25))
        a, b = np.triu_indices(k, 1)
        s = np.concatenate([s, a.astype(np.uint32)])
        d = np.concatenate([d, b.astype(np.uint32)])
        rp, col = oracle.csr_dedup(n, s, d)
        want, _ = oracle.bz(rp, col)
        got = simulate_stale(rp, col, np.random.default_rng(seed * 10), self_requeue=False)
        assert (got >= want).all()  # estimates stay upper bounds either way
        wrong += not np.array_equal(got, want)
    assert wrong > 0
