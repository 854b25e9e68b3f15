"""Seeded synthetic workloads built with the device generators.

The reference is benchmarked on SuiteSparse / KONECT files; the workloads here
are synthetic stand-ins with documented shapes:
  * single graphs: R-MAT, Erdos-Renyi G(n, m), R-MAT plus a planted dense
    subgraph (see pico_gb300.rmat_graph / er_graph / rmat_planted_graph);
  * batch_mix: thousands of independent graphs of uneven size packed as one
    segmented CSR -- n = floor(10^U(2, 5)), generator uniform over
    {Erdos-Renyi, R-MAT (a, b, c = .57, .19, .19), Barabasi-Albert}, average
    degree d ~ U[4, 64] setting m = round(n d / 2) for Erdos-Renyi and R-MAT
    (R-MAT over 2^ceil(log2 n) ids, draws outside [0, n) rejected), and
    Barabasi-Albert with its own m_BA ~ U{1..32} edges per vertex (average
    degree about 2 m_BA).  All draws come from numpy's PCG64 seeded with
    `seed`; per-graph generator seeds come from the same stream.
"""
import ctypes

import numpy as np

from . import (DeviceBuffer, Graph, RMAT_ABC, check, lib)

KIND_ER, KIND_RMAT, KIND_BA = 0, 1, 2


def mix_params(num_graphs=4096, seed=4, log_n=(2.0, 5.0), deg=(4.0, 64.0), m_ba=(1, 32)):
    """Per-graph (n, kind, edges to draw, parameter, seed) of a batch mix."""
    rng = np.random.default_rng(seed)
    n = np.floor(10.0 ** rng.uniform(log_n[0], log_n[1], num_graphs)).astype(np.int64)
    kind = rng.integers(0, 3, num_graphs)
    d = rng.uniform(deg[0], deg[1], num_graphs)
    mba = rng.integers(m_ba[0], m_ba[1] + 1, num_graphs)
    seeds = rng.integers(0, 2 ** 62, num_graphs)
    m = np.where(kind == KIND_BA, n * mba, np.round(n * d / 2.0).astype(np.int64))
    m = np.where(kind == KIND_ER, np.minimum(m, n * (n - 1) // 2), m)
    return dict(n=n, kind=kind, d=d, m_ba=mba, m=m, seed=seeds)


def batch_mix(num_graphs=4096, seed=4, device=0, **kw):
    """(packed Graph, vbase uint32[G+1], params): the graphs of a batch mix
    packed into one de-duplicated, symmetrised segmented CSR."""
    p = mix_params(num_graphs, seed, **kw)
    n, kind, m = p["n"], p["kind"], p["m"]
    vbase = np.zeros(num_graphs + 1, dtype=np.int64)
    np.cumsum(n, out=vbase[1:])
    if vbase[-1] >= 2 ** 32:
        raise ValueError("packed vertex count exceeds uint32")
    ebase = np.zeros(num_graphs + 1, dtype=np.int64)
    np.cumsum(m, out=ebase[1:])
    M = int(ebase[-1])
    src = DeviceBuffer(4 * M, device)
    dst = DeviceBuffer(4 * M, device)
    L = lib()
    a, b, c = RMAT_ABC
    for i in range(num_graphs):
        ps = ctypes.c_void_p(src.ptr + 4 * int(ebase[i]))
        pd = ctypes.c_void_p(dst.ptr + 4 * int(ebase[i]))
        ni, mi, si = int(n[i]), int(m[i]), int(p["seed"][i])
        if kind[i] == KIND_ER:
            check(L.kc_gen_er(ni, mi, si, ps, pd, None))
        elif kind[i] == KIND_RMAT:
            check(L.kc_gen_rmat_bounded(ni, mi, a, b, c, si, ps, pd, None))
        else:
            check(L.kc_gen_ba(ni, int(p["m_ba"][i]), si, ps, pd, None))
        check(L.kc_edges_offset(ps, pd, mi, int(vbase[i]), None))
    check(L.kc_device_synchronize(device))
    g = Graph.from_edges_device(src.ptr, dst.ptr, M, int(vbase[-1]), dedup=True, device=device)
    src.free()
    dst.free()
    return g, vbase.astype(np.uint32), p


def graph_csr_host(kind, n, m, seed, m_ba=4, device=0):
    """One Erdos-Renyi / R-MAT / Barabasi-Albert graph built on the device and
    returned as a host CSR (rowptr int64, col uint32)."""
    L = lib()
    mm = int(m)
    src = DeviceBuffer(4 * max(mm, 1), device)
    dst = DeviceBuffer(4 * max(mm, 1), device)
    a, b, c = RMAT_ABC
    ps, pd = ctypes.c_void_p(src.ptr), ctypes.c_void_p(dst.ptr)
    if kind == KIND_ER:
        check(L.kc_gen_er(int(n), mm, int(seed), ps, pd, None))
    elif kind == KIND_RMAT:
        check(L.kc_gen_rmat_bounded(int(n), mm, a, b, c, int(seed), ps, pd, None))
    else:
        check(L.kc_gen_ba(int(n), int(m_ba), int(seed), ps, pd, None))
    check(L.kc_device_synchronize(device))
    g = Graph.from_edges_device(src.ptr, dst.ptr, mm, int(n), dedup=True, device=device)
    src.free()
    dst.free()
    rp, col = g.csr()
    g.free()
    return rp, col


def edge_keys(rowptr, col):
    """Sorted canonical keys (min << 32 | max) of a symmetric CSR's edges."""
    n = rowptr.size - 1
    s = np.repeat(np.arange(n, dtype=np.uint64), np.diff(rowptr))
    d = col.astype(np.uint64)
    keep = s < d
    return np.sort((s[keep] << np.uint64(32)) | d[keep])


def serve_stream(base_rowptr, base_col, num_requests, seed=5, rate_hz=200.0, update_frac=0.5,
                 batch_log=(3.0, 6.0), graph_log_n=(2.0, 5.0), device=0):
    """A Poisson request stream against a resident graph (host CSR given).

    Each request is, with probability update_frac, an edge-update batch of
    size floor(10^U(batch_log)) split evenly between insertions and
    deletions, else the decomposition of a fresh graph drawn like one graph of
    batch_mix.  Deletions are drawn uniformly, without replacement over the
    whole stream, from the base graph's edges; insertions are uniform vertex
    pairs that are neither self-loops nor base edges nor earlier insertions.
    Returns a list of dicts: {t (arrival s), kind, ...}."""
    rng = np.random.default_rng(seed)
    n = base_rowptr.size - 1
    keys = edge_keys(base_rowptr, base_col)
    t = np.cumsum(rng.exponential(1.0 / rate_hz, num_requests))
    is_upd = rng.random(num_requests) < update_frac
    sizes = np.floor(10.0 ** rng.uniform(batch_log[0], batch_log[1], num_requests)).astype(np.int64)
    n_del_total = int(sum(sizes[i] - sizes[i] // 2 for i in range(num_requests) if is_upd[i]))
    del_order = rng.permutation(keys.size)[:min(n_del_total, keys.size)]
    dpos = 0
    inserted = set()
    out = []
    for i in range(num_requests):
        if is_upd[i]:
            ni = int(sizes[i] // 2)
            nd = int(sizes[i] - ni)
            dk = keys[del_order[dpos:dpos + nd]]
            dpos += nd
            ins_s, ins_d = [], []
            while len(ins_s) < ni:
                a = rng.integers(0, n, size=2 * (ni - len(ins_s)) + 16)
                b = rng.integers(0, n, size=a.size)
                lo, hi = np.minimum(a, b).astype(np.uint64), np.maximum(a, b).astype(np.uint64)
                k = (lo << np.uint64(32)) | hi
                pos = np.searchsorted(keys, k)
                exists = (pos < keys.size) & (keys[np.minimum(pos, keys.size - 1)] == k)
                for x, y, kk, ex in zip(a, b, k, exists):
                    if x == y or ex or int(kk) in inserted:
                        continue
                    inserted.add(int(kk))
                    ins_s.append(x)
                    ins_d.append(y)
                    if len(ins_s) == ni:
                        break
            out.append(dict(t=float(t[i]), kind="update",
                            ins=(np.array(ins_s, dtype=np.uint32), np.array(ins_d, dtype=np.uint32)),
                            dels=((dk >> np.uint64(32)).astype(np.uint32),
                                  (dk & np.uint64(0xffffffff)).astype(np.uint32))))
        else:
            gn = int(np.floor(10.0 ** rng.uniform(graph_log_n[0], graph_log_n[1])))
            kind = int(rng.integers(0, 3))
            d = rng.uniform(4.0, 64.0)
            mba = int(rng.integers(1, 33))
            m = gn * mba if kind == KIND_BA else int(round(gn * d / 2.0))
            if kind == KIND_ER:
                m = min(m, gn * (gn - 1) // 2)
            rp, col = graph_csr_host(kind, gn, m, int(rng.integers(0, 2 ** 62)), m_ba=mba, device=device)
            out.append(dict(t=float(t[i]), kind="decompose", rowptr=rp, col=col))
    return out


def run_stream(server, stream, realtime=True, want_core=False):
    """Submit the requests at their arrival times (or all at once) and wait
    for all of them.  Returns the per-request results in stream order."""
    import time
    t0 = time.perf_counter()
    tickets = []
    for r in stream:
        if realtime:
            delay = r["t"] - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
        if r["kind"] == "update":
            tickets.append(server.submit_update(r["ins"], r["dels"], want_core=want_core))
        else:
            tickets.append(server.submit_decompose(r["rowptr"], r["col"]))
    return [server.wait(tk) for tk in tickets]
