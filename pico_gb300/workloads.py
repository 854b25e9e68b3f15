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
