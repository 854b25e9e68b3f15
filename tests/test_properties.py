"""Property tests of the oracle on small seeded random graphs: every restated
driver gives the Batagelj-Zaversnik core numbers, the result passes the local
k-core check, and relabelling the vertices permutes the cores.  (Seeded numpy
draws rather than a property-testing library, so the same cases run on every
host, including those without one.)"""
import numpy as np
import pytest

import oracle


def random_graph(rng):
    """A multigraph edge list with self-loops: n in [1, 60], m in [0, 4n]."""
    n = int(rng.integers(1, 61))
    m = int(rng.integers(0, 4 * n + 1))
    s = rng.integers(0, n, m).astype(np.uint32)
    d = rng.integers(0, n, m).astype(np.uint32)
    return n, s, d


@pytest.mark.parametrize("seed", range(150))
def test_restated_drivers_equal_bz(seed):
    n, s, d = random_graph(np.random.default_rng(seed))
    rp, col = oracle.csr_dedup(n, s, d)
    core, kmax = oracle.bz(rp, col)
    assert oracle.check_local(rp, col, core) == 0
    assert int(core.max(initial=0)) == kmax
    assert np.array_equal(oracle.hindex_jacobi(rp, col)[0], core)
    assert np.array_equal(oracle.peel_rounds(rp, col)[0], core)
    assert np.array_equal(oracle.peel_dyn(rp, col)[0], core)
    gp = oracle.gpp(rp, col)[0]
    assert np.array_equal(gp, np.where(np.diff(rp) == 0, 1, core))


@pytest.mark.parametrize("seed", range(100))
def test_relabelling_permutes_cores(seed):
    rng = np.random.default_rng(1000 + seed)
    n, s, d = random_graph(rng)
    perm = rng.permutation(n).astype(np.uint32)
    rp, col = oracle.csr_dedup(n, s, d)
    rp2, col2 = oracle.csr_dedup(n, perm[s], perm[d])
    core = oracle.bz(rp, col)[0]
    core2 = oracle.bz(rp2, col2)[0]
    assert np.array_equal(core2[perm], core)
