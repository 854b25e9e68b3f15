"""Property tests of the oracle on small random graphs (hypothesis): every
restated driver gives the Batagelj-Zaversnik core numbers, the result passes
the local k-core check, and relabelling the vertices permutes the cores."""
import numpy as np
import pytest

import oracle

hyp = pytest.importorskip("hypothesis")
st = pytest.importorskip("hypothesis.strategies")


@st.composite
def graphs(draw):
    n = draw(st.integers(1, 60))
    m = draw(st.integers(0, 4 * n))
    s = np.array(draw(st.lists(st.integers(0, n - 1), min_size=m, max_size=m)), dtype=np.uint32)
    d = np.array(draw(st.lists(st.integers(0, n - 1), min_size=m, max_size=m)), dtype=np.uint32)
    return n, s, d


@hyp.settings(max_examples=150, deadline=None)
@hyp.given(graphs())
def test_restated_drivers_equal_bz(g):
    n, s, d = g
    rp, col = oracle.csr_dedup(n, s, d)
    core, kmax = oracle.bz(rp, col)
    assert oracle.check_local(rp, col, core) == 0
    assert int(core.max(initial=0)) == kmax
    assert np.array_equal(oracle.hindex_jacobi(rp, col)[0], core)
    assert np.array_equal(oracle.peel_rounds(rp, col)[0], core)
    assert np.array_equal(oracle.peel_dyn(rp, col)[0], core)
    gp = oracle.gpp(rp, col)[0]
    assert np.array_equal(gp, np.where(np.diff(rp) == 0, 1, core))


@hyp.settings(max_examples=100, deadline=None)
@hyp.given(graphs(), st.integers(0, 2**32 - 1))
def test_relabelling_permutes_cores(g, seed):
    n, s, d = g
    perm = np.random.default_rng(seed).permutation(n).astype(np.uint32)
    rp, col = oracle.csr_dedup(n, s, d)
    rp2, col2 = oracle.csr_dedup(n, perm[s], perm[d])
    core = oracle.bz(rp, col)[0]
    core2 = oracle.bz(rp2, col2)[0]
    assert np.array_equal(core2[perm], core)
