"""Failure detection without a GPU fault: a bounded inter-CTA wait that runs
out (one CTA withholds its signal, a flag nothing else sets) ends the call
with KC_ERR_TIMEOUT, and the same graph then decomposes exactly."""
import time

import numpy as np
import pytest

import oracle
import pico_gb300 as pg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", ["peelone_dyn", "peel_dyn", "histo", "cnt"])
def test_wait_runs_out_then_context_is_usable(method):
    g = pg.rmat_graph(13, 8, seed=21)
    rp, col = g.csr()
    ref, _ = oracle.bz(rp, col)
    g.set_param("wait.timeout_us", 50000)
    g.set_param("test.withhold", 1)
    t0 = time.time()
    with pytest.raises(pg.KCoreError) as e:
        g.decompose(method)
    dt = time.time() - t0
    assert e.value.code == pg.KC_ERR_TIMEOUT
    assert dt < 20.0
    # no result is published after a failed run
    with pytest.raises(pg.KCoreError) as e2:
        g.device_core()
    assert e2.value.code == pg.KC_ERR_STATE
    g.set_param("test.withhold", 0)
    core, st = g.decompose(method)
    assert np.array_equal(core, ref) and st.kmax == int(ref.max())
    # and other graphs on the same context are unaffected
    h = pg.er_graph(5000, 40000, seed=2)
    core2, _ = h.decompose(method)
    assert np.array_equal(core2, oracle.bz(*h.csr())[0])
    g.free()
    h.free()


def test_wait_limit_is_validated():
    g = pg.er_graph(100, 300, seed=1)
    with pytest.raises(pg.KCoreError):
        g.set_param("wait.timeout_us", 10)
    g.free()
