"""Bounded waits of the tile kernels' TMA copies.

Every mbarrier wait of the multi-step tile kernels gives up after a time limit
(TOMO_WAIT_LIMIT_NS), records the failure in a host-visible word and leaves the launch; the
call that synchronises then returns TOMO_ERR_TIMEOUT.  The test makes the region barrier
expect bytes that no copy delivers (TOMO_TEST_UNDELIVERED_TX), so every block's wait runs out
after 2 ms: nothing faults or hangs, the status comes back, and a context created afterwards in
the same process computes the oracle's records.
"""
import numpy as np
import pytest

import oracle_lib as O
import tomo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def cfg():
    return tomo.cfg_config(nx=128, ny=128, nt=120, n_transducers=32, group_size=4, radius=50.0)


def test_timed_out_copy_wait_is_a_status(monkeypatch):
    fo = tomo.phantom_cfg(128, 128, 0, 3, 5.0, 15.0, 0.1, 0.0, 40.0, 1001)
    monkeypatch.setenv("TOMO_TILE", "1")
    monkeypatch.setenv("TOMO_STRIP_ROWS", "8")
    monkeypatch.setenv("TOMO_WAIT_LIMIT_NS", "2000000")
    monkeypatch.setenv("TOMO_TEST_UNDELIVERED_TX", "16")
    with tomo.Context(cfg()) as ctx:
        with pytest.raises(tomo.TomoError) as e:
            ctx.forward(fo)
        assert e.value.status == tomo.ERR_TIMEOUT, e.value
        assert "did not arrive" in str(e.value)
    monkeypatch.delenv("TOMO_TEST_UNDELIVERED_TX")
    monkeypatch.delenv("TOMO_WAIT_LIMIT_NS")
    with tomo.Context(cfg()) as ctx:
        rec = ctx.forward(fo)
    rec_o = O.forward(cfg(), fo.astype(np.float64))
    assert np.linalg.norm(rec - rec_o) <= 1e-5 * np.linalg.norm(rec_o)
