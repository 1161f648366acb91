"""Bounded waits of the tile kernels' TMA copies and grid barriers, and their persistent form.

Every mbarrier wait of the multi-step tile kernels gives up after a time limit
(TOMO_WAIT_LIMIT_NS), records the failure in a host-visible word and leaves the launch; the
call that synchronises then returns TOMO_ERR_TIMEOUT.  The test makes the region barrier
expect bytes that no copy delivers (TOMO_TEST_UNDELIVERED_TX), so every block's wait runs out
after 2 ms: nothing faults or hangs, the status comes back, and a context created afterwards in
the same process computes the oracle's records.  The persistent form (TOMO_PERSIST=1: one
cooperative launch per sweep segment, a grid barrier between its chunks) is checked the same way
for its barrier (TOMO_TEST_GRID_BARRIER_EXTRA: an arrival that never comes) and bit for bit
against one launch per chunk.
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


def test_timed_out_grid_barrier_is_a_status(monkeypatch):
    """A persistent tile launch whose grid barrier waits for an arrival that never comes gives up
    after the wait limit: the call returns TOMO_ERR_TIMEOUT and a new context works."""
    fo = tomo.phantom_cfg(128, 128, 0, 3, 5.0, 15.0, 0.1, 0.0, 40.0, 1001)
    monkeypatch.setenv("TOMO_TILE", "1")
    monkeypatch.setenv("TOMO_STRIP_ROWS", "8")
    monkeypatch.setenv("TOMO_WAIT_LIMIT_NS", "2000000")
    monkeypatch.setenv("TOMO_PERSIST", "1")
    monkeypatch.setenv("TOMO_TEST_GRID_BARRIER_EXTRA", "1")
    with tomo.Context(cfg()) as ctx:
        with pytest.raises(tomo.TomoError) as e:
            ctx.forward(fo)
        assert e.value.status == tomo.ERR_TIMEOUT, e.value
    monkeypatch.delenv("TOMO_TEST_GRID_BARRIER_EXTRA")
    monkeypatch.delenv("TOMO_WAIT_LIMIT_NS")
    with tomo.Context(cfg()) as ctx:
        rec = ctx.forward(fo)
    rec_o = O.forward(cfg(), fo.astype(np.float64))
    assert np.linalg.norm(rec - rec_o) <= 1e-5 * np.linalg.norm(rec_o)


@pytest.mark.parametrize("shape", ["16", "10"])
def test_persistent_sweeps_match_per_chunk_launches(shape, monkeypatch):
    """Tile sweeps as one persistent launch per segment (grid barriers between the 8- and 6-step
    chunks) give the bits of one launch per chunk: records, a normalised SIRT iteration under a
    checkpoint plan (forward, recompute and adjoint segments) and an ART iteration."""
    fo = tomo.phantom_cfg(128, 128, 0, 3, 5.0, 15.0, 0.1, 0.0, 40.0, 1002)
    monkeypatch.setenv("TOMO_TILE", "1")
    monkeypatch.setenv("TOMO_TILE_WARPS", shape)
    monkeypatch.setenv("TOMO_STRIP_ROWS", "8")
    sched = tomo.schedule(omega=0.02, normalize=1)
    outs = []
    for persist in ("1", "0"):
        monkeypatch.setenv("TOMO_PERSIST", persist)
        c = tomo.cfg_config(nx=128, ny=128, nt=120, n_transducers=32, group_size=4, radius=50.0,
                            ckpt_interval=20)
        with tomo.Context(c) as ctx:
            rec = ctx.forward(fo)
            ctx.set_records(rec)
            f = np.zeros_like(fo)
            e1 = ctx.iterate(tomo.SIRT_NORM, sched, 0, f, None, fo).epsilon
            e2 = ctx.iterate(tomo.ART, sched, 1, f, None, fo).epsilon
            outs.append((rec, f, e1, e2))
    (r1, f1, a1, b1), (r0, f0, a0, b0) = outs
    assert np.array_equal(r1, r0)
    assert np.array_equal(f1, f0)
    assert (a1, b1) == (a0, b0)
    assert np.isfinite(f1).all() and b1 < 100.0
