"""Timed memory plan (ckpt_interval = -1).

tomo_create times one gradient pass under each memory plan that fits -- full forward history,
two chunks, the interval of least memory ceil(sqrt(2 (nt - 2))), and an interval whose chunk of
the pass fits in half the L2 -- and keeps the fastest.  The plans hold exact slices, so the
chosen plan must give the fixed plans' gradients and iterations bit for bit (and the oracle's
at the parity bars), stay inside the memory cap, and be recorded in and read back from the
tuning cache.
"""
import math

import numpy as np
import pytest

import oracle_lib as O
import tomo

pytestmark = pytest.mark.gpu

TOL_GRAD = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def c1(**kw):
    """The 128x128 workload: nt 600, 32 transducers in 8 groups of 4 on a radius-50 circle."""
    return tomo.cfg_config(nx=128, ny=128, nt=600, n_transducers=32, group_size=4, radius=50.0, **kw)


def candidates(nt):
    ks = max(4, math.ceil(math.sqrt(2.0 * (nt - 2))))
    return {nt - 2, (nt - 1) // 2, ks}


@pytest.fixture(scope="module")
def problem():
    fo = tomo.phantom_cfg(128, 128, 0, 3, 5.0, 15.0, 0.1, 0.0, 40.0, 1001)
    meas = O.forward(c1(), fo.astype(np.float64))
    f0 = (0.5 * fo).astype(np.float32)
    dfg_o, r2_o = O.gradient(c1(), f0.astype(np.float64), meas)
    return fo, meas, f0, dfg_o, r2_o


def run(cfg, fo, meas, f0):
    with tomo.Context(cfg) as ctx:
        info = (ctx.info.ckpt_interval, ctx.info.groups_per_pass, ctx.info.device_bytes)
        dfg, _, r2 = ctx.gradient(f0, meas)
        f = np.zeros_like(fo)
        ctx.set_records(meas)
        st = ctx.iterate(tomo.SIRT_NORM, tomo.schedule(omega=0.02, normalize=1), 0, f, None, fo)
    return info, dfg, r2, f, st.epsilon


@pytest.mark.parametrize("mem_limit_mb", [0, 160], ids=["all-memory", "160MiB"])
def test_timed_plan_matches_fixed_plans_and_oracle(problem, mem_limit_mb, monkeypatch, tmp_path):
    monkeypatch.setenv("TOMO_TUNE_CACHE", str(tmp_path / "tune.txt"))
    fo, meas, f0, dfg_o, r2_o = problem
    fixed = run(c1(ckpt_interval=10_000), fo, meas, f0)
    timed = run(c1(ckpt_interval=-1, mem_limit_mb=mem_limit_mb), fo, meas, f0)
    (K, P, nbytes) = timed[0]
    assert K in candidates(600) or 4 <= K < 598, K
    assert 1 <= P <= 8
    if mem_limit_mb:
        assert nbytes <= mem_limit_mb << 20, (nbytes, K, P)
    assert np.array_equal(timed[1], fixed[1]), (K, P)
    assert timed[2] == fixed[2]
    assert np.array_equal(timed[3], fixed[3]), (K, P)
    assert rel(timed[1], dfg_o) <= TOL_GRAD, (rel(timed[1], dfg_o), K, P)
    assert abs(timed[2] - r2_o) <= 1e-5 * r2_o
    print(f"timed plan K {K} P {P}: one normalised SIRT iteration, image error vs phantom {timed[4]:.4f} %")
    lines = [ln.split() for ln in open(tmp_path / "tune.txt") if ln.startswith("tomo-plan-1 ")]
    assert lines, "plan choice not recorded"
    full, k, p = map(int, lines[-1][-3:])
    assert (k, p) == (K, P) and full == (K >= 598)


def test_timed_plan_reads_the_cache(problem, tmp_path, monkeypatch):
    """A recorded choice is taken without timing (here the least-memory interval, all groups)."""
    ks = max(4, math.ceil(math.sqrt(2.0 * 598)))
    path = tmp_path / "tune.txt"
    path.write_text(f"tomo-plan-1 {tomo.PROFILE_CFG} 128 128 600 8 4 0 0 {ks} 8\n")
    monkeypatch.setenv("TOMO_TUNE_CACHE", str(path))
    fo, meas, f0, dfg_o, _ = problem
    timed = run(c1(ckpt_interval=-1), fo, meas, f0)
    assert timed[0][:2] == (ks, 8)
    fixed = run(c1(ckpt_interval=ks), fo, meas, f0)
    assert np.array_equal(timed[1], fixed[1])
    assert rel(timed[1], dfg_o) <= TOL_GRAD
