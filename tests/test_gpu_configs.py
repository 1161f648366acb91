"""GPU parity at the benchmark workloads' own sizes, against the FP64 oracle.

The small-grid parity tests (test_gpu_parity.py) cover every kernel and rule;
these run the two single-phantom workloads the benchmark times at full size,
through the kernels the benchmark runs:

  128x128 workload: nt 600, 32 transducers on a radius-50 circle in 8 groups
      of 4, phantom of 3 seeded discs (radius 5-15, value U[-0.1, 0.1]),
      5 plain uniform SIRT iterations (classic rule, direction scaled to
      max 1, step 0.1) from f = 0.
  512x512 workload: nt 2500, 256 transducers on a radius-220 circle in 32
      groups of 8, forward history checkpointed every 50 steps, phantom of
      8 seeded ellipses plus smoothed noise; records of all 32 groups, the
      per-group gradients of two groups, and one plain weighted (normalised)
      SIRT iteration.

Bars (relative L2): wavefields and records 1e-5; gradients and images 1e-4.
Each assertion message carries the image error against the true phantom.
The 512x512 cases run once with the kernels the autotuner picks and once per
fixed kernel choice the autotuner can make there (TOMO_* overrides), so the
production kernels are compared with the oracle whatever the tuner picks.
"""
import numpy as np
import pytest

import oracle_lib as O
import tomo

pytestmark = pytest.mark.gpu

TOL_FIELD = 1e-5
TOL_GRAD = 1e-4
TOL_IMG = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def eps_of(f, fo):
    """Image error against the true phantom, percent."""
    return 100.0 * rel(f, fo)


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


# ---- 128x128 workload --------------------------------------------------------------------
def c1_config():
    return tomo.cfg_config(nx=128, ny=128, nt=600, n_transducers=32, group_size=4, radius=50.0)


def c1_phantom():
    return tomo.phantom_cfg(128, 128, 0, 3, 5.0, 15.0, 0.1, 0.0, 40.0, 1001)


def test_c1_records_and_five_uniform_sirt_iterations():
    cfg = c1_config()
    fo = c1_phantom()
    rec_o, ul_o = O.forward(cfg, fo.astype(np.float64), u_last=True)
    sched = tomo.schedule(omega=0.1, normalize=1)
    f = np.zeros_like(fo)
    f_o = np.zeros(fo.shape, np.float64)
    with tomo.Context(cfg) as ctx:
        assert ctx.G == 8
        rec, ul = ctx.forward(fo, u_last=True)
        assert rel(ul, ul_o) <= TOL_FIELD, rel(ul, ul_o)
        assert rel(rec, rec_o) <= TOL_FIELD, rel(rec, rec_o)
        ctx.set_records(rec_o)
        for it in range(5):
            st = ctx.iterate(tomo.SIRT_CLASSIC, sched, it, f, None, fo)
            eps_o = O.iterate(cfg, tomo.SIRT_CLASSIC, sched, it, f_o, rec_o, fo.astype(np.float64))[0]
            msg = (f"iteration {it}: image vs oracle {rel(f, f_o):.2e}; image error vs phantom "
                   f"gpu {eps_of(f, fo):.4f} % oracle {eps_o:.4f} %")
            assert rel(f, f_o) <= TOL_IMG, msg
            assert abs(st.epsilon - eps_o) <= 1e-4 * eps_o, msg
    assert eps_o < 100.0


# ---- 512x512 workload --------------------------------------------------------------------
def c2_config(**kw):
    return tomo.cfg_config(nx=512, ny=512, nt=2500, n_transducers=256, group_size=8, radius=220.0,
                           ckpt_interval=50, **kw)


def c2_phantom():
    return tomo.phantom_cfg(512, 512, 1, 8, 10.0, 60.0, 0.15, 0.01, 176.0, 2001)


# kernel choices: None = the autotuner's pick; otherwise TOMO_* overrides (one-step forward
# rows or staged code; two-step adjoint code)
KERNELS = {
    "autotuned": None,
    "fwd3208-adj3308": dict(TOMO_STRIP_ROWS="8", TOMO_FWD_ROWS="3208", TOMO_FWD_PAIR="0", TOMO_ADJ_PAIR="1",
                            TOMO_ADJ_PAIR_ROWS="3308", TOMO_TILE="0"),
    "fwd6008-adj7016": dict(TOMO_STRIP_ROWS="8", TOMO_FWD_ROWS="6008", TOMO_FWD_PAIR="0", TOMO_ADJ_PAIR="1",
                            TOMO_ADJ_PAIR_ROWS="7016", TOMO_TILE="0"),
    # prefetching lean forward and the packed staged two-step adjoint
    "fwd6108-adj18408": dict(TOMO_STRIP_ROWS="8", TOMO_FWD_ROWS="6108", TOMO_FWD_PAIR="0", TOMO_ADJ_PAIR="1",
                             TOMO_ADJ_PAIR_ROWS="18408", TOMO_TILE="0"),
    "tiles": dict(TOMO_STRIP_ROWS="8", TOMO_FWD_PAIR="0", TOMO_ADJ_PAIR="0", TOMO_TILE="1"),
}

_C2 = {}


def c2_oracle():
    """Oracle records and last wavefields of all 32 groups at the phantom, the gradients of
    groups 0 and 17 at f = fo / 2, and one normalised SIRT iteration from f = 0 (cached)."""
    if not _C2:
        cfg = c2_config()
        fo = c2_phantom()
        rec, ul = O.forward(cfg, fo.astype(np.float64), u_last=True)
        f_half = (0.5 * fo).astype(np.float32)
        d0, _ = O.gradient_groups(cfg, f_half.astype(np.float64), rec, 0, 1)
        d17, _ = O.gradient_groups(cfg, f_half.astype(np.float64), rec, 17, 1)
        f1 = np.zeros(fo.shape, np.float64)
        eps1 = O.iterate(cfg, tomo.SIRT_NORM, tomo.schedule(omega=0.02, normalize=1), 0, f1, rec,
                         fo.astype(np.float64))[0]
        _C2.update(fo=fo, rec=rec, ul=ul, f_half=f_half, dfg={0: d0[0], 17: d17[0]}, f1=f1, eps1=eps1)
    return _C2


@pytest.mark.parametrize("kernels", sorted(KERNELS))
def test_c2_full_size_against_oracle(kernels, monkeypatch):
    for k, v in (KERNELS[kernels] or {}).items():
        monkeypatch.setenv(k, v)
    monkeypatch.delenv("TOMO_TUNE_CACHE", raising=False)
    o = c2_oracle()
    fo = o["fo"]
    cfg = c2_config()
    with tomo.Context(cfg) as ctx:
        assert ctx.G == 32 and ctx.info.ckpt_interval == 50
        rec, ul = ctx.forward(fo, u_last=True)
        assert rel(ul, o["ul"]) <= TOL_FIELD, ("last wavefields", rel(ul, o["ul"]))
        assert rel(rec, o["rec"]) <= TOL_FIELD, ("records", rel(rec, o["rec"]))
        worst = max(rel(rec[g], o["rec"][g]) for g in range(32))
        assert worst <= 2 * TOL_FIELD, ("worst group's records", worst)
        dfg, _, _ = ctx.gradient(o["f_half"], o["rec"])
        for g, want in o["dfg"].items():
            assert rel(dfg[g], want) <= TOL_GRAD, (f"gradient of group {g}", rel(dfg[g], want))
        f = np.zeros_like(fo)
        st = ctx.iterate(tomo.SIRT_NORM, tomo.schedule(omega=0.02, normalize=1), 0, f, None, fo)
        msg = (f"one normalised SIRT iteration: image vs oracle {rel(f, o['f1']):.2e}; image error vs "
               f"phantom gpu {eps_of(f, fo):.4f} % oracle {o['eps1']:.4f} %")
        assert rel(f, o["f1"]) <= TOL_IMG, msg
        assert abs(st.epsilon - o["eps1"]) <= 1e-4 * o["eps1"], msg
