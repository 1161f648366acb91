"""Known-answer and consistency tests of the CPU oracle (no GPU).

- homogeneous medium: the first arrival at a receiver comes after distance/C
  time steps (cfg profile, c0 = h = 1);
- the sponge absorbs: the wavefield energy after the wave has left decays;
- cfg profile: the adjoint is the exact discrete adjoint, so the gradient
  matches a central finite difference of J = 1/2 ||P u - meas||^2;
- FP32 and FP64 transcriptions agree to single-precision accuracy;
- every update rule keeps the field outside the mask unchanged.
"""
import numpy as np
import pytest

import oracle_lib as O
import tomo


def tiny_cfg(**kw):
    base = dict(nx=40, ny=36, nt=90, n_transducers=12, group_size=3, radius=12.0,
                cells_per_wavelength=8.0, sponge_width=6)
    base.update(kw)
    return tomo.cfg_config(**base)


def test_arrival_time_homogeneous():
    cfg = tomo.cfg_config(nx=96, ny=96, nt=260, n_transducers=8, group_size=1, radius=40.0,
                          cells_per_wavelength=12.0, sponge_width=8)
    rec = O.forward(cfg, np.zeros((96, 96)))
    ii, jj = O.transducers(cfg)
    # group 0 emits from transducer 0; receiver 4 sits opposite (distance ~80 cells)
    dist = np.hypot(ii[4] - ii[0], jj[4] - jj[0])
    trace = rec[0, :, 4]
    t_peak_src = 1.5 * 12.0 / 0.5          # Ricker delay t0 = 1.5/fp in steps (dt = C = 0.5)
    k_peak = int(np.argmax(np.abs(trace)))
    expected = t_peak_src + dist / 0.5
    assert abs(k_peak - expected) < 0.08 * expected


def test_sponge_absorbs_energy():
    """With the sponge the field left after the wave has crossed the grid is a
    fraction of the field with reflecting (zero) walls."""
    def last(smax):
        cfg = tomo.cfg_config(nx=64, ny=64, nt=400, n_transducers=4, group_size=4, radius=20.0,
                              cells_per_wavelength=8.0, sponge_width=16, sponge_max=smax)
        return O.forward(cfg, np.zeros((64, 64)), u_last=True)[1]
    assert np.linalg.norm(last(0.05)) < 0.35 * np.linalg.norm(last(0.0))


def J(cfg, f, meas):
    rec = O.forward(cfg, f).astype(np.float64)
    return 0.5 * float(((rec - meas) ** 2).sum())


def test_cfg_gradient_matches_finite_difference():
    cfg = tiny_cfg()
    rng = np.random.default_rng(0)
    fo = np.zeros((cfg.ny, cfg.nx))
    fo[14:22, 16:24] = 0.1
    meas = O.forward(cfg, fo).astype(np.float64)
    f = 0.01 * rng.standard_normal((cfg.ny, cfg.nx))
    dfg, _ = O.gradient(cfg, f, meas.astype(np.float32))
    # dfg = -dJ/df * 1/(1+f)  ->  -dJ/df = dfg * (1+f)
    g = dfg.sum(0) * (1.0 + f)
    h = 1e-3
    for (j, i) in [(18, 20), (15, 18), (20, 22), (12, 26)]:
        e = np.zeros_like(f)
        e[j, i] = h
        fd = -(J(cfg, f + e, meas) - J(cfg, f - e, meas)) / (2 * h)
        assert abs(fd - g[j, i]) <= 2e-3 * max(abs(fd), 1e-3 * np.abs(g).max()), (j, i, fd, g[j, i])


@pytest.mark.parametrize("maker", ["ref", "cfg"])
def test_fp32_tracks_fp64(maker):
    if maker == "ref":
        cfg = tomo.ref_config(nx=48, ny=48, nt=120, ring_lo=6, ring_hi=40, group_size=34)
    else:
        cfg = tiny_cfg()
    fo = np.zeros((cfg.ny, cfg.nx))
    fo[18:28, 16:26] = 0.05
    r64 = O.forward(cfg, fo, prec=64)
    r32 = O.forward(cfg, fo, prec=32)
    assert np.linalg.norm(r32 - r64) / np.linalg.norm(r64) < 5e-6
    d64, _ = O.gradient(cfg, np.zeros_like(fo), r64, prec=64)
    d32, _ = O.gradient(cfg, np.zeros_like(fo), r64, prec=32)
    assert np.linalg.norm(d32 - d64) / np.linalg.norm(d64) < 1e-4


@pytest.mark.parametrize("method", range(7))
def test_updates_respect_mask(method):
    cfg = tomo.ref_config(nx=48, ny=48, nt=100, ring_lo=6, ring_hi=40, group_size=34)
    fo = np.zeros((48, 48))
    fo[20:28, 18:26] = 0.05
    meas = O.forward(cfg, fo)
    f = np.full((48, 48), 0.001)
    O.iterate(cfg, method, tomo.schedule(omega=2e3), 0, f, meas, fo)
    m = O.mask(cfg).astype(bool)
    if method != tomo.SIRT_AVG_WEIGHT:      # that rule adds an unmasked sum (reference quirk)
        assert np.all(f[~m] == 0.001)
        assert np.any(f[m] != 0.001)
