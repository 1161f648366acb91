"""GPU checks of the in-loop record noise (tomo_set_residual_noise): the residual the
engine forms equals measured - simulated * (1 + level (2U - 1)) with U the counter-based
draw restated here in numpy; fixed draws repeat, fresh draws change per sweep and are
reproducible from the seed; noise of level 0 changes nothing."""
import numpy as np
import pytest

import tomo

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


def noise_uniform(key, g, k, c):
    """numpy restatement of the engine's noise_uniform (splitmix64 finaliser of the indices)."""
    g, k, c = (np.asarray(a, np.uint64) for a in np.broadcast_arrays(g, k, c))
    with np.errstate(over="ignore"):
        z = np.uint64(key) ^ (g << np.uint64(42)) ^ (k << np.uint64(20)) ^ c
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)


def cfg_small():
    return tomo.cfg_config(nx=96, ny=96, nt=300, n_transducers=24, group_size=4, radius=36.0,
                           cells_per_wavelength=10.0, sponge_width=10)


def phantom(cfg, seed):
    return tomo.phantom_cfg(cfg.nx, cfg.ny, 0, 3, 4, 9, 0.1, 0.0, 28.0, seed)


@pytest.mark.parametrize("kernels", ["tuned", "tiles"])
def test_fixed_noise_residual_matches_restatement(built_lib, kernels, monkeypatch):
    """The residual under fixed noise against the numpy restatement of the draw, through the
    kernels the tuner picks and through the multi-step tile kernels (whose forward has a
    separate instantiation for noisy launches)."""
    if kernels == "tiles":
        monkeypatch.setenv("TOMO_TILE", "1")
        monkeypatch.setenv("TOMO_STRIP_ROWS", "8")
    cfg = cfg_small()
    fo = phantom(cfg, 3)
    f0 = np.zeros_like(fo)
    level, seed = 0.1, 12345
    with tomo.Context(cfg) as ctx:
        meas = ctx.forward(fo)
        sim = ctx.forward(f0)
        ctx.set_residual_noise(3, level, seed)
        _, _, r2 = ctx.gradient(f0, meas)
    G, nt, nch = sim.shape
    g, k, c = np.meshgrid(np.arange(G), np.arange(nt), np.arange(nch), indexing="ij")
    fac = np.float32(1) + np.float32(level) * (np.float32(2) * noise_uniform(seed, g, k, c) - np.float32(1))
    res = meas.astype(np.float64) - (sim * fac).astype(np.float64)
    res[:, :2] = 0.0                      # slices 0 and 1 are not recorded
    want = float((res ** 2).sum())
    assert abs(r2 - want) <= 1e-5 * want


def test_noise_level_zero_and_off_change_nothing(built_lib):
    cfg = cfg_small()
    fo = phantom(cfg, 4)
    f0 = (0.3 * phantom(cfg, 5)).astype(np.float32)
    with tomo.Context(cfg) as ctx:
        meas = ctx.forward(fo)
        d0, _, r0 = ctx.gradient(f0, meas)
        ctx.set_residual_noise(3, 0.0, 7)
        d1, _, r1 = ctx.gradient(f0, meas)
        ctx.set_residual_noise(0)
        d2, _, r2 = ctx.gradient(f0, meas)
    assert np.array_equal(d0, d1) and r0 == r1
    assert np.array_equal(d0, d2) and r0 == r2


def test_fresh_noise_changes_per_sweep_and_repeats_from_seed(built_lib):
    cfg = cfg_small()
    fo = phantom(cfg, 6)
    f0 = np.zeros_like(fo)
    with tomo.Context(cfg) as ctx:
        meas = ctx.forward(fo)
        ctx.set_residual_noise(2, 0.1, 99)
        a = [ctx.gradient(f0, meas)[2] for _ in range(2)]
        ctx.set_residual_noise(2, 0.1, 99)
        b = [ctx.gradient(f0, meas)[2] for _ in range(2)]
        ctx.set_residual_noise(3, 0.1, 99)
        c = [ctx.gradient(f0, meas)[2] for _ in range(2)]
    assert a[0] != a[1]
    assert a == b
    assert c[0] == c[1]


def test_data_and_residual_share_the_fixed_draw(built_lib):
    """kind 3 in generate_data and in the loop with one seed: at the true field the residual
    vanishes up to rounding (the reference's shared-factor model)."""
    cfg = cfg_small()
    fo = phantom(cfg, 8)
    with tomo.Context(cfg) as ctx:
        meas = ctx.generate_data(fo, noise_level=0.1, seed=5, kind=3)
        ctx.set_residual_noise(3, 0.1, 5)
        _, _, r2 = ctx.gradient(fo, meas)
    assert r2 <= 1e-10 * float((meas.astype(np.float64) ** 2).sum())
