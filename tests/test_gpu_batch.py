"""GPU checks of tomo_iterate_batch: independent reconstructions of different grid
sizes advanced together give the same bits as the same contexts run one after
another (each context's kernels and reductions are deterministic)."""
import numpy as np
import pytest

import tomo

pytestmark = pytest.mark.gpu


def configs():
    return [tomo.cfg_config(nx=N, ny=N, nt=8 * N, n_transducers=N // 2, group_size=8, radius=0.43 * N,
                            ckpt_interval=int(round((16 * N) ** 0.5)), cells_per_wavelength=10.0,
                            sponge_width=10)
            for N in (64, 96, 128)]


def test_batch_matches_sequential(built_lib):
    import torch

    dev = torch.device("cuda", 0)
    sched = tomo.schedule(omega=0.02, normalize=1)
    results = []
    for batched in (False, True):
        ctxs, d_fs, d_fts = [], [], []
        for i, cfg in enumerate(configs()):
            fo = tomo.phantom_cfg(cfg.nx, cfg.ny, 1, 4, cfg.nx / 40, cfg.nx / 8, 0.1, 0.0, 0.8 * cfg.radius, 40 + i)
            ctx = tomo.Context(cfg)
            ctx.set_records(ctx.generate_data(fo, noise_level=0.01, seed=7 + i))
            ctxs.append(ctx)
            d_fs.append(torch.zeros(fo.shape, dtype=torch.float32, device=dev))
            d_fts.append(torch.from_numpy(fo).to(dev))
        torch.cuda.synchronize(dev)
        if batched:
            eps, secs = tomo.iterate_batch(ctxs, tomo.SIRT_NORM, sched, 0, 3, [t.data_ptr() for t in d_fs],
                                           [t.data_ptr() for t in d_fts])
            assert secs > 0
        else:
            eps = np.array([[ctx.iterate_device(tomo.SIRT_NORM, sched, it, f.data_ptr(), 0, ft.data_ptr()).epsilon
                             for it in range(3)] for ctx, f, ft in zip(ctxs, d_fs, d_fts)])
        for c in ctxs:
            c.synchronize()
        results.append((eps, [f.cpu().numpy() for f in d_fs]))
        for c in ctxs:
            c.close()
    (e0, f0), (e1, f1) = results
    assert np.array_equal(e0, e1)
    for a, b in zip(f0, f1):
        assert np.array_equal(a, b)
    assert np.all(e1[:, -1] < e1[:, 0])


def test_batch_rejects_duplicates(built_lib):
    import torch

    cfg = configs()[0]
    with tomo.Context(cfg) as ctx:
        d = torch.zeros((cfg.ny, cfg.nx), dtype=torch.float32, device="cuda")
        with pytest.raises(tomo.TomoError):
            tomo.iterate_batch([ctx, ctx], tomo.SIRT_NORM, tomo.schedule(omega=0.02, normalize=1), 0, 1,
                               [d.data_ptr(), d.data_ptr()])
