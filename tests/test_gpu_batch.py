"""GPU checks of tomo_iterate_batch: independent reconstructions of different grid
sizes advanced together give the same bits as the same contexts run one after
another (each context's kernels and reductions are deterministic), and every
phantom's images match the FP64 oracle's iterations at the parity bar (1e-4
relative L2), with the image error against the true phantom in the message."""
import numpy as np
import pytest

import oracle_lib as O
import tomo

TOL_IMG = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


pytestmark = pytest.mark.gpu


def configs():
    return [tomo.cfg_config(nx=N, ny=N, nt=8 * N, n_transducers=N // 2, group_size=8, radius=0.43 * N,
                            ckpt_interval=int(round((16 * N) ** 0.5)), cells_per_wavelength=10.0,
                            sponge_width=10)
            for N in (64, 96, 128)]


@pytest.mark.parametrize("form", ["graph", "threads"])
def test_batch_matches_sequential(built_lib, form, monkeypatch):
    """Both forms of the batch (one recorded graph per iteration; a host thread per context)."""
    import torch

    if form == "threads":
        monkeypatch.setenv("TOMO_BATCH_THREADS", "1")
    else:
        monkeypatch.delenv("TOMO_BATCH_THREADS", raising=False)
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


def test_batch_matches_oracle(built_lib):
    """Three phantoms of 64^2, 96^2 and 128^2 with the oracle's records: two normalised SIRT
    iterations through the batch against the oracle's, phantom by phantom."""
    import torch

    dev = torch.device("cuda", 0)
    sched = tomo.schedule(omega=0.02, normalize=1)
    ctxs, d_fs, d_fts, want = [], [], [], []
    for i, cfg in enumerate(configs()):
        fo = tomo.phantom_cfg(cfg.nx, cfg.ny, 1, 4, cfg.nx / 40, cfg.nx / 8, 0.1, 0.0, 0.8 * cfg.radius, 50 + i)
        meas = O.forward(cfg, fo.astype(np.float64))
        f_o = np.zeros(fo.shape, np.float64)
        eps_o = [O.iterate(cfg, tomo.SIRT_NORM, sched, it, f_o, meas, fo.astype(np.float64))[0] for it in range(2)]
        want.append((fo, f_o, eps_o))
        ctx = tomo.Context(cfg)
        ctx.set_records(meas)
        ctxs.append(ctx)
        d_fs.append(torch.zeros(fo.shape, dtype=torch.float32, device=dev))
        d_fts.append(torch.from_numpy(fo).to(dev))
    torch.cuda.synchronize(dev)
    eps, _ = tomo.iterate_batch(ctxs, tomo.SIRT_NORM, sched, 0, 2, [t.data_ptr() for t in d_fs],
                                [t.data_ptr() for t in d_fts])
    for c in ctxs:
        c.synchronize()
    for i, ((fo, f_o, eps_o), d_f) in enumerate(zip(want, d_fs)):
        f = d_f.cpu().numpy()
        msg = (f"phantom {i} ({fo.shape[0]}^2): image vs oracle {rel(f, f_o):.2e}; image error vs phantom "
               f"gpu {eps[i, -1]:.4f} % oracle {eps_o[-1]:.4f} %")
        assert rel(f, f_o) <= TOL_IMG, msg
        for e, eo in zip(eps[i], eps_o):
            assert abs(e - eo) <= 1e-4 * eo, msg
    for c in ctxs:
        c.close()
