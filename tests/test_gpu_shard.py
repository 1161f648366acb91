"""Group-sharded SIRT through the C ABI on one GPU: two contexts stand for two ranks, each runs
the gradient sweeps of its own group range (tomo_gradient_groups_device); their correlations
are moved into one context (tomo_get/set_correlations_device, the data the reduce_df exchange
carries between GPUs) and tomo_update_device applies the update rule.  The field must equal a
single context's tomo_iterate_device bit for bit, for every SIRT rule, over two iterations.
No kernel of one context waits on the other's."""
import numpy as np
import pytest

import shard
import tomo

pytestmark = pytest.mark.gpu


def case():
    cfg = tomo.cfg_config(nx=96, ny=80, nt=200, n_transducers=28, group_size=4, radius=32.0,
                          cells_per_wavelength=10.0, sponge_width=10)
    y, x = np.mgrid[0:80, 0:96]
    fo = (0.08 * (((x - 45) ** 2 + (y - 38) ** 2) <= 64) - 0.05 * (((x - 58) ** 2 + (y - 45) ** 2) <= 25))
    return cfg, fo.astype(np.float32)


SIRT = [
    (tomo.SIRT_CLASSIC, tomo.schedule(omega=0.02, normalize=1)),
    (tomo.SIRT_SCALED, tomo.schedule(tomo.SCHED_POWER, omega=0.02, alpha=0.5, beta=0.5, gamma=1.0, normalize=1)),
    (tomo.SIRT_NORM, tomo.schedule(omega=0.02, normalize=1)),
    (tomo.SIRT_WEIGHT, tomo.schedule(omega=0.02, normalize=1)),
    (tomo.SIRT_AVG_WEIGHT, tomo.schedule(omega=0.01)),
]


@pytest.mark.parametrize("method,sched", SIRT, ids=[tomo.METHOD_NAMES[m] for m, _ in SIRT])
def test_two_context_shards_match_one_context(built_lib, method, sched):
    import torch

    cfg, fo = case()
    dev = torch.device("cuda", 0)
    with tomo.Context(cfg) as one, tomo.Context(cfg) as a, tomo.Context(cfg) as b:
        rec = one.generate_data(fo)
        d_rec = torch.from_numpy(rec).to(dev)
        d_ft = torch.from_numpy(fo).to(dev)
        for c in (one, a, b):
            c.set_records(rec)
        G = one.G
        ranges = [shard.group_range(G, r, 2) for r in range(2)]
        d_one = torch.zeros(fo.shape, dtype=torch.float32, device=dev)
        d_sh = torch.zeros_like(d_one)
        corr = torch.empty((G,) + fo.shape, dtype=torch.float32, device=dev)
        for it in range(2):
            st1 = one.iterate_device(method, sched, it, d_one.data_ptr(), 0, d_ft.data_ptr())
            r2 = 0.0
            for c, (g0, ng) in zip((a, b), ranges):
                r2 += c.gradient_groups_device(d_sh.data_ptr(), g0, ng)
                c.get_correlations_device(g0, ng, corr[g0].data_ptr())
                c.synchronize()
            a.set_correlations_device(0, G, corr.data_ptr())
            st2 = a.update_device(method, sched, it, d_sh.data_ptr(), d_ft.data_ptr())
            a.synchronize()
            one.synchronize()
            assert torch.equal(d_one, d_sh), (it, float((d_one - d_sh).abs().max()))
            assert st2.epsilon == st1.epsilon
            assert abs(r2 - st1.resid_norm2) <= 1e-12 * st1.resid_norm2
        del d_rec


def test_update_device_rejects_art(built_lib):
    import torch

    cfg, fo = case()
    with tomo.Context(cfg) as c:
        d = torch.zeros(fo.shape, dtype=torch.float32, device="cuda")
        with pytest.raises(tomo.TomoError) as e:
            c.update_device(tomo.ART, tomo.schedule(omega=0.01), 0, d.data_ptr())
        assert e.value.status == tomo.ERR_ARG
        with pytest.raises(tomo.TomoError) as e:
            c.gradient_groups_device(d.data_ptr(), 0, 1)      # no records set
        assert e.value.status == tomo.ERR_STATE
