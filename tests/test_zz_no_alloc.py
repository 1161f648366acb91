"""The allocation-free forward entry point, tomo_forward_noalloc.

Some callers cannot call cudaMalloc -- applications whose own pool allocator
owns all device memory, or latency-bound loops where an allocation would
synchronise the device -- so this entry point runs the forward solve in a
fixed device array compiled into libtomo.so and the caller's own buffers.
These tests call it through the C ABI, twice in a row with different fields,
and compare each result with the context-based tomo_forward, within the
wavefield tolerance of the parity tests (1e-5 relative L2).  They also check
that the second call leaves device free memory unchanged and that a problem
beyond the array's limits is refused.

This file sorts last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import tomo

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def phantom(seed, ny, nx):
    rng = np.random.default_rng(seed)
    f = np.zeros((ny, nx), np.float32)
    for _ in range(3):
        cy, cx = rng.uniform(0.35, 0.65) * ny, rng.uniform(0.35, 0.65) * nx
        yy, xx = np.mgrid[0:ny, 0:nx]
        f[(yy - cy) ** 2 + (xx - cx) ** 2 <= rng.uniform(4, 9) ** 2] += rng.uniform(-0.08, 0.08)
    return f


@pytest.mark.parametrize("make", [
    lambda: tomo.cfg_config(nx=96, ny=80, nt=220, n_transducers=24, group_size=6, radius=30.0,
                            cells_per_wavelength=10.0, sponge_width=10),
    lambda: tomo.ref_config(nx=64, ny=60, nt=160, ring_lo=8, ring_hi=50, group_size=24),
], ids=["cfg", "ref"])
def test_noalloc_forward_matches_context_forward(built_lib, make):
    import torch

    cfg = make()
    dev = torch.device("cuda", 0)
    G, nch = tomo.n_groups(cfg), tomo.n_channels(cfg)
    d_rec = torch.empty((G, cfg.nt, nch), dtype=torch.float32, device=dev)
    with tomo.Context(cfg) as ctx:
        for call, seed in enumerate((1, 2)):
            f = phantom(seed, cfg.ny, cfg.nx)
            want = ctx.forward(f)
            d_f = torch.from_numpy(f).to(dev)
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info(dev)[0]
            st = built_lib.tomo_forward_noalloc(C.byref(cfg), C.c_void_p(d_f.data_ptr()),
                                                C.c_void_p(d_rec.data_ptr()), None)
            assert st == tomo.OK
            torch.cuda.synchronize()
            if call == 1:
                # set-up was done by the first call; the second must not allocate
                # (device allocations come in >= 2 MiB granules)
                assert free0 - torch.cuda.mem_get_info(dev)[0] < (1 << 20)
            got = d_rec.cpu().numpy()
            assert rel(got, want) <= TOL, (call, rel(got, want))


def test_noalloc_rejects_oversized_problem(built_lib):
    import torch

    cfg = tomo.cfg_config(nx=1024, ny=1024, nt=100, n_transducers=16, group_size=4, radius=400.0)
    d = torch.zeros(16, dtype=torch.float32, device="cuda")
    st = built_lib.tomo_forward_noalloc(C.byref(cfg), C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), None)
    assert st == tomo.ERR_ARG
