"""The allocation-free forward entry point, tomo_forward_noalloc.

Some callers cannot call cudaMalloc -- applications whose own pool allocator
owns all device memory, or latency-bound loops where an allocation would
synchronise the device -- so this entry point runs the forward solve in a
fixed device array compiled into libtomo.so and the caller's own buffers.
These tests call it through the C ABI, twice in a row with different fields,
on the legacy default stream and on a stream of their own, and compare each
result with the context-based tomo_forward, within the wavefield tolerance of
the parity tests (1e-5 relative L2), including a grid of exactly the array's
512 x 512 cell limit.  They also check that the second call leaves device free
memory unchanged and that problems just beyond the array's limits (cells,
record channels, time steps) are refused with TOMO_ERR_ARG before any work.

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


CASES = {
    "cfg": lambda: tomo.cfg_config(nx=96, ny=80, nt=220, n_transducers=24, group_size=6, radius=30.0,
                                   cells_per_wavelength=10.0, sponge_width=10),
    "ref": lambda: tomo.ref_config(nx=64, ny=60, nt=160, ring_lo=8, ring_hi=50, group_size=24),
    # exactly the array's cell limit (512 x 512), short run
    "cfg-512": lambda: tomo.cfg_config(nx=512, ny=512, nt=90, n_transducers=32, group_size=8, radius=220.0),
}


@pytest.mark.parametrize("on_stream", [False, True], ids=["default-stream", "own-stream"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_noalloc_forward_matches_context_forward(built_lib, case, on_stream):
    import torch

    cfg = CASES[case]()
    dev = torch.device("cuda", 0)
    G, nch = tomo.n_groups(cfg), tomo.n_channels(cfg)
    d_rec = torch.empty((G, cfg.nt, nch), dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev) if on_stream else None
    handle = C.c_void_p(stream.cuda_stream) if stream is not None else None
    with tomo.Context(cfg) as ctx:
        for call, seed in enumerate((1, 2)):
            f = phantom(seed, cfg.ny, cfg.nx)
            want = ctx.forward(f)
            d_f = torch.from_numpy(f).to(dev)
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info(dev)[0]
            st = built_lib.tomo_forward_noalloc(C.byref(cfg), C.c_void_p(d_f.data_ptr()),
                                                C.c_void_p(d_rec.data_ptr()), handle)
            assert st == tomo.OK
            if stream is not None:
                stream.synchronize()
            torch.cuda.synchronize()
            if call == 1:
                # set-up was done by the first call; the second must not allocate
                # (device allocations come in >= 2 MiB granules)
                assert free0 - torch.cuda.mem_get_info(dev)[0] < (1 << 20)
            got = d_rec.cpu().numpy()
            assert rel(got, want) <= TOL, (call, rel(got, want))


@pytest.mark.parametrize("make,why", [
    (lambda: tomo.cfg_config(nx=1024, ny=1024, nt=100, n_transducers=16, group_size=4, radius=400.0), "cells"),
    # one row over 512 x 512
    (lambda: tomo.cfg_config(nx=512, ny=513, nt=100, n_transducers=16, group_size=4, radius=200.0), "cells"),
    # 4 * 516 = 2064 reference-profile channels, with fewer cells than the limit (516 x 508)
    (lambda: tomo.ref_config(nx=516, ny=508, nt=100, ring_lo=20, ring_hi=480, group_size=40), "channels"),
    (lambda: tomo.cfg_config(nx=64, ny=64, nt=16385, n_transducers=16, group_size=4, radius=20.0), "steps"),
], ids=["1024x1024", "512x513", "ref-516x508", "nt-16385"])
def test_noalloc_rejects_oversized_problem(built_lib, make, why):
    import torch

    cfg = make()
    d = torch.zeros(16, dtype=torch.float32, device="cuda")
    st = built_lib.tomo_forward_noalloc(C.byref(cfg), C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), None)
    assert st == tomo.ERR_ARG, why
