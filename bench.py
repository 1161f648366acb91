#!/usr/bin/env python3
"""Benchmark of the reconstruction hot path: one plain weighted SIRT iteration.

Workload (default): 512x512 grid, nt 2500, Courant 0.5, 16-cell quadratic
sponge, 256 transducers on a radius-220 circle in 32 groups of 8, Ricker
source at 12 cells per wavelength, forward history checkpointed every 50
steps; phantom of 8 seeded ellipses plus smoothed noise, records with 1%
Gaussian noise (synthetic, seeded).  A step is one normalised-weight SIRT
iteration: forward sweep of all 32 groups, residual, adjoint sweep with the
fused correlation, checkpoint recompute, and the update.

metric: stencil GB/s, algorithmic bytes per iteration = G*nx*ny*(nt-2)*(16+20)
(16 B per forward and 20 B per adjoint cell-update; recompute not credited).
On c2 the line also carries time_to_image: wall time of 30 plain weighted SIRT
iterations from f = 0 against the learned update (the shipped network in
weights/learned_update.bin, residual-checked) run until it reaches the same
image error, with the speed-up, the gradient sweeps each used and the learned
run's steps (L learned, x rejected proposal + plain step, p plain step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl tomo|reference]
                    [--workload c2|c1|c3|ref192|c5|net] [--no-cpu] [--no-learned] [--nt T]
--workload net times the learned update network alone (tensor-core kernels): one
inference on a 512x512 field and one training step on a batch of 16 fields of
256x256 (shipped weights, synthetic inputs), wall clock per call.
Under torchrun each rank reconstructs its own independent phantom on its own
GPU (weak scaling over independent reconstructions, no collective on the
data path); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "tomographic-image-reconstruction-algorithms_gb300")
sys.path.insert(0, os.path.join(PKG, "python"))
sys.path.insert(0, PKG)

import numpy as np  # noqa: E402

import tomo  # noqa: E402

WORKLOADS = {
    "c2": dict(desc="512x512, nt 2500, 256 transducers r=220, 32 groups of 8, sponge 16/0.05, "
                    "Ricker 12 cells/wavelength, checkpoint every 50 steps, plain weighted SIRT",
               cfg=dict(nx=512, ny=512, nt=2500, n_transducers=256, group_size=8, radius=220.0,
                        ckpt_interval=50),
               phantom=(1, 8, 10.0, 60.0, 0.15, 0.01, 176.0), noise=0.01,
               method=tomo.SIRT_NORM, sched=dict(omega=0.02, normalize=1)),
    "c1": dict(desc="128x128, nt 600, 32 transducers r=50, 8 groups of 4, plain uniform SIRT step 0.1",
               cfg=dict(nx=128, ny=128, nt=600, n_transducers=32, group_size=4, radius=50.0),
               phantom=(0, 3, 5.0, 15.0, 0.1, 0.0, 40.0), noise=0.0,
               method=tomo.SIRT_CLASSIC, sched=dict(omega=0.1, normalize=1)),
    "c5": dict(desc="2048x2048, nt 8000, 512 transducers r=950, 64 groups of 8, checkpoint every 200 steps",
               cfg=dict(nx=2048, ny=2048, nt=8000, n_transducers=512, group_size=8, radius=950.0,
                        ckpt_interval=200),
               phantom=(1, 16, 20.0, 240.0, 0.15, 0.01, 760.0), noise=0.01,
               method=tomo.SIRT_NORM, sched=dict(omega=0.02, normalize=1)),
    "ref192": dict(desc="reference problem: 192x192, nt 401, 640 transducers on the square ring, "
                        "group size 10 (64 groups), normalised SIRT",
                   cfg=None, phantom=None, noise=0.0, method=tomo.SIRT_NORM,
                   sched=dict(kind=tomo.SCHED_POWER, omega=1e5, alpha=0.5, beta=0.5, gamma=1.0)),
}


C3_SIZES = (128, 192, 256, 384, 512)


def c3_configs(device, n=64, timed_plans=False, memory=None):
    """The batched workload: n phantoms cycling through the grid sizes N, N/2 transducers on a
    radius-0.43N circle in groups of 8, nt = 10 N.  Checkpoint interval: about sqrt(2 nt), or
    with timed_plans the library's timed choice (ckpt_interval -1) under a per-phantom memory cap
    (c3_memory_caps over `memory` bytes)."""
    out = []
    for i in range(n):
        N = C3_SIZES[i % len(C3_SIZES)]
        nt = 10 * N
        out.append(tomo.cfg_config(nx=N, ny=N, nt=nt, n_transducers=N // 2, group_size=8, radius=0.43 * N,
                                   ckpt_interval=-1 if timed_plans else int(round((2 * nt) ** 0.5)), device=device))
    if timed_plans:
        for cfg, cap in zip(out, c3_memory_caps(out, memory)):
            cfg.mem_limit_mb = int(cap // (1 << 20))
    return out


def plan_bytes(cfg, full, K=0):
    """Device bytes of a context under a memory plan with all groups resident: the plan's
    per-group buffers (forward slots, adjoint ring of 4, checkpoints, residual records) and the
    fixed ones, as the library's plan counts them (plus 64 MiB of slack)."""
    G, N, nt, nch = tomo.n_groups(cfg), cfg.nx * cfg.ny, cfg.nt, tomo.n_channels(cfg)
    slots = nt if full else K + 1
    chunks = 0 if full else -(-(nt - 2) // K)
    per_group = 4 * ((slots + 4 + 2 * chunks) * N + nt * nch)
    fixed = 4 * 7 * N + 4 * 2 * G * N + 4 * 2 * G * nt * nch + 8 * G * nt + 8 * (G + 2) * 1024 + (64 << 20)
    return G * per_group + fixed


def c3_memory_caps(cfgs, memory):
    """Memory caps of the batch: every phantom gets its least-memory plan (K = ceil(sqrt(2 (nt-2))));
    what is left goes, smallest first, to phantoms whose full forward history then fits; the rest
    is shared in proportion to the caps.  The library times its plans inside each cap."""
    ks = [max(4, math.ceil(math.sqrt(2.0 * (c.nt - 2)))) for c in cfgs]
    caps = [plan_bytes(c, False, k) for c, k in zip(cfgs, ks)]
    left = memory - sum(caps)
    if left < 0:
        raise RuntimeError(f"the batch needs {sum(caps) / 1e9:.1f} GB at least, {memory / 1e9:.1f} GB available")
    for i in sorted(range(len(cfgs)), key=lambda i: plan_bytes(cfgs[i], True)):
        extra = plan_bytes(cfgs[i], True) - caps[i]
        if 0 < extra <= left:
            caps[i] += extra
            left -= extra
    tot = sum(caps)
    return [c + left * c / tot for c in caps]


def run_batch(args, local, rank, world, dist):
    """c3: 64 independent reconstructions of uneven sizes advanced together (tomo_iterate_batch)."""
    import torch

    dev = torch.device("cuda", local)
    # plan and kernel choices are timed once per grid size and reused through the tuning cache
    if not os.environ.get("TOMO_TUNE_CACHE"):
        os.environ["TOMO_TUNE_CACHE"] = os.path.join(tempfile.mkdtemp(prefix="tomo_tune_"), "tune.txt")
    free_b, _ = torch.cuda.mem_get_info(dev)
    cfgs = c3_configs(local, timed_plans=True, memory=0.85 * free_b)
    ctxs, d_fs, d_fts, recs, fos = [], [], [], [], []
    for i, cfg in enumerate(cfgs):
        N = cfg.nx
        fo = tomo.phantom_cfg(N, N, 1, 8, N / 50.0, N / 8.5, 0.15, 0.01, 0.8 * cfg.radius, 5000 + i + 1000 * rank)
        ctx = tomo.Context(cfg)
        rec = ctx.generate_data(fo, noise_level=0.01, seed=5000 + i)
        ctx.set_records(rec)
        ctxs.append(ctx)
        fos.append(fo)
        recs.append(torch.from_numpy(rec).pin_memory())
        d_fs.append(torch.zeros(fo.shape, dtype=torch.float32, device=dev))
        d_fts.append(torch.from_numpy(fo).to(dev))
    torch.cuda.synchronize(dev)
    sched = tomo.schedule(omega=0.02, normalize=1)
    bytes_it = sum(algorithmic_bytes(c, tomo.n_groups(c)) for c in cfgs)
    # the timed memory plan each grid size got: K (nt - 2 = full history) and groups per pass
    plans = {}
    for cfg, ctx in zip(cfgs, ctxs):
        K, P = ctx.info.ckpt_interval, ctx.info.groups_per_pass
        plans.setdefault(str(cfg.nx), set()).add(("full" if K >= cfg.nt - 2 else f"K {K}") + f", P {P}"
                                                 + f" of {tomo.n_groups(cfg)}")
    plans = {k: sorted(v) for k, v in plans.items()}
    ptrs = [t.data_ptr() for t in d_fs]
    tptrs = [t.data_ptr() for t in d_fts]
    tomo.iterate_batch(ctxs, tomo.SIRT_NORM, sched, 0, args.warmup, ptrs, tptrs)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        eps, secs = tomo.iterate_batch(ctxs, tomo.SIRT_NORM, sched, args.warmup, args.steps, ptrs, tptrs)
    clocks = clk.summary()
    t_max = max_over_ranks(secs, dist, dev)
    value = world * bytes_it * args.steps / t_max / 1e9
    # end to end: every step copies each phantom's records and field in from pinned host memory and
    # the field back out
    f_host = [torch.zeros(fo.shape, dtype=torch.float32).pin_memory() for fo in fos]
    t0 = time.perf_counter()
    for s_ in range(args.steps):
        for i, ctx in enumerate(ctxs):
            ctx.set_records(recs[i].numpy())
            d_fs[i].copy_(f_host[i], non_blocking=True)
        torch.cuda.synchronize(dev)
        tomo.iterate_batch(ctxs, tomo.SIRT_NORM, sched, args.warmup + args.steps + s_, 1, ptrs, tptrs)
        for i in range(len(ctxs)):
            f_host[i].copy_(d_fs[i], non_blocking=True)
        torch.cuda.synchronize(dev)
    e2e_s = time.perf_counter() - t0
    h2d = sum(4 * (fo.size + r.numel()) for fo, r in zip(fos, recs))
    if rank == 0:
        line = {
            "metric": metric_name(args.workload), "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded ellipse phantoms + smoothed noise, 1% Gaussian record noise)",
            "config": {"workload": "c3: 64 phantoms of N in {128,192,256,384,512} cycling, N/2 transducers "
                                   "r=0.43N, groups of 8, nt 10N, memory plan timed per phantom (checkpoint interval "
                                   "and groups per pass, see plans), plain weighted SIRT, "
                                   "all phantoms advanced together (tomo_iterate_batch)",
                       "phantoms": len(cfgs), "l2": "inputs larger than L2",
                       "parallelism": f"replicas{world}" if world > 1 else "single GPU"},
            "plans": plans,
            "phantom_iter_per_s": world * len(cfgs) * args.steps / t_max,
            "epsilon_last_mean": float(np.nanmean(eps[:, -1])),
            "e2e": {"value": world * bytes_it * args.steps / e2e_s / 1e9, "unit": "GB/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": sum(4 * fo.size for fo in fos)},
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    for c in ctxs:
        c.close()


def make_config(w, device):
    if w["cfg"] is None:
        return tomo.ref_config(device=device)
    return tomo.cfg_config(device=device, **w["cfg"])


def make_phantom(w, cfg, seed):
    if w["phantom"] is None:
        return tomo.phantom_ref()
    kind, n, rmin, rmax, vmax, sig, sup = w["phantom"]
    return tomo.phantom_cfg(cfg.nx, cfg.ny, kind, n, rmin, rmax, vmax, sig, sup, seed)


def algorithmic_bytes(cfg, G):
    return float(G) * cfg.nx * cfg.ny * (cfg.nt - 2) * 36.0


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        self.tmp.flush()
        try:
            rows = [r.split(",") for r in open(self.tmp.name).read().strip().splitlines() if r.strip()]
        except Exception:
            rows = []
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and "Active" in r[5 + i]
                          and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_sample(w, cfg, fo, rec, target_s=12.0):
    """Oracle FP32 OpenMP forward+adjoint sweeps of whole groups (all host threads)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_lib as O

    O.build()
    cores = os.cpu_count() or 1
    f64 = np.zeros(fo.shape, np.float64)
    t0 = time.perf_counter()
    cu = 0.0
    ng = 0
    while True:
        cu += O.sweep(cfg, f64, rec, ng % tomo.n_groups(cfg), 1, prec=32, threads=cores)
        ng += 1
        if time.perf_counter() - t0 > target_s or ng >= tomo.n_groups(cfg):
            break
    dt = time.perf_counter() - t0
    gbs = cu / 2 * 36.0 / dt / 1e9
    return {"value": gbs, "unit": "GB/s", "cores": cores, "kind": "port",
            "sample": f"{ng} group forward+adjoint sweep(s) of the full {cfg.nx}x{cfg.ny}x{cfg.nt} problem, "
                      f"oracle FP32 transcription, OpenMP over {cores} threads, {dt:.1f} s",
            "seconds": dt, "cell_updates": cu}


def reference_arm(args, w, rank, world):
    if rank != 0:
        return
    if w is None:   # c3: the sweep of its largest phantom stands for the batch
        cfg = c3_configs(0)[C3_SIZES.index(512)]
        w = {"desc": "largest c3 phantom (512x512, nt 5120, 256 transducers, 32 groups of 8)"}
    else:
        cfg = make_config(w, 0)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_lib as O

    O.build()
    G = tomo.n_groups(cfg)
    nch = tomo.n_channels(cfg)
    # the sweep's work does not depend on the values: homogeneous field, zero data
    rec = np.zeros((G, cfg.nt, nch), np.float32)
    cores = os.cpu_count() or 1
    f64 = np.zeros((cfg.ny, cfg.nx), np.float64)
    for _ in range(args.warmup):
        O.sweep(cfg, f64, rec, 0, 1, prec=32, threads=cores)
    ts = []
    cu = 0.0
    for s in range(args.steps):
        t0 = time.perf_counter()
        cu = O.sweep(cfg, f64, rec, s % G, 1, prec=32, threads=cores)
        ts.append(time.perf_counter() - t0)
    dt = sum(ts)
    gbs = cu * args.steps / 2 * 36.0 / dt / 1e9
    line = {
        "impl": "reference", "metric": metric_name(args.workload), "value": gbs, "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded phantom)", "config": {"workload": args.workload + ": " + w["desc"]},
        "cpu_baseline": {"value": gbs, "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": "each step: one group's forward+adjoint sweep of the full problem, oracle FP32 "
                                   "transcription of the reference kernels (the reference ships no CPU path)"},
        "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def metric_name(workload="c2"):
    """The metric of a workload's line (both arms print the same string for the same workload)."""
    what = {"c1": "one plain uniform SIRT iteration", "c3": "one batched plain weighted SIRT iteration",
            "ref192": "one normalised SIRT iteration"}.get(workload, "one plain weighted SIRT iteration")
    return "stencil GB/s (algorithmic 36 B per forward+adjoint cell-update) of " + what


WEIGHTS = os.path.join(PKG, "weights", "learned_update.bin")


def time_to_image(ctx, w, sched, d_f, d_ft, torch, dev, plain_iters=30):
    """Wall time of plain weighted SIRT for plain_iters iterations from f = 0 against the learned
    update (shipped network, residual-checked, fused run loop) to the same image error."""
    if not os.path.exists(WEIGHTS):
        return {"unavailable": "no trained weights at " + os.path.relpath(WEIGHTS, REPO)}
    net = tomo.Net(dev.index or 0)
    net.load(WEIGHTS)
    ctx.set_learned_scale(tomo.LEARNED_SCALE)
    d_f.zero_()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    eps = [ctx.iterate_device(w["method"], sched, it, d_f.data_ptr(), 0, d_ft.data_ptr()).epsilon
           for it in range(plain_iters)]
    ctx.synchronize()
    t_plain = time.perf_counter() - t0
    d_f.zero_()
    torch.cuda.synchronize(dev)
    ctx.run_learned(net, sched, d_f.data_ptr(), d_ft.data_ptr(), -1.0, 1)    # warm-up: illumination, graphs
    d_f.zero_()
    torch.cuda.synchronize(dev)
    leps, kind, sweeps, t_learned = ctx.run_learned(net, sched, d_f.data_ptr(), d_ft.data_ptr(), eps[-1],
                                                    3 * plain_iters)
    net.close()
    reached = bool(leps[-1] <= eps[-1])
    return {"plain_seconds": t_plain, "plain_iters": plain_iters, "target_epsilon": eps[-1],
            "learned_seconds": t_learned, "learned_iters": len(leps),
            "learned_steps": "".join({1: "L", 2: "l", 0: "x", -1: "p"}[int(k)] for k in kind),
            "learned_epsilon": float(leps[-1]), "reached": reached,
            "acceptance": {"min_decrease": tomo.LEARNED_MIN_DECREASE, "patience": tomo.LEARNED_PATIENCE,
                           "scale": tomo.LEARNED_SCALE},
            "gradient_sweeps": {"plain": plain_iters, "learned": sweeps},
            "speedup": t_plain / t_learned if reached else None}


def art_iteration(ctx, sched, d_f, d_ft, sirt_ms, iters=2):
    """One ART iteration (art-mimo.cu:688-736: each group's gradient sweep and update in turn) on
    the same workload, after one untimed iteration that captures the per-group graphs; reported
    beside the SIRT iteration it is compared with."""
    ctx.iterate_device(tomo.ART, sched, 0, d_f.data_ptr(), 0, d_ft.data_ptr())
    ctx.synchronize()
    ms = []
    for it in range(1, 1 + iters):
        st = ctx.iterate_device(tomo.ART, sched, it, d_f.data_ptr(), 0, d_ft.data_ptr())
        ms.append(st.seconds * 1e3)
    ms = min(ms)
    return {"iteration_ms": ms, "sirt_iteration_ms": sirt_ms, "ratio_to_sirt": ms / sirt_ms,
            "kernel_launches": st.kernel_launches}


NET_FLOP_PER_PIXEL = 2 * 9 * (16 * 32 + 3 * 32 * 32 + 32 * 16)   # forward GEMMs as issued (padded channels)


def run_net(args):
    """The learned update network alone: inference on 1 x 512 x 512 and a training step on
    16 x 256 x 256 (forward, loss, data and weight gradients, Adam), wall clock per call with the
    call's own synchronisation; FLOP counts are the tensor-core GEMMs as issued (the backward
    pass issues twice the forward's)."""
    import torch

    dev = torch.device("cuda", 0)
    net = tomo.Net(0, seed=1)
    if os.path.exists(WEIGHTS):
        net.load(WEIGHTS)
    out = {}
    for name, (B, H, W) in (("inference_1x512x512", (1, 512, 512)), ("train_16x256x256", (16, 256, 256))):
        g = torch.Generator(device=dev).manual_seed(7)
        feat = torch.randn((B, 3, H, W), device=dev, generator=g)
        res = torch.empty((B, H, W), device=dev)
        tgt = 0.01 * torch.randn((B, H, W), device=dev, generator=g)
        msk = torch.ones((B, H, W), device=dev)
        train = name.startswith("train")

        def call():
            if train:
                net.train_step_device(feat.data_ptr(), tgt.data_ptr(), msk.data_ptr(), B, H, W, 1e-6)
            else:
                net.forward_device(feat.data_ptr(), B, H, W, res.data_ptr())

        for _ in range(args.warmup):
            call()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            call()
        ms = (time.perf_counter() - t0) / args.steps * 1e3
        flop = (3 if train else 1) * NET_FLOP_PER_PIXEL * B * H * W
        out[name] = {"ms": ms, "tflops": flop / (ms * 1e-3) / 1e12}
    net.close()
    line = {"metric": "learned update network: wall time per call", "value": out["inference_1x512x512"]["ms"],
            "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": False,
            "dtype": "bf16 (fp32 accumulate)", "data": "synthetic features, shipped weights",
            "config": {"workload": "net: 5-layer 3x3 CNN, 32 channels, tcgen05 implicit-GEMM kernels"},
            "calls": out}
    print(json.dumps(line))


def max_over_ranks(x, dist, dev=None):
    """The largest x over all ranks (x itself without a process group)."""
    if not dist:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=dev if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def read_tuning(path):
    """The strip-kernel choice of the autotuner, from its cache file (last line)."""
    try:
        lines = [l.split() for l in open(path) if l.startswith("tomo-tune-1")]
    except OSError:
        return None
    if not lines:
        return None
    v = [int(x) for x in lines[-1][7:]] + [0] * 4
    out = {"fwd": f"two steps/launch, code {v[6]}" if v[5] else f"one step/launch, code {v[0]}",
           "adj": f"two steps/launch, code {v[4]}" if v[3] else f"one step/launch, {v[1]} rows, variant {v[2]}"}
    if v[7]:
        out["fwd"] = "tiles, 8 steps/launch"
    if v[8]:
        out["adj"] = "tiles, 6 steps/launch"
    out["one_group_passes"] = {"fwd": "tiles" if v[9] else "as above", "adj": "tiles" if v[10] else "as above"}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="tomo", choices=["tomo", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS) + ["c3", "net"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-learned", action="store_true", help="skip the time-to-image leg (c2)")
    ap.add_argument("--no-art", action="store_true", help="skip the ART iteration leg (c2, c1)")
    ap.add_argument("--nt", type=int, default=0,
                    help="time steps instead of the workload's (small cases for profiling; the workload "
                         "name in the line says so)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    w = WORKLOADS.get(args.workload)
    if w is not None and args.nt > 0 and w["cfg"] is not None:
        w = dict(w, cfg=dict(w["cfg"], nt=args.nt), desc=w["desc"] + f" [nt {args.nt} instead]")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        import torch

        dist = dist_mod
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)

    if args.impl == "reference":
        reference_arm(args, w, rank, world)
        if dist:
            dist.destroy_process_group()
        return

    import torch

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU (libtomo.so has no CPU path)")
    tomo.lib()
    if args.workload == "net":
        return run_net(args)
    if args.workload == "c3":
        run_batch(args, local, rank, world, dist)
        if dist:
            dist.destroy_process_group()
        return
    cfg = make_config(w, local)
    fo = make_phantom(w, cfg, 2001 + 1000 * rank)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        # the oracle runs before the first GPU call of this process
        G0 = tomo.n_groups(cfg)
        cpu = cpu_sample(w, cfg, fo, np.zeros((G0, cfg.nt, tomo.n_channels(cfg)), np.float32))

    # the kernel choice is recorded in a tuning cache (reused when TOMO_TUNE_CACHE names one)
    own_cache = not os.environ.get("TOMO_TUNE_CACHE")
    if own_cache:
        os.environ["TOMO_TUNE_CACHE"] = os.path.join(tempfile.mkdtemp(prefix="tomo_tune_"), "tune.txt")
    ctx = tomo.Context(cfg)
    G = ctx.G
    rec = ctx.generate_data(fo, noise_level=w["noise"], seed=77 + rank)
    tuning = read_tuning(os.environ["TOMO_TUNE_CACHE"])
    sched = tomo.schedule(**w["sched"])
    dev = torch.device("cuda", local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    d_f = torch.zeros(fo.shape, dtype=torch.float32, device=dev)
    d_ft = torch.from_numpy(fo).to(dev)
    d_rec = torch.from_numpy(rec).to(dev)
    torch.cuda.synchronize(dev)
    # records go to the context once; each step then reads them from HBM
    ctx.iterate_device(w["method"], sched, 0, d_f.data_ptr(), d_rec.data_ptr(), d_ft.data_ptr())
    ctx.synchronize()
    for it in range(1, args.warmup):
        ctx.iterate_device(w["method"], sched, it, d_f.data_ptr(), 0, d_ft.data_ptr())
    ctx.synchronize()

    def barrier():
        if dist:
            dist.barrier()

    launches = 0.0
    eps = []
    barrier()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.nvtx.range_push("timed_steps")     # lets ncu --nvtx-include select the timed region
        e0.record(stream)
        for s in range(args.steps):
            st = ctx.iterate_device(w["method"], sched, args.warmup + s, d_f.data_ptr(), 0, d_ft.data_ptr())
            launches += st.kernel_launches
            eps.append(st.epsilon)
        e1.record(stream)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize(dev)
    barrier()
    ms = e0.elapsed_time(e1)
    clocks = clk.summary()
    t_max = max_over_ranks(ms, dist, dev)
    bytes_step = algorithmic_bytes(cfg, G)
    value = world * bytes_step * args.steps / (t_max * 1e-3) / 1e9

    # end to end through the public host-buffer API: pinned f and records in, f out, every step
    f_host = torch.zeros(fo.shape, dtype=torch.float32).pin_memory()
    rec_host = torch.from_numpy(rec).pin_memory()
    ft_host = torch.from_numpy(fo).pin_memory()
    fa = f_host.numpy()
    barrier()
    t0 = time.perf_counter()
    for s in range(args.steps):
        ctx.iterate(w["method"], sched, s, fa, rec_host.numpy(), ft_host.numpy())
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_max = max_over_ranks(e2e_s, dist, dev)
    e2e_val = world * bytes_step * args.steps / e2e_max / 1e9
    h2d = 4 * (fo.size * 2 + rec.size)
    d2h = 4 * fo.size + 8

    tti = time_to_image(ctx, w, sched, d_f, d_ft, torch, dev) if args.workload == "c2" and not args.no_learned else None
    art = art_iteration(ctx, sched, d_f, d_ft, t_max / args.steps) if args.workload in ("c2", "c1") and not args.no_art \
        else None

    # roofline of the dominant kernel, timed live on the context stream
    info = ctx.info
    nt, K, nseg = cfg.nt, info.ckpt_interval, info.n_segments
    fwd_launches = (nt - 2) + (0 if nseg == 1 else (nseg - 1) * (K - 1))
    adj_launches = nt - 2
    fwd_ms, fwd_b = ctx.time_kernel(0, 200)
    adj_ms, adj_b = ctx.time_kernel(1, 200)
    share_f = fwd_launches * fwd_ms
    share_a = adj_launches * adj_ms
    dom = ("forward_step", fwd_ms, fwd_b) if share_f >= share_a else ("adjoint_step", adj_ms, adj_b)
    peak, peak_kind = peaks()
    achieved = dom[2] / (dom[1] * 1e-3) / 1e9
    traffic, tr_all = None, {}
    tpath = os.path.join(REPO, "profiles", f"traffic_{args.workload}.json")
    if os.path.exists(tpath) and args.nt <= 0:
        try:
            tr_all = json.load(open(tpath))
            traffic = tr_all.get(dom[0])
        except Exception:
            traffic, tr_all = None, {}
    # the sweep's time accounted by the per-step kernel times (graph-replayed, as in the iteration)
    sweep_ms = fwd_launches * fwd_ms + adj_launches * adj_ms

    if rank == 0:
        line = {
            "metric": metric_name(args.workload), "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded ellipse phantom + smoothed noise, 1% Gaussian record noise)",
            "config": {"workload": args.workload + ": " + w["desc"], "groups": G,
                       "groups_per_pass": info.groups_per_pass, "ckpt_interval": K,
                       "l2": "inputs larger than L2 (%.1f GB resident working set)" % (info.device_bytes / 1e9),
                       "parallelism": f"replicas{world}" if world > 1 else "single GPU",
                       "strip_kernels": tuning},
            "sirt_iter_per_s": world * args.steps / (t_max * 1e-3),
            "cell_updates_per_s": world * 2.0 * G * cfg.nx * cfg.ny * (nt - 2) * args.steps / (t_max * 1e-3),
            "epsilon_last": eps[-1] if eps else None,
            "gpu_launches": launches,
            "e2e": {"value": e2e_val, "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": {"kernel": dom[0], "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "ms_per_launch": dom[1], "bytes_per_launch": dom[2],
                         "other": {"forward_step_GBps": fwd_b / (fwd_ms * 1e-3) / 1e9,
                                   "adjoint_step_GBps": adj_b / (adj_ms * 1e-3) / 1e9,
                                   "forward_step_ms": fwd_ms, "adjoint_step_ms": adj_ms,
                                   "forward_steps": fwd_launches, "adjoint_steps": adj_launches,
                                   "steps_ms": sweep_ms,
                                   "algorithmic_bytes": {"forward_step": fwd_b, "adjoint_step": adj_b},
                                   "dram_bytes": {k: tr_all.get(k) for k in ("forward_step", "adjoint_step")}}},
            "clocks": clocks,
        }
        if tti is not None:
            line["time_to_image"] = tti
        if art is not None:
            line["art"] = art
        if cpu:
            line["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
