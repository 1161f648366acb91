"""Training and evaluation of the learned update (the 5-layer CNN in libtomo.so).

Pipeline, all compute in libtomo.so's kernels (torch only holds device buffers):
  1. data: seeded 256x256 ellipse phantoms (8 ellipses, axes 8..45 cells,
     f in U[-0.15, 0.15], smoothed noise 0.01), the 512x512 workload's physics
     scaled to 256x256 (nt 1250, 128 transducers on radius 110, groups of 8,
     1% record noise).  Plain weighted SIRT (normalised-weight direction,
     step `STEP` along the direction scaled to max 1) runs `iters` iterations
     per phantom; iteration t gives the pair
        features (f_t, direction_t, illumination)  ->  target  f_{t+K} - f_t
     the field change of the next K plain steps (the look-ahead K defaults to
     6): the network learns to jump ahead along the plain trajectory.
  2. training: Adam on the masked mean squared error, on the GPU.
  3. evaluation (time to image): on the 512x512 workload, plain weighted SIRT
     runs `plain_iters` iterations; the learned iteration (a network proposal
     is accepted only when it lowers the record residual by 5 %, else the plain
     step is taken, and after 2 rejections in a row only plain steps; see
     tomo_run_learned) runs until it reaches the plain method's final image
     error.

Usage:  python learn.py [--phantoms 400] [--iters 36] [--lookahead 6] [--epochs 12]
                        [--onpolicy-phantoms 200] [--out weights.bin]
        (the defaults are the settings of the shipped weights/learned_update.bin:
        12,400 pairs, network seed 7, data seeds 4000.., shuffling seed 0)
        python learn.py --eval-only --out weights.bin --eval-seeds 2001,2002
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import tomo  # noqa: E402

STEP = 0.02          # plain weighted SIRT step (direction scaled to max 1 over the mask)
LEARNED_SCALE = tomo.LEARNED_SCALE   # the proposal is f + LEARNED_SCALE * mask * net(features)
WEIGHTS = os.path.join(tomo.PKG_DIR, "weights", "learned_update.bin")


def train_config(device=0):
    return tomo.cfg_config(nx=256, ny=256, nt=1250, n_transducers=128, group_size=8, radius=110.0,
                           ckpt_interval=0, device=device)


def eval_config(device=0):
    return tomo.cfg_config(nx=512, ny=512, nt=2500, n_transducers=256, group_size=8, radius=220.0,
                           ckpt_interval=50, device=device)


def phantom(cfg, seed, rmin, rmax):
    return tomo.phantom_cfg(cfg.nx, cfg.ny, 1, 8, rmin, rmax, 0.15, 0.01, 0.8 * cfg.radius, seed)


TRAIN_RADII = (8.0, 45.0)   # range of the training ellipses' axes (diameters, cells)


def mask_of(cfg):
    y, x = np.mgrid[0:cfg.ny, 0:cfg.nx]
    r = cfg.radius - 1.5
    return (((x - 0.5 * cfg.nx) ** 2 + (y - 0.5 * cfg.ny) ** 2) < r * r).astype(np.float32)


def generate(n_phantoms, iters, lookahead=6, seed0=4000, device=0, target="lookahead", log=print):
    """Plain weighted SIRT trajectories -> (features [M,3,H,W], targets [M,H,W], mask [H,W]) on the GPU,
    M = n_phantoms * (iters - lookahead + 1).  target "lookahead": f_{t+K} - f_t; "truth":
    mask * (f_true - f_t), the update that would complete the image."""
    import torch

    dev = torch.device("cuda", device)
    cfg = train_config(device)
    m = torch.from_numpy(mask_of(cfg)).to(dev)
    per = iters - lookahead + 1
    M = n_phantoms * per
    feats = torch.empty((M, 3, cfg.ny, cfg.nx), dtype=torch.float32, device=dev)
    tgts = torch.empty((M, cfg.ny, cfg.nx), dtype=torch.float32, device=dev)
    traj = torch.empty((iters + 1, cfg.ny, cfg.nx), dtype=torch.float32, device=dev)
    feat_t = torch.empty((iters, 3, cfg.ny, cfg.nx), dtype=torch.float32, device=dev)
    t0 = time.time()
    j = 0
    with tomo.Context(cfg) as ctx:
        for ph in range(n_phantoms):
            fo = phantom(cfg, seed0 + ph, *TRAIN_RADII)
            ctx.set_records(ctx.generate_data(fo, noise_level=0.01, seed=seed0 + ph))
            d_fo = torch.from_numpy(fo).to(dev)
            traj[0].zero_()
            for it in range(iters):
                torch.cuda.synchronize(dev)   # torch writes the trajectory on its own stream
                ctx.features_device(traj[it].data_ptr(), feat_t[it].data_ptr())
                traj[it + 1] = traj[it] + STEP * m * feat_t[it, 1]      # the plain weighted SIRT step
            feats[j:j + per] = feat_t[:per]
            if target == "truth":
                tgts[j:j + per] = m * (d_fo - traj[:per])
            else:
                tgts[j:j + per] = traj[lookahead:lookahead + per] - traj[:per]
            j += per
            if ph % 100 == 0:
                log(f"  data: phantom {ph}/{n_phantoms}, {time.time() - t0:.1f} s")
    torch.cuda.synchronize(dev)
    return feats, tgts, m, time.time() - t0


def generate_onpolicy(net, n_phantoms, iters, lookahead=6, seed0=9000, device=0, log=print):
    """States the learned iteration itself visits (the residual check of tomo_run_learned, proposing
    at every state), each paired with the field change of `lookahead` plain weighted-SIRT
    steps taken from that state; a network trained on plain trajectories alone drifts off them.
    Returns (features [M,3,H,W], targets [M,H,W]), M = n_phantoms * iters."""
    import torch

    dev = torch.device("cuda", device)
    cfg = train_config(device)
    m = torch.from_numpy(mask_of(cfg)).to(dev)
    H, W = cfg.ny, cfg.nx
    M = n_phantoms * iters
    feats = torch.empty((M, 3, H, W), dtype=torch.float32, device=dev)
    tgts = torch.empty((M, H, W), dtype=torch.float32, device=dev)
    cur = torch.empty((3, H, W), dtype=torch.float32, device=dev)
    nxt = torch.empty_like(cur)
    tmp = torch.empty_like(cur)
    out = torch.empty((1, H, W), dtype=torch.float32, device=dev)
    t0 = time.time()
    j, acc = 0, 0
    with tomo.Context(cfg) as ctx:
        for ph in range(n_phantoms):
            fo = phantom(cfg, seed0 + ph, *TRAIN_RADII)
            ctx.set_records(ctx.generate_data(fo, noise_level=0.01, seed=seed0 + ph))
            f = torch.zeros((H, W), dtype=torch.float32, device=dev)
            torch.cuda.synchronize(dev)
            r0 = ctx.features_device(f.data_ptr(), cur.data_ptr())
            for t in range(iters):
                feats[j] = cur
                g = f + STEP * m * cur[1]
                for _ in range(lookahead - 1):
                    torch.cuda.synchronize(dev)
                    ctx.features_device(g.data_ptr(), tmp.data_ptr())
                    g = g + STEP * m * tmp[1]
                tgts[j] = g - f
                j += 1
                torch.cuda.synchronize(dev)
                net.forward_device(cur.data_ptr(), 1, H, W, out.data_ptr())
                fp = f + m * out[0]
                torch.cuda.synchronize(dev)
                r1 = ctx.features_device(fp.data_ptr(), nxt.data_ptr())
                if r1 <= (1.0 - tomo.LEARNED_MIN_DECREASE) * r0:
                    f, r0, acc = fp, r1, acc + 1
                    cur, nxt = nxt, cur
                else:
                    f = f + STEP * m * cur[1]
                    torch.cuda.synchronize(dev)
                    r0 = ctx.features_device(f.data_ptr(), cur.data_ptr())
            if ph % 50 == 0:
                log(f"  on-policy data: phantom {ph}/{n_phantoms}, {acc}/{j} accepted, {time.time() - t0:.1f} s")
    torch.cuda.synchronize(dev)
    return feats, tgts, time.time() - t0


def masked_mse(out, tgts, mask):
    """Mean over samples of sum(mask*(out-t)^2)/sum(mask)."""
    return float(((out - tgts) ** 2 * mask).sum() / (mask.sum() * out.shape[0]))


def baselines(feats, tgts, mask, lookahead):
    """Losses of two fixed predictors: zero, and lookahead plain steps along the current direction."""
    return {"zero": masked_mse(0 * tgts, tgts, mask),
            "linear": masked_mse(lookahead * STEP * feats[:, 1] * mask, tgts, mask)}


def evaluate(net, feats, tgts, mask, batch=16):
    import torch

    M, _, H, W = feats.shape
    out = torch.empty((batch, H, W), dtype=torch.float32, device=feats.device)
    acc, n = 0.0, 0
    for b in range(0, M - batch + 1, batch):
        fb = feats[b:b + batch].contiguous()
        torch.cuda.synchronize(feats.device)
        net.forward_device(fb.data_ptr(), batch, H, W, out.data_ptr())
        torch.cuda.synchronize(feats.device)
        acc += masked_mse(out, tgts[b:b + batch], mask) * batch
        n += batch
    return acc / max(n, 1)


def train(net, feats, tgts, mask, epochs, batch=16, lr=1e-3, seed=0, log=print):
    M, _, H, W = feats.shape
    bm = mask.expand(batch, H, W).contiguous()
    rng = np.random.default_rng(seed)
    steps = epochs * (M // batch)
    t0 = time.time()
    s = 0
    losses = []
    import torch

    for ep in range(epochs):
        perm = torch.from_numpy(rng.permutation(M)).to(feats.device)
        acc = 0.0
        for b in range(M // batch):
            idx = perm[b * batch:(b + 1) * batch]
            fb = feats[idx].contiguous()
            tb = tgts[idx].contiguous()
            torch.cuda.synchronize(feats.device)
            cur = lr * 0.5 * (1 + np.cos(np.pi * s / steps))      # cosine decay
            acc += net.train_step_device(fb.data_ptr(), tb.data_ptr(), bm.data_ptr(), batch, H, W, cur)
            s += 1
        losses.append(acc / max(M // batch, 1))
        log(f"  epoch {ep}: loss {losses[-1]:.3e}, {time.time() - t0:.1f} s")
    return losses, time.time() - t0


def time_to_image(net, plain_iters=30, seed=2001, device=0,
                  rules=((tomo.LEARNED_MIN_DECREASE, tomo.LEARNED_PATIENCE),), log=print):
    """Plain weighted SIRT for plain_iters iterations vs the learned iteration to the same image error."""
    import torch

    dev = torch.device("cuda", device)
    cfg = eval_config(device)
    fo = phantom(cfg, seed, 10.0, 60.0)
    sched = tomo.schedule(omega=STEP, normalize=1)
    out = {}
    with tomo.Context(cfg) as ctx:
        rec = ctx.generate_data(fo, noise_level=0.01, seed=77)
        d_fo = torch.from_numpy(fo).to(dev)
        d_rec = torch.from_numpy(rec).to(dev)
        d_f = torch.zeros_like(d_fo)
        torch.cuda.synchronize(dev)
        ctx.iterate_device(tomo.SIRT_NORM, sched, 0, d_f.data_ptr(), d_rec.data_ptr(), d_fo.data_ptr())
        d_f.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eps = []
        for it in range(plain_iters):
            st = ctx.iterate_device(tomo.SIRT_NORM, sched, it, d_f.data_ptr(), 0, d_fo.data_ptr())
            eps.append(st.epsilon)
        ctx.synchronize()
        t_plain = time.perf_counter() - t0
        target = eps[-1]
        log(f"  plain: {plain_iters} iterations, eps {eps[0]:.3f} -> {target:.3f} %, {t_plain:.3f} s")
        d_f.zero_()
        torch.cuda.synchronize(dev)
        ctx.run_learned(net, sched, d_f.data_ptr(), d_fo.data_ptr(), -1.0, 1)   # warm up (illumination, graphs)
        out = {"plain_iters": plain_iters, "plain_seconds": t_plain, "plain_final_epsilon": target,
               "plain_epsilon": eps, "learned": {}}
        for rule in rules:
            md, pat = rule[0], rule[1]
            scale = rule[2] if len(rule) > 2 else LEARNED_SCALE
            back = rule[3] if len(rule) > 3 else 0
            resume = rule[4] if len(rule) > 4 else 0
            ctx.set_learned_scale(scale)
            ctx.set_learned_backtrack(back)
            ctx.set_learned_resume(resume)
            d_f.zero_()
            torch.cuda.synchronize(dev)
            leps, kind, sweeps, t_learned = ctx.run_learned(net, sched, d_f.data_ptr(), d_fo.data_ptr(), target,
                                                            3 * plain_iters, md, pat)
            leps = [float(e) for e in leps]
            reached = bool(leps[-1] <= target)
            steps = "".join({1: "L", 2: "l", 0: "x", -1: "p"}[int(k)] for k in kind)
            log(f"  learned (min decrease {md}, patience {pat}, scale {scale}, backtrack {back}, resume {resume}): "
                f"{steps}, "
                f"{sweeps} sweeps, "
                f"eps -> {leps[-1]:.3f} %, {t_learned:.3f} s, speedup "
                f"{t_plain / t_learned if reached else float('nan'):.2f}")
            out["learned"]["%g/%d/%g/%d/%d" % (md, pat, scale, back, resume)] = {
                "iters": len(leps), "steps": steps, "sweeps": sweeps, "seconds": t_learned,
                "final_epsilon": leps[-1], "epsilon": leps, "reached": reached,
                "speedup": t_plain / t_learned if reached else None}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--phantoms", type=int, default=400)
    ap.add_argument("--iters", type=int, default=36)
    ap.add_argument("--lookahead", type=int, default=6)
    ap.add_argument("--target", default="lookahead", choices=["lookahead", "truth"])
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--onpolicy-phantoms", type=int, default=0)
    ap.add_argument("--onpolicy-iters", type=int, default=20)
    ap.add_argument("--eval-only", action="store_true")
    ap.add_argument("--eval-seeds", default="2001", help="comma-separated phantom seeds of the evaluation")
    ap.add_argument("--eval-scales", default="", help="comma-separated learned-step scales to evaluate "
                                                         "(default: the shipped one)")
    ap.add_argument("--eval-rules", default="", help="comma-separated scale:backtrack[:resume] rules to evaluate "
                                                        "(backtrack: retries of a rejected proposal at half scale; "
                                                        "resume: plain steps before paused proposals resume)")
    args = ap.parse_args()
    import torch

    net = tomo.Net(0, seed=7)
    report = {}
    if not args.eval_only:
        feats, tgts, m, t_data = generate(args.phantoms, args.iters, args.lookahead, target=args.target)
        report["target"] = args.target
        report["lookahead"] = args.lookahead
        report["pairs"] = int(feats.shape[0])
        report["data_seconds"] = t_data
        nval = max(16, int(0.05 * feats.shape[0]) // 16 * 16)      # held out: the last phantoms
        if feats.shape[0] < nval + 16:
            raise SystemExit(f"{feats.shape[0]} pairs: need at least {nval + 16} (more phantoms or iterations)")
        fv, tv = feats[-nval:], tgts[-nval:]
        feats, tgts = feats[:-nval], tgts[:-nval]
        report["baseline_loss"] = baselines(fv, tv, m, args.lookahead)
        print(f"  held-out baselines: {report['baseline_loss']}")
        losses, t_train = train(net, feats, tgts, m, args.epochs, args.batch, args.lr)
        report["losses"] = losses
        report["train_seconds"] = t_train
        report["val_loss"] = evaluate(net, fv, tv, m)
        print(f"  held-out loss {report['val_loss']:.3e}")
        if args.onpolicy_phantoms > 0:
            # a second round on the states the trained network's own iteration visits
            os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
            net.save(args.out + ".round1")
            fo_, to_, t_on = generate_onpolicy(net, args.onpolicy_phantoms, args.onpolicy_iters, args.lookahead)
            report["onpolicy_pairs"] = int(fo_.shape[0])
            report["onpolicy_seconds"] = t_on
            feats, tgts = torch.cat([feats, fo_]), torch.cat([tgts, to_])
            del fo_, to_
            net = tomo.Net(0, seed=7)
            losses, t_train = train(net, feats, tgts, m, args.epochs, args.batch, args.lr, seed=1)
            report["losses_round2"] = losses
            report["train_seconds"] += t_train
            report["val_loss_round2"] = evaluate(net, fv, tv, m)
            print(f"  held-out loss after the on-policy round {report['val_loss_round2']:.3e}")
        os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
        net.save(args.out)
        del feats, tgts, fv, tv
    else:
        net.load(args.out)
    report["time_to_image"] = {}
    for seed in [int(x) for x in args.eval_seeds.split(",")]:
        print(f"  evaluation phantom seed {seed}")
        if args.eval_rules:
            rules = tuple((tomo.LEARNED_MIN_DECREASE, tomo.LEARNED_PATIENCE, float(x.split(":")[0]),
                           int(x.split(":")[1]), int(x.split(":")[2]) if x.count(":") > 1 else 0)
                          for x in args.eval_rules.split(","))
        else:
            rules = tuple((tomo.LEARNED_MIN_DECREASE, tomo.LEARNED_PATIENCE, float(x))
                          for x in (args.eval_scales.split(",") if args.eval_scales else [LEARNED_SCALE]))
        report["time_to_image"][str(seed)] = time_to_image(net, seed=seed, rules=rules)
    print(json.dumps(report))


if __name__ == "__main__":
    main()
