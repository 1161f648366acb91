"""Freeze the oracle's outputs on small seeded problems as golden vectors.

Writes tests/golden/oracle_small.npz: for a reference-profile problem (40x40 grid, nt 100,
sensor ring 6..33, 4 groups of 27) and a benchmark-profile problem (72x64, nt 180, 24
transducers in groups of 4), the inputs (phantom, perturbed field) and the FP64 oracle's
records and last wavefield of a forward solve of the phantom, the per-group gradients and
residual at the perturbed field against those records, and the images and epsilons of a few
normalised SIRT iterations from f = 0, each with its parity tolerance (the
reference-profile bounds are widened to three times the distance of the reference scheme's
FP32 arithmetic from FP64, as in the live parity tests).  The oracle itself is pinned
against the reference's recorded epsilon logs (ref_eps_logs.json); these vectors freeze its
output so that a change of the oracle or of the CUDA path shows against committed numbers.

Usage (repository root): python tests/golden/make_oracle_fixtures.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "tomographic-image-reconstruction-algorithms_gb300", "python"))

import oracle_lib as O  # noqa: E402
import tomo  # noqa: E402

OUT = os.path.join(HERE, "oracle_small.npz")

CASES = {
    "ref": ("ref", dict(nx=40, ny=40, nt=100, ring_lo=6, ring_hi=33, group_size=27)),
    "cfg": ("cfg", dict(nx=72, ny=64, nt=180, n_transducers=24, group_size=4, radius=24.0,
                        cells_per_wavelength=10.0, sponge_width=8)),
}
# per case: method, schedule, iterations
RUNS = {
    "ref": (tomo.SIRT_NORM, dict(kind=tomo.SCHED_POWER, omega=3e4, alpha=0.5, beta=0.5, gamma=1.5), 3),
    "cfg": (tomo.SIRT_NORM, dict(omega=0.02, normalize=1), 2),
}
TOL_FIELD, TOL_GRAD, TOL_IMG = 1e-5, 1e-4, 1e-4


def make_config(profile, kw):
    return tomo.ref_config(**kw) if profile == "ref" else tomo.cfg_config(**kw)


def blob_phantom(ny, nx, seed=0, amp=0.05):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:ny, 0:nx]
    f = np.zeros((ny, nx))
    for _ in range(3):
        cx, cy = rng.uniform(0.35, 0.65) * nx, rng.uniform(0.35, 0.65) * ny
        r = rng.uniform(3, 7)
        f += rng.uniform(-amp, amp) * (((x - cx) ** 2 + (y - cy) ** 2) <= r * r)
    return f.astype(np.float32)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def main():
    out = {}
    meta = {"cases": {}, "runs": {}}
    for name, (profile, kw) in CASES.items():
        cfg = make_config(profile, kw)
        ref = profile == "ref"
        meta["cases"][name] = {"profile": profile, "config": kw}
        # forward solve of the phantom; its records are the measured data of the other cases
        fo = blob_phantom(cfg.ny, cfg.nx, seed=1, amp=0.05 if ref else 0.1)
        rec, ul = O.forward(cfg, fo.astype(np.float64), u_last=True)
        tol_u = tol_r = TOL_FIELD
        if ref:
            rec32, ul32 = O.forward(cfg, fo.astype(np.float64), prec=32, u_last=True)
            tol_u, tol_r = max(TOL_FIELD, 3 * rel(ul32, ul)), max(TOL_FIELD, 3 * rel(rec32, rec))
        out[f"{name}/fwd/f"] = fo
        out[f"{name}/fwd/records"] = rec.astype(np.float32)
        out[f"{name}/fwd/u_last"] = ul.astype(np.float32)
        out[f"{name}/fwd/tol"] = np.array([tol_u, tol_r])
        # gradient of every group at a perturbed field
        meas = rec
        f = blob_phantom(cfg.ny, cfg.nx, seed=2, amp=0.01)
        dfg, r2 = O.gradient(cfg, f.astype(np.float64), meas)
        tol_g, tol_r2 = TOL_GRAD, 1e-4 * r2
        if ref:
            dfg32, r2_32 = O.gradient(cfg, f.astype(np.float64), meas, prec=32)
            tol_g, tol_r2 = max(TOL_GRAD, 3 * rel(dfg32, dfg)), max(tol_r2, 3 * abs(r2_32 - r2))
        out[f"{name}/grad/f"] = f
        out[f"{name}/grad/dfg"] = dfg.astype(np.float32)
        out[f"{name}/grad/resid2"] = np.array([r2])
        out[f"{name}/grad/tol"] = np.array([tol_g])
        out[f"{name}/grad/resid2_tol"] = np.array([tol_r2])
        # a few SIRT iterations from f = 0
        method, sched_kw, n_it = RUNS[name]
        sched = tomo.schedule(**sched_kw)
        fi, meas_i = fo, rec
        f_o = np.zeros(fi.shape, np.float64)
        f_32 = np.zeros(fi.shape, np.float64)
        imgs, eps, tols, eps_tol = [], [], [], []
        for it in range(n_it):
            e_o = O.iterate(cfg, method, sched, it, f_o, meas_i, fi.astype(np.float64))[0]
            tol_i, tol_e = TOL_IMG, 1e-4 * e_o
            if ref:
                e_32 = O.iterate(cfg, method, sched, it, f_32, meas_i, fi.astype(np.float64), prec=32)[0]
                tol_i, tol_e = max(TOL_IMG, 3 * rel(f_32, f_o)), max(1e-4 * e_o, 3 * abs(e_32 - e_o))
            imgs.append(f_o.astype(np.float32))
            eps.append(e_o)
            tols.append(tol_i)
            eps_tol.append(tol_e)
        meta["runs"][name] = {"method": method, "schedule": sched_kw, "iterations": n_it}
        out[f"{name}/iter/images"] = np.stack(imgs)
        out[f"{name}/iter/epsilon"] = np.array(eps)
        out[f"{name}/iter/tol"] = np.array(tols)
        out[f"{name}/iter/eps_tol"] = np.array(eps_tol)
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
