"""The oracle reproduces its frozen golden vectors (tests/golden/oracle_small.npz).

The vectors hold the FP64 oracle's records, last wavefields, per-group gradients,
residuals and SIRT images on a small reference-profile and a small benchmark-profile
problem (made by tests/golden/make_oracle_fixtures.py).  The GPU parity tests compare
the CUDA path with the same vectors (tests/test_gpu_golden.py).  Stored arrays are
float32, so the oracle's FP64 results match them to float32 rounding.
"""
import json
import os

import numpy as np
import pytest

import oracle_lib as O
import tomo

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_small.npz")
F32 = 1e-6   # relative L2 of a float32-rounded copy


def load():
    d = np.load(GOLDEN)
    meta = json.loads(str(d["meta"]))
    return d, meta


def config(meta, name):
    c = meta["cases"][name]
    return tomo.ref_config(**c["config"]) if c["profile"] == "ref" else tomo.cfg_config(**c["config"])


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", ["ref", "cfg"])
def test_oracle_reproduces_golden(name):
    d, meta = load()
    cfg = config(meta, name)
    fo = d[f"{name}/fwd/f"]
    rec, ul = O.forward(cfg, fo.astype(np.float64), u_last=True)
    assert rel(rec, d[f"{name}/fwd/records"]) <= F32
    assert rel(ul, d[f"{name}/fwd/u_last"]) <= F32
    meas = d[f"{name}/fwd/records"]
    dfg, r2 = O.gradient(cfg, d[f"{name}/grad/f"].astype(np.float64), meas)
    assert rel(dfg, d[f"{name}/grad/dfg"]) <= 1e-5   # measured records enter as float32 either way
    assert abs(r2 - d[f"{name}/grad/resid2"][0]) <= 1e-6 * r2
    run = meta["runs"][name]
    sched = tomo.schedule(**run["schedule"])
    f = np.zeros(fo.shape, np.float64)
    for it in range(run["iterations"]):
        eps = O.iterate(cfg, run["method"], sched, it, f, meas, fo.astype(np.float64))[0]
        assert rel(f, d[f"{name}/iter/images"][it]) <= 1e-5, it
        assert abs(eps - d[f"{name}/iter/epsilon"][it]) <= 1e-6 * eps, it


def test_golden_tolerances_are_stated():
    d, meta = load()
    for name in meta["cases"]:
        assert d[f"{name}/fwd/tol"].shape == (2,) and np.all(d[f"{name}/fwd/tol"] >= 1e-5)
        assert np.all(d[f"{name}/grad/tol"] >= 1e-4) and np.all(d[f"{name}/iter/tol"] >= 1e-4)
        # the widened reference-profile bounds stay well below 1 %
        assert np.all(d[f"{name}/grad/tol"] < 1e-2) and np.all(d[f"{name}/iter/tol"] < 1e-2)
