"""GPU parity against the committed golden vectors (tests/golden/oracle_small.npz).

The CUDA path (libtomo.so) is run on the vectors' inputs and compared with the FP64
oracle's outputs stored there, at the tolerances stored beside them: records and last
wavefield 1e-5, gradients and images 1e-4 relative L2, epsilon 1e-4 relative, each
widened on the reference profile to three times the distance of the reference scheme's
own FP32 arithmetic from FP64 (the same rule as tests/test_gpu_parity.py).  No oracle
code runs here: the numbers come from the committed file.
"""
import json
import os

import numpy as np
import pytest

import tomo

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_small.npz")


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def load():
    d = np.load(GOLDEN)
    return d, json.loads(str(d["meta"]))


def config(meta, name):
    c = meta["cases"][name]
    return tomo.ref_config(**c["config"]) if c["profile"] == "ref" else tomo.cfg_config(**c["config"])


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", ["ref", "cfg"])
def test_forward_matches_golden(name):
    d, meta = load()
    cfg = config(meta, name)
    tol_u, tol_r = d[f"{name}/fwd/tol"]
    with tomo.Context(cfg) as ctx:
        rec, ul = ctx.forward(d[f"{name}/fwd/f"], u_last=True)
    assert rel(rec, d[f"{name}/fwd/records"]) <= tol_r
    assert rel(ul, d[f"{name}/fwd/u_last"]) <= tol_u


@pytest.mark.parametrize("name", ["ref", "cfg"])
def test_gradient_matches_golden(name):
    d, meta = load()
    cfg = config(meta, name)
    tol = d[f"{name}/grad/tol"][0]
    dfg_o = d[f"{name}/grad/dfg"]
    with tomo.Context(cfg) as ctx:
        dfg, df, r2 = ctx.gradient(d[f"{name}/grad/f"], d[f"{name}/fwd/records"])
    assert rel(dfg, dfg_o) <= tol
    assert rel(df, dfg_o.astype(np.float64).sum(0)) <= tol
    assert abs(r2 - d[f"{name}/grad/resid2"][0]) <= d[f"{name}/grad/resid2_tol"][0]


@pytest.mark.parametrize("name", ["ref", "cfg"])
def test_sirt_iterations_match_golden(name):
    d, meta = load()
    cfg = config(meta, name)
    run = meta["runs"][name]
    sched = tomo.schedule(**run["schedule"])
    fo = d[f"{name}/fwd/f"]
    f = np.zeros_like(fo)
    with tomo.Context(cfg) as ctx:
        ctx.set_records(d[f"{name}/fwd/records"])
        for it in range(run["iterations"]):
            st = ctx.iterate(run["method"], sched, it, f, None, fo)
            assert rel(f, d[f"{name}/iter/images"][it]) <= d[f"{name}/iter/tol"][it], it
            assert abs(st.epsilon - d[f"{name}/iter/epsilon"][it]) <= d[f"{name}/iter/eps_tol"][it], it
