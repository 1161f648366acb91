"""Pin the CPU oracle to the reference's own recorded outputs.

The reference ships epsilon-per-iteration logs of its line-search SIRT drivers
(data_dynamic/, kept as tests/golden/ref_eps_logs.json).  Replaying each log's
recorded step sizes on generate-field's phantom with generate-data's records
must reproduce the logged epsilon.  Across all eight noise-free logs the FP64
oracle lands 1.7e-4 .. 7e-4 (relative) below the logged values, consistently
on the better side, and the oracle's own grid line search picks the logged
step (or its neighbour on the 100-step grid).  A wrong sensor row, injection
sign, mask or scale moves epsilon by percents, far outside these bounds.
"""
import json
import os

import numpy as np
import pytest

import oracle_lib as O
import tomo

HERE = os.path.dirname(os.path.abspath(__file__))
LOGS = json.load(open(os.path.join(HERE, "golden", "ref_eps_logs.json")))
METHOD = {"scaled": tomo.SIRT_SCALED, "norm": tomo.SIRT_NORM}

# (file, iterations replayed, relative bound)
CASES = [
    ("sirt-dyn-160-0.txt", 4, 1e-3),
    ("sirt-norm-dyn-160-0.txt", 4, 1e-3),
    ("sirt-dyn-32-0.txt", 2, 1e-3),
    ("sirt-norm-dyn-32-0.txt", 2, 1e-3),
    ("sirt-dyn-20-0.txt", 2, 1e-3),
    ("sirt-norm-dyn-20-0.txt", 2, 1e-3),
    ("sirt-dyn-10-0.txt", 2, 1e-3),
    ("sirt-norm-dyn-10-0.txt", 2, 1e-3),
]


@pytest.fixture(scope="module")
def phantom():
    return O.phantom_ref().astype(np.float64)


@pytest.mark.parametrize("name,n_it,bound", CASES, ids=[c[0] for c in CASES])
def test_replay_recorded_steps(phantom, name, n_it, bound):
    log = LOGS[name]
    cfg = tomo.ref_config(group_size=log["group_size"])
    meas = O.forward(cfg, phantom)
    f = np.zeros_like(phantom)
    for it in range(n_it):
        step = log["rows"][it][3]
        eps = O.iterate(cfg, METHOD[log["method"]], tomo.schedule(omega=step), it, f, meas, phantom)[0]
        ref_eps = log["rows"][it][1]
        assert abs(eps / ref_eps - 1) < bound, (it, eps, ref_eps)


def test_line_search_picks_recorded_step(phantom):
    """sirt-test-weight.cu:320-405: best of steps 0,100,...,1e6 against the phantom."""
    log = LOGS["sirt-dyn-160-0.txt"]
    cfg = tomo.ref_config(group_size=160)
    meas = O.forward(cfg, phantom)
    dfg, _ = O.gradient(cfg, np.zeros_like(phantom), meas)
    m = O.mask(cfg).astype(bool)
    d = np.where(m, dfg.sum(0) / dfg.shape[0], 0.0)
    steps = np.arange(0, 1e6 + 1, 100.0)
    r = -phantom
    eps = 100 * np.sqrt((r * r).sum() + 2 * steps * (r * d).sum() + steps ** 2 * (d * d).sum()) / np.linalg.norm(phantom)
    best = steps[int(np.argmin(eps))]
    assert abs(best - log["rows"][0][3]) <= 100


def test_phantom_matches_generate_field():
    fo = O.phantom_ref()
    assert fo.shape == (192, 192)
    assert set(np.unique(fo)) == {0.0, np.float32(0.03), np.float32(0.05)}
    # the 15 mm disc centred at cell (100, 100), small discs of 5 mm
    assert fo[100, 100] == np.float32(0.03)
    assert (fo == np.float32(0.05)).sum() > 3 * 60


def test_transducer_ring_matches_position_transducers():
    cfg = tomo.ref_config()
    ii, jj = O.transducers(cfg)
    # sirt-mimo.cu:443-465, 1-based
    assert (ii[0], jj[0]) == (22, 181) and (ii[159], jj[159]) == (181, 181)
    assert (ii[160], jj[160]) == (181, 180) and (ii[319], jj[319]) == (181, 21)
    assert (ii[320], jj[320]) == (180, 21) and (ii[479], jj[479]) == (21, 21)
    assert (ii[480], jj[480]) == (21, 22) and (ii[639], jj[639]) == (21, 181)
