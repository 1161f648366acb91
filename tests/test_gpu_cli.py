"""GPU checks of the command-line drivers built on the C ABI: the hybrid ART -> SIRT driver
(sirt-mimo-seq.cu) and the alternating-relaxation driver (sirt-mimo-norm-alt.cu) give the
same epsilons and image as the same method/schedule sequence through tomo_iterate, and the
FP64 oracle replaying that sequence on the same records gives the same epsilons and image
within the reference-profile parity bars (1e-4 relative, widened to three times the
reference scheme's own FP32-vs-FP64 distance where that is larger)."""
import os
import subprocess

import numpy as np
import pytest

import oracle_lib as O
import tomo

pytestmark = pytest.mark.gpu

BIN = os.path.join(os.path.dirname(tomo.LIB_PATH), "..", "bin")


def run(tmp, *args):
    r = subprocess.run([os.path.join(BIN, args[0]), *args[1:]], cwd=tmp, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout


def table_eps(out):
    """(iter, epsilon) rows of the normalised drivers' table."""
    rows = []
    for line in out.splitlines():
        parts = line.split()
        if len(parts) >= 3 and parts[0].isdigit():
            rows.append(float(parts[1]))
    return rows


def api_run(methods, scales, gs=160):
    cfg = tomo.ref_config(group_size=gs)
    with tomo.Context(cfg) as ctx:
        fo = tomo.phantom_ref()
        rec = ctx.generate_data(fo)
        f = np.zeros_like(fo)
        eps, prev = [], 100.0
        for it, (m, sc) in enumerate(zip(methods, scales)):
            st = ctx.iterate(m, sc, it, f, rec, fo)
            e = float(np.float32(st.epsilon))
            eps.append(e)
            if e > prev:
                break
            prev = e
    return eps, f


def oracle_replay(methods, scales, rec, fo, prec, gs=160):
    """The oracle's epsilons and image for the same sequence and stopping rule."""
    cfg = tomo.ref_config(group_size=gs)
    f = np.zeros(fo.shape, np.float64)
    eps, prev = [], 100.0
    for it, (m, sc) in enumerate(zip(methods, scales)):
        e = O.iterate(cfg, m, sc, it, f, rec, fo.astype(np.float64), prec=prec)[0]
        eps.append(e)
        if e > prev:
            break
        prev = e
    return eps, f


def check_against_oracle(eps_cli, img_cli, methods, scales, tmp):
    """eps_cli and the driver's image against the oracle on the driver's own records."""
    fo = tomo.phantom_ref()
    with tomo.Context(tomo.ref_config(group_size=160)) as ctx:
        rec = ctx.generate_data(fo)            # the records generate-data wrote, bit for bit
    eps64, f64 = oracle_replay(methods, scales, rec, fo, 64)
    eps32, f32 = oracle_replay(methods, scales, rec, fo, 32)
    n = min(len(eps_cli), len(eps64), len(eps32))
    assert n >= 5
    for it in range(n):
        tol = max(1e-4 * eps64[it], 3 * abs(eps32[it] - eps64[it]))
        assert abs(eps_cli[it] - eps64[it]) <= tol, (it, eps_cli[it], eps64[it], tol)
    if len(eps_cli) == len(eps64) == len(eps32):
        tol = max(1e-4, 3 * (np.linalg.norm(f32 - f64) / np.linalg.norm(f64)))
        err = np.linalg.norm(img_cli - f64) / np.linalg.norm(f64)
        assert err <= tol, (f"image vs oracle {err:.2e} (bar {tol:.2e}); image error vs phantom "
                            f"{100 * np.linalg.norm(img_cli - fo) / np.linalg.norm(fo):.3f} %")


def prepare(tmp):
    run(tmp, "generate-field")
    run(tmp, "generate-data", "fo.txt", "160")


def test_cli_hybrid_art_then_sirt(built_lib, tmp_path):
    prepare(tmp_path)
    out = run(tmp_path, "sirt-mimo-seq", "fo.txt", "160", "0", "7", "1e4", "0.5", "0.5", "1")
    eps_cli = table_eps(out)
    sched = tomo.schedule(tomo.SCHED_POWER, 1e4, 0.5, 0.5, 1.0)
    eps_api, f_api = api_run([tomo.ART] * 5 + [tomo.SIRT_NORM] * 2, [sched] * 7)
    assert len(eps_cli) == len(eps_api) and np.all(np.isfinite(eps_api)) and eps_api[-1] < eps_api[0]
    assert np.allclose(eps_cli, eps_api, rtol=1e-6, atol=0)
    img = np.array(open(tmp_path / "sirt-norm-160-fo.txt").read().split(), np.float32).reshape(192, 192)
    if len(eps_api) == 7:
        assert np.array_equal(img, f_api)
    check_against_oracle(eps_cli, img, [tomo.ART] * 5 + [tomo.SIRT_NORM] * 2, [sched] * 7, tmp_path)


def test_cli_alternating_relaxation(built_lib, tmp_path):
    prepare(tmp_path)
    out = run(tmp_path, "sirt-mimo-norm-alt", "fo.txt", "160", "0", "0", "6", "10", "2", "1", "6", "1", "1")
    eps_cli = table_eps(out)
    scales = []
    for it in range(6):
        k = it + 1
        s = 1e4 + 2e3 / k if k % 2 else 6e3 - 1e3 / k
        scales.append(tomo.schedule(tomo.SCHED_CONST, np.float32(s)))
    eps_api, f_api = api_run([tomo.SIRT_NORM] * 6, scales)
    assert len(eps_cli) == len(eps_api) and np.all(np.isfinite(eps_api))
    assert np.allclose(eps_cli, eps_api, rtol=1e-6, atol=0)
    img = np.array(open(tmp_path / "sirt-norm-160-fo.txt").read().split(), np.float32).reshape(192, 192)
    check_against_oracle(eps_cli, img, [tomo.SIRT_NORM] * 6, scales, tmp_path)


def test_cli_binary_files_match_text(built_lib, tmp_path):
    """generate-data and sirt-mimo-norm on the binary form give the text form's numbers bit for bit."""
    txt, bn = tmp_path / "txt", tmp_path / "bin"
    txt.mkdir()
    bn.mkdir()
    prepare(txt)
    run(bn, "generate-field", "--binary")
    run(bn, "generate-data", "fo.bin", "160")
    for side in ("bottom", "right", "top", "left"):
        a = np.array(open(txt / f"fo-data-{side}-160.txt").read().split(), np.float32)
        raw = open(bn / f"fo-data-{side}-160.bin", "rb").read()
        assert raw[:8] == b"TOMOF32\n"
        assert np.array_equal(a, np.frombuffer(raw[24:], "<f4"))
    args = ["160", "0", "3", "1e5", "0.5", "0.5", "1"]
    out_t = run(txt, "sirt-mimo-norm", "fo.txt", *args)
    out_b = run(bn, "sirt-mimo-norm", "fo.bin", *args)
    assert table_eps(out_t) == table_eps(out_b)
    img_t = np.array(open(txt / "sirt-norm-160-fo.txt").read().split(), np.float32)
    raw = open(bn / "sirt-norm-160-fo.bin", "rb").read()
    assert np.array_equal(img_t, np.frombuffer(raw[24:], "<f4"))
