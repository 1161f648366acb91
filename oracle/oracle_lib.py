"""ctypes loader of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference arm of bench.py, never by the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "tomographic-image-reconstruction-algorithms_gb300", "python"))
import tomo  # noqa: E402  (ctypes struct layouts shared with include/tomo.h)

LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


def build(force: bool = False) -> str:
    """Compile liboracle.so (serial/OpenMP C++; -ffp-contract=off so x86 and Arm agree)."""
    src = os.path.join(HERE, "oracle.cpp")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "oracle.h")),
            os.path.getmtime(os.path.join(REPO, "include", "tomo.h"))):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-I" + os.path.join(REPO, "include"), src, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_L = None


def lib() -> C.CDLL:
    global _L
    if _L is None:
        L = C.CDLL(build())
        CP, DP, FP, IP = (C.POINTER(tomo.Config), C.POINTER(C.c_double), C.POINTER(C.c_float),
                          C.POINTER(C.c_int32))
        i32 = C.c_int32
        L.orc_info_get.argtypes = [CP, C.POINTER(C.c_int32 * 3)]
        L.orc_transducers.argtypes = [CP, IP, IP]
        L.orc_mask.argtypes = [CP, C.POINTER(C.c_uint8)]
        L.orc_phantom_ref.argtypes = [i32, i32, FP]
        L.orc_forward.argtypes = [CP, i32, i32, DP, FP, DP]
        L.orc_gradient.argtypes = [CP, i32, i32, DP, FP, DP, DP]
        L.orc_gradient_groups.argtypes = [CP, i32, i32, DP, FP, i32, i32, DP, DP]
        L.orc_iterate.argtypes = [CP, i32, i32, i32, C.POINTER(tomo.Schedule), i32, DP, FP, DP, DP]
        L.orc_sweep.argtypes = [CP, i32, i32, DP, FP, i32, i32, DP]
        for n in ("orc_info_get", "orc_transducers", "orc_mask", "orc_phantom_ref", "orc_forward",
                  "orc_gradient", "orc_gradient_groups", "orc_iterate", "orc_sweep"):
            getattr(L, n).restype = i32
        _L = L
    return _L


def _chk(st, what):
    if st:
        raise RuntimeError(f"oracle {what} failed with status {st}")


def _d(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _f(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def info(cfg):
    out = (C.c_int32 * 3)()
    _chk(lib().orc_info_get(C.byref(cfg), C.byref(out)), "info")
    return {"n_groups": out[0], "n_channels": out[1], "n_transducers": out[2]}


def transducers(cfg):
    n = info(cfg)["n_transducers"]
    ii = np.zeros(n, np.int32)
    jj = np.zeros(n, np.int32)
    _chk(lib().orc_transducers(C.byref(cfg), ii.ctypes.data_as(C.POINTER(C.c_int32)),
                               jj.ctypes.data_as(C.POINTER(C.c_int32))), "transducers")
    return ii, jj


def mask(cfg):
    m = np.zeros((cfg.ny, cfg.nx), np.uint8)
    _chk(lib().orc_mask(C.byref(cfg), m.ctypes.data_as(C.POINTER(C.c_uint8))), "mask")
    return m


def phantom_ref(nx=192, ny=192):
    fo = np.zeros((ny, nx), np.float32)
    _chk(lib().orc_phantom_ref(nx, ny, _f(fo)), "phantom_ref")
    return fo


def forward(cfg, f, prec=64, threads=0, u_last=False):
    inf = info(cfg)
    f = np.ascontiguousarray(f, np.float64)
    rec = np.zeros((inf["n_groups"], cfg.nt, inf["n_channels"]), np.float32)
    ul = np.zeros((inf["n_groups"], cfg.ny, cfg.nx), np.float64) if u_last else None
    _chk(lib().orc_forward(C.byref(cfg), prec, threads, _d(f), _f(rec), _d(ul)), "forward")
    return (rec, ul) if u_last else rec


def gradient(cfg, f, meas, prec=64, threads=0):
    inf = info(cfg)
    f = np.ascontiguousarray(f, np.float64)
    meas = np.ascontiguousarray(meas, np.float32)
    dfg = np.zeros((inf["n_groups"], cfg.ny, cfg.nx), np.float64)
    r2 = C.c_double()
    _chk(lib().orc_gradient(C.byref(cfg), prec, threads, _d(f), _f(meas), _d(dfg), C.byref(r2)), "gradient")
    return dfg, r2.value


def gradient_groups(cfg, f, meas, g0, ng, prec=64, threads=0):
    """Per-group gradients of groups g0 .. g0+ng-1 only (ng, ny, nx) and their squared residual."""
    f = np.ascontiguousarray(f, np.float64)
    meas = np.ascontiguousarray(meas, np.float32)
    dfg = np.zeros((ng, cfg.ny, cfg.nx), np.float64)
    r2 = C.c_double()
    _chk(lib().orc_gradient_groups(C.byref(cfg), prec, threads, _d(f), _f(meas), g0, ng, _d(dfg), C.byref(r2)),
         "gradient_groups")
    return dfg, r2.value


def iterate(cfg, method, sched, it, f, meas, f_true=None, prec=64, threads=0):
    """One iteration in place on the float64 array f; returns (eps, resid2, scale)."""
    assert f.dtype == np.float64 and f.flags.c_contiguous
    stats = np.zeros(3, np.float64)
    ft = None if f_true is None else np.ascontiguousarray(f_true, np.float64)
    _chk(lib().orc_iterate(C.byref(cfg), prec, threads, method, C.byref(sched), it, _d(f),
                           _f(np.ascontiguousarray(meas, np.float32)), _d(ft), _d(stats)), "iterate")
    return tuple(stats)


def sweep(cfg, f, meas, g0, ng, prec=32, threads=0):
    cu = C.c_double()
    _chk(lib().orc_sweep(C.byref(cfg), prec, threads, _d(np.ascontiguousarray(f, np.float64)),
                         _f(np.ascontiguousarray(meas, np.float32)), g0, ng, C.byref(cu)), "sweep")
    return cu.value
