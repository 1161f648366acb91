"""Build recipe of libtomo.so and the CLI drivers (nvcc, sm_103a only).

Every translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a``; outputs stay in-tree:
``lib/libtomo.so`` and ``bin/<driver>``.  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CLI = os.path.join(PKG, "cli")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib", "libtomo.so")
BIN = os.path.join(PKG, "bin")
INCLUDE = os.path.join(REPO, "include")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-I" + INCLUDE, "-I" + CSRC]

LIB_SOURCES = ["kernels.cu", "strip.cu", "tile.cu", "engine.cu", "geometry.cpp", "noalloc.cu", "cnn.cu", "net.cu"]
# driver name -> -D selector of cli/tomo_cli.cpp
DRIVERS = {
    "generate-field": "GENERATE_FIELD",
    "generate-data": "GENERATE_DATA",
    "sirt-mimo": "SIRT_MIMO",
    "sirt-mimo-io": "SIRT_MIMO_IO",
    "sirt-mimo-norm": "SIRT_MIMO_NORM",
    "sirt-mimo-norm-mem": "SIRT_MIMO_NORM_MEM",
    "sirt-mimo-weight": "SIRT_MIMO_WEIGHT",
    "sirt-mimo-avg": "SIRT_MIMO_AVG",
    "sirt-mimo-avg-weight": "SIRT_MIMO_AVG_WEIGHT",
    "sirt-iter": "SIRT_ITER",
    "sirt-iter-norm": "SIRT_ITER_NORM",
    "art-mimo": "ART_MIMO",
    "art-mimo-io": "ART_MIMO_IO",
    "sirt-mimo-seq": "SIRT_MIMO_SEQ",
    "sirt-mimo-norm-alt": "SIRT_MIMO_NORM_ALT",
    "tomo": "TOMO_MULTI",
}
HEADERS = [os.path.join(INCLUDE, "tomo.h"), os.path.join(CSRC, "internal.h"), os.path.join(CSRC, "cell.cuh"),
           os.path.join(CSRC, "async.cuh"), os.path.join(CSRC, "cnn.h")]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _compile(src: str, obj: str) -> None:
    cmd = [NVCC, *ARCH, *COMMON, "-Xcompiler", "-fPIC", "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        # host arithmetic (the reference-profile source table) rounds every operation, as the
        # oracle does: no fused multiply-add contraction on either host architecture
        cmd.insert(1, "-x")
        cmd.insert(2, "c++")
        cmd += ["-Xcompiler", "-ffp-contract=off"]
    _run(cmd)


def build(force: bool = False, jobs: int | None = None, drivers: bool = True) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    jobs = jobs or min(8, os.cpu_count() or 4)
    objs = []
    todo = []
    for s in LIB_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s + ".o")
        objs.append(obj)
        if force or _newer(obj, [src, *HEADERS]):
            todo.append((src, obj))
    cli_src = os.path.join(CLI, "tomo_cli.cpp")
    cli_objs = {}
    if drivers:
        for name, sel in DRIVERS.items():
            obj = os.path.join(OBJ, f"cli_{name}.o")
            cli_objs[name] = obj
            if force or _newer(obj, [cli_src, os.path.join(CLI, "textio.h"), *HEADERS]):
                todo.append((cli_src, obj, sel))
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = []
        for t in todo:
            if len(t) == 2:
                futs.append(ex.submit(_compile, *t))
            else:
                src, obj, sel = t
                futs.append(ex.submit(_run, ["g++", "-O2", "-std=c++17", "-fPIC", f"-DTOMO_DRIVER_{sel}",
                                             "-I" + INCLUDE, "-I" + CLI, "-c", src, "-o", obj]))
        for f in futs:
            f.result()
    if force or _newer(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
        os.replace(tmp, LIB)
    if drivers:
        libdir = os.path.dirname(LIB)
        links = []
        for name, obj in cli_objs.items():
            exe = os.path.join(BIN, name)
            if force or _newer(exe, [obj, LIB]):
                links.append(["g++", "-o", exe, obj, "-L" + libdir, "-ltomo", "-Wl,-rpath,$ORIGIN/../lib"])
        with cf.ThreadPoolExecutor(jobs) as ex:
            for f in [ex.submit(_run, c) for c in links]:
                f.result()
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(LIB)
