"""C ABI checks that need no GPU.

libtomo.so builds, loads and exports every function declared in
include/tomo.h; host-side entry points (config defaults, phantoms, argument
validation) work without a device; with no device, tomo_create fails with a
status instead of crashing.  The CLI writes the reference's fo.txt format.
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import oracle_lib as O
import tomo

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "tomo.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tomo_[a-z_]+)\s*\(", text)))


def test_exports_every_declared_symbol(built_lib):
    names = declared_functions()
    assert len(names) >= 18
    out = subprocess.run(["nm", "-D", "--defined-only", tomo.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (tomo_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        getattr(built_lib, n)


def test_config_defaults(built_lib):
    c = tomo.Config()
    assert built_lib.tomo_config_init(C.byref(c), tomo.PROFILE_REF) == 0
    assert (c.nx, c.ny, c.nt, c.group_size, c.ring_lo, c.ring_hi) == (192, 192, 401, 10, 20, 180)
    assert built_lib.tomo_config_init(C.byref(c), tomo.PROFILE_CFG) == 0
    assert (c.nx, c.nt, c.n_transducers, c.group_size) == (128, 600, 32, 4)
    assert built_lib.tomo_config_init(C.byref(c), 7) == tomo.ERR_ARG
    assert built_lib.tomo_abi_version() == 1
    assert built_lib.tomo_status_string(tomo.ERR_OOM) == b"out of device memory"


def test_phantom_matches_oracle(built_lib):
    assert np.array_equal(tomo.phantom_ref(), O.phantom_ref())
    a = tomo.phantom_cfg(128, 128, 0, 3, 5, 15, 0.1, 0.0, 45.0, 1000)
    b = tomo.phantom_cfg(128, 128, 0, 3, 5, 15, 0.1, 0.0, 45.0, 1000)
    assert np.array_equal(a, b) and np.abs(a).max() <= 0.3 and (a != 0).sum() > 100
    e = tomo.phantom_cfg(256, 256, 1, 8, 10, 60, 0.15, 0.01, 110.0, 7)
    assert e.std() > 0.005


def test_host_allocation_failure_is_a_status(built_lib):
    # a 2^30 x 2^30 phantom needs a host buffer larger than the address space: the C++
    # exception below the entry point comes back as a status (nothing is written to fo)
    fo = np.zeros(4, np.float32)
    st = built_lib.tomo_phantom_cfg(1 << 30, 1 << 30, 1, 0, 10.0, 20.0, 0.1, 0.0, 50.0, 1,
                                    fo.ctypes.data_as(C.POINTER(C.c_float)))
    assert st == tomo.ERR_OOM
    assert not fo.any()


def test_null_handles_are_statuses(built_lib):
    """Every entry point answers a NULL context or network with TOMO_ERR_ARG (no device touched)."""
    L = built_lib
    sch = tomo.schedule(omega=1.0)
    st = tomo.IterStats()
    d = C.c_double()
    i = C.c_int32()
    calls = {
        "tomo_forward": (None, None, None, None),
        "tomo_generate_data": (None, None, None, None),
        "tomo_set_records": (None, None),
        "tomo_set_residual_noise": (None, None),
        "tomo_gradient": (None, None, None, None, None, None),
        "tomo_iterate": (None, 0, C.byref(sch), 0, None, None, None, C.byref(st)),
        "tomo_run": (None, 0, C.byref(sch), None, None, None, 0.0, 1, None, None),
        "tomo_forward_device": (None, None, None),
        "tomo_iterate_device": (None, 0, C.byref(sch), 0, None, None, None, C.byref(st)),
        "tomo_features_device": (None, None, None, None),
        "tomo_iterate_learned": (None, None, C.byref(sch), 0, None, None, C.byref(st), C.byref(i)),
        "tomo_run_learned": (None, None, C.byref(sch), None, None, 0.0, 1, 0.05, 2, None, None, None, None, None),
        "tomo_time_kernel": (None, 0, 1, C.byref(d), None),
        "tomo_iterate_batch": (None, 1, 0, C.byref(sch), 0, 1, None, None, None, None),
        "tomo_synchronize": (None,),
        "tomo_set_learned_scale": (None, 1.0),
        "tomo_set_learned_backtrack": (None, 1),
        "tomo_set_learned_resume": (None, 3),
        "tomo_gradient_groups_device": (None, None, 0, 1, None),
        "tomo_get_correlations_device": (None, 0, 1, None),
        "tomo_set_correlations_device": (None, 0, 1, None),
        "tomo_update_device": (None, 0, C.byref(sch), 0, None, None, C.byref(st)),
        "tomo_get_info": (None, None),
        "tomo_transducers": (None, None, None),
        "tomo_forward_noalloc": (None, None, None, None),
        "tomo_net_get_params": (None, None),
        "tomo_net_set_params": (None, None),
        "tomo_net_save": (None, b"x"),
        "tomo_net_load": (None, b"x"),
        "tomo_net_forward_device": (None, None, 1, 8, 64, None),
        "tomo_net_grad_device": (None, None, None, None, 1, 8, 64, None, None),
        "tomo_net_train_step_device": (None, None, None, None, 1, 8, 64, 1e-3, None),
    }
    for name, args in calls.items():
        assert getattr(L, name)(*args) == tomo.ERR_ARG, name
    assert L.tomo_stream(None) is None
    assert L.tomo_net_last_error(None) == b""
    L.tomo_destroy(None)
    L.tomo_net_destroy(None)


def test_net_create_without_gpu_is_a_status(built_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert built_lib.tomo_net_create(0, 1, C.byref(h)) == tomo.ERR_CUDA and not h.value


C_CLIENT = r"""
#include <stdio.h>
#include <stdlib.h>
#include "tomo.h"

int main(void) {
    tomo_config cfg;
    if (tomo_config_init(&cfg, TOMO_PROFILE_REF) != TOMO_OK || cfg.nx != 192) return 1;
    float* fo = (float*)calloc((size_t)cfg.nx * cfg.ny, sizeof(float));
    if (!fo || tomo_phantom_ref(cfg.nx, cfg.ny, fo) != TOMO_OK) return 2;
    int disc = 0;
    for (int q = 0; q < cfg.nx * cfg.ny; ++q) disc += fo[q] > 0.f;
    tomo_ctx* ctx = NULL;
    cfg.group_size = 0;                                  /* invalid: rejected before any device call */
    if (tomo_create(&cfg, &ctx) != TOMO_ERR_ARG || ctx != NULL) return 3;
    printf("%d %d %s|%s\n", tomo_abi_version(), disc, tomo_status_string(TOMO_ERR_ARG), tomo_last_error(NULL));
    free(fo);
    return 0;
}
"""


def test_header_is_c_and_links_from_c(built_lib, tmp_path):
    """include/tomo.h compiles as strict C99 and a C program links against libtomo.so and runs
    the host-side entry points."""
    src = tmp_path / "client.c"
    src.write_text(C_CLIENT)
    exe = tmp_path / "client"
    libdir = os.path.dirname(tomo.LIB_PATH)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I" + os.path.join(REPO, "include"),
                        str(src), "-o", str(exe), "-L" + libdir, "-ltomo", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    ver, disc, rest = out.stdout.strip().split(" ", 2)
    assert ver == "1" and int(disc) > 500
    assert rest.startswith("invalid argument|") and len(rest) > len("invalid argument|")


LAYOUT_CLIENT = r"""
#include <stddef.h>
#include <stdio.h>
#include "tomo.h"
#define F(s, m) printf(#s " " #m " %zu %zu\n", offsetof(s, m), sizeof(((s*)0)->m));
int main(void) {
    printf("tomo_config size %zu\n", sizeof(tomo_config));
    printf("tomo_schedule size %zu\n", sizeof(tomo_schedule));
    printf("tomo_iter_stats size %zu\n", sizeof(tomo_iter_stats));
    printf("tomo_info size %zu\n", sizeof(tomo_info));
    printf("tomo_noise size %zu\n", sizeof(tomo_noise));
    %FIELDS%
    return 0;
}
"""


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of the header's structs have the C compiler's field offsets and sizes."""
    structs = {"tomo_config": tomo.Config, "tomo_schedule": tomo.Schedule, "tomo_iter_stats": tomo.IterStats,
               "tomo_info": tomo.Info, "tomo_noise": tomo.Noise}
    fields = "\n    ".join(f"F({cn}, {name})" for cn, py in structs.items() for name, _ in py._fields_)
    src = tmp_path / "layout.c"
    src.write_text(LAYOUT_CLIENT.replace("%FIELDS%", fields))
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-I" + os.path.join(REPO, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60).stdout.split("\n")
    for line in filter(None, out):
        parts = line.split()
        py = structs[parts[0]]
        if parts[1] == "size":
            assert C.sizeof(py) == int(parts[2]), line
        else:
            d = getattr(py, parts[1])
            assert (d.offset, d.size) == (int(parts[2]), int(parts[3])), line


def test_bad_config_rejected_before_device(built_lib):
    for bad in (tomo.ref_config(ring_lo=1), tomo.ref_config(ring_hi=190), tomo.ref_config(group_size=0),
                tomo.cfg_config(radius=70.0), tomo.cfg_config(courant=0.9)):
        h = C.c_void_p()
        st = built_lib.tomo_create(C.byref(bad), C.byref(h))
        assert st == tomo.ERR_ARG and not h.value
        assert built_lib.tomo_last_error(None)


def test_create_without_gpu_is_a_status(built_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    st = built_lib.tomo_create(C.byref(tomo.ref_config()), C.byref(h))
    assert st == tomo.ERR_CUDA and not h.value


def test_cli_generate_field(built_lib, tmp_path):
    exe = os.path.join(os.path.dirname(tomo.LIB_PATH), "..", "bin", "generate-field")
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    vals = np.array(open(tmp_path / "fo.txt").read().split(), np.float32)
    assert np.array_equal(vals.reshape(192, 192), O.phantom_ref())
    lines = open(tmp_path / "fo.txt").read().split("\n")
    assert len(lines[0].split()) == 192 and lines[192] == ""


@pytest.mark.parametrize("driver", ["sirt-mimo-norm", "sirt-mimo-seq", "sirt-mimo-norm-alt"])
def test_cli_usage_errors(built_lib, tmp_path, driver):
    exe = os.path.join(os.path.dirname(tomo.LIB_PATH), "..", "bin", driver)
    r = subprocess.run([exe, "fo.txt"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "Usage" in r.stderr


def read_bin(path):
    raw = open(path, "rb").read()
    assert raw[:8] == b"TOMOF32\n"
    dims = np.frombuffer(raw[8:24], "<i4")
    return dims, np.frombuffer(raw[24:], "<f4")


def test_cli_generate_field_binary(built_lib, tmp_path):
    """The binary form (magic, four int32 dims, float32 values) holds the same phantom."""
    exe = os.path.join(os.path.dirname(tomo.LIB_PATH), "..", "bin", "generate-field")
    r = subprocess.run([exe, "--binary"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    dims, vals = read_bin(tmp_path / "fo.bin")
    assert list(dims) == [192, 192, 1, 1]
    assert np.array_equal(vals.reshape(192, 192), O.phantom_ref())


def test_net_parameter_count_matches_oracle_layout(built_lib):
    """The network's flat parameter vector has the oracle's layout size (first layer stored with
    its 3 feature channels zero-padded to 16), so weights move between the two unchanged."""
    import cnn_oracle as K

    assert tomo.lib().tomo_net_num_params() == K.N_PARAMS == sum(int(np.prod(s)) for _, s in K.SHAPES)
