"""Python binding of libtomo.so, the C ABI declared in include/tomo.h.

This module is a thin ctypes layer used by the tests, the benchmark and
notebook users.  All compute runs in libtomo.so's CUDA kernels; nothing here
computes a wavefield.  Importing the module does not load the library; the
first call to :func:`lib` does, and raises if the CUDA library is missing
(there is no CPU fallback).

Array conventions follow include/tomo.h: FP32, i (x) fastest, records laid out
as ``rec[g, k, c]`` (groups, time steps, channels).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_DIR = os.path.dirname(PKG_DIR)
LIB_PATH = os.path.join(PKG_DIR, "lib", "libtomo.so")

# tomo_status
OK, ERR_ARG, ERR_CUDA, ERR_OOM, ERR_TIMEOUT, ERR_DIVERGED, ERR_IO, ERR_STATE = range(8)
# tomo_profile
PROFILE_REF, PROFILE_CFG = 0, 1
# tomo_method
SIRT_CLASSIC, SIRT_SCALED, SIRT_NORM, SIRT_WEIGHT, SIRT_AVG, SIRT_AVG_WEIGHT, ART = range(7)
METHOD_NAMES = {
    SIRT_CLASSIC: "sirt-classic", SIRT_SCALED: "sirt-scaled", SIRT_NORM: "sirt-norm",
    SIRT_WEIGHT: "sirt-weight", SIRT_AVG: "sirt-avg", SIRT_AVG_WEIGHT: "sirt-avg-weight",
    ART: "art",
}
# tomo_sched_kind
SCHED_CONST, SCHED_POWER, SCHED_LINEAR = range(3)
# acceptance rule of the learned step (tomo_run_learned): a proposal must lower the squared
# record residual by 5 %; after 2 rejections in a row the run continues with plain steps
LEARNED_MIN_DECREASE, LEARNED_PATIENCE = 0.05, 2
# scale of the learned proposal f + LEARNED_SCALE * mask * net(features) (tomo_set_learned_scale)
LEARNED_SCALE = 1.0


class Config(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nt", C.c_int32),
        ("profile", C.c_int32), ("group_size", C.c_int32),
        ("ring_lo", C.c_int32), ("ring_hi", C.c_int32),
        ("n_transducers", C.c_int32), ("radius", C.c_float), ("courant", C.c_float),
        ("cells_per_wavelength", C.c_float), ("sponge_width", C.c_int32),
        ("sponge_max", C.c_float),
        ("ckpt_interval", C.c_int32), ("groups_per_pass", C.c_int32), ("device", C.c_int32),
        ("mem_limit_mb", C.c_int32), ("reserved", C.c_int32 * 3),
    ]


class Schedule(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("omega", C.c_float), ("alpha", C.c_float),
        ("beta", C.c_float), ("gamma", C.c_float), ("normalize", C.c_int32),
        ("reserved", C.c_int32 * 2),
    ]


class IterStats(C.Structure):
    _fields_ = [
        ("epsilon", C.c_double), ("resid_norm2", C.c_double), ("scale", C.c_double),
        ("seconds", C.c_double), ("cell_updates", C.c_double), ("kernel_launches", C.c_double),
    ]


class Info(C.Structure):
    _fields_ = [
        ("n_groups", C.c_int32), ("n_channels", C.c_int32), ("n_transducers", C.c_int32),
        ("groups_per_pass", C.c_int32), ("ckpt_interval", C.c_int32),
        ("n_segments", C.c_int32), ("device_bytes", C.c_int64),
    ]


class Noise(C.Structure):
    _fields_ = [("kind", C.c_int32), ("level", C.c_float), ("seed", C.c_uint64)]


def ref_config(nx=192, ny=192, nt=401, group_size=10, ring_lo=20, ring_hi=180, **kw) -> Config:
    """The reference problem (sirt-mimo.cu:17-35), optionally resized."""
    c = Config(nx=nx, ny=ny, nt=nt, profile=PROFILE_REF, group_size=group_size,
               ring_lo=ring_lo, ring_hi=ring_hi)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def cfg_config(nx=128, ny=128, nt=600, n_transducers=32, group_size=4, radius=50.0,
               courant=0.5, cells_per_wavelength=12.0, sponge_width=16, sponge_max=0.05,
               **kw) -> Config:
    """A synthetic-workload problem (defaults: the 128^2 / 32-transducer case)."""
    c = Config(nx=nx, ny=ny, nt=nt, profile=PROFILE_CFG, group_size=group_size,
               n_transducers=n_transducers, radius=radius, courant=courant,
               cells_per_wavelength=cells_per_wavelength, sponge_width=sponge_width,
               sponge_max=sponge_max)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def schedule(kind=SCHED_CONST, omega=1.0, alpha=0.0, beta=0.0, gamma=1.0, normalize=0) -> Schedule:
    return Schedule(kind=kind, omega=omega, alpha=alpha, beta=beta, gamma=gamma, normalize=normalize)


def n_groups(cfg: Config) -> int:
    ns = 4 * (cfg.ring_hi - cfg.ring_lo) if cfg.profile == PROFILE_REF else cfg.n_transducers
    return ns // cfg.group_size


def n_channels(cfg: Config) -> int:
    return 4 * cfg.nx if cfg.profile == PROFILE_REF else cfg.n_transducers


_LIB = None


def _fp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int32))


def lib(path: str | None = None) -> C.CDLL:
    """Load libtomo.so (built in-tree by the package build)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libtomo.so not built at {p}; run __graft_entry__.build()")
    L = C.CDLL(p)
    vp, i32, f32, u64 = C.c_void_p, C.c_int32, C.c_float, C.c_uint64
    FP, DP, IP = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int32)
    sig = {
        "tomo_abi_version": (i32, []),
        "tomo_status_string": (C.c_char_p, [i32]),
        "tomo_config_init": (i32, [C.POINTER(Config), i32]),
        "tomo_create": (i32, [C.POINTER(Config), C.POINTER(vp)]),
        "tomo_destroy": (None, [vp]),
        "tomo_last_error": (C.c_char_p, [vp]),
        "tomo_get_info": (i32, [vp, C.POINTER(Info)]),
        "tomo_stream": (vp, [vp]),
        "tomo_transducers": (i32, [vp, IP, IP]),
        "tomo_phantom_ref": (i32, [i32, i32, FP]),
        "tomo_phantom_cfg": (i32, [i32, i32, i32, i32, f32, f32, f32, f32, f32, u64, FP]),
        "tomo_forward": (i32, [vp, FP, FP, FP]),
        "tomo_generate_data": (i32, [vp, FP, FP, C.POINTER(Noise)]),
        "tomo_set_records": (i32, [vp, FP]),
        "tomo_set_residual_noise": (i32, [vp, C.POINTER(Noise)]),
        "tomo_gradient": (i32, [vp, FP, FP, FP, FP, DP]),
        "tomo_iterate": (i32, [vp, i32, C.POINTER(Schedule), i32, FP, FP, FP, C.POINTER(IterStats)]),
        "tomo_run": (i32, [vp, i32, C.POINTER(Schedule), FP, FP, FP, f32, i32, DP, IP]),
        "tomo_forward_device": (i32, [vp, vp, vp]),
        "tomo_iterate_device": (i32, [vp, i32, C.POINTER(Schedule), i32, vp, vp, vp, C.POINTER(IterStats)]),
        "tomo_synchronize": (i32, [vp]),
        "tomo_gradient_groups_device": (i32, [vp, vp, i32, i32, DP]),
        "tomo_get_correlations_device": (i32, [vp, i32, i32, vp]),
        "tomo_set_correlations_device": (i32, [vp, i32, i32, vp]),
        "tomo_update_device": (i32, [vp, i32, C.POINTER(Schedule), i32, vp, vp, C.POINTER(IterStats)]),
        "tomo_time_kernel": (i32, [vp, i32, i32, DP, DP]),
        "tomo_forward_noalloc": (i32, [C.POINTER(Config), vp, vp, vp]),
        "tomo_net_num_params": (C.c_int64, []),
        "tomo_net_create": (i32, [i32, u64, C.POINTER(vp)]),
        "tomo_net_destroy": (None, [vp]),
        "tomo_net_last_error": (C.c_char_p, [vp]),
        "tomo_net_get_params": (i32, [vp, FP]),
        "tomo_net_set_params": (i32, [vp, FP]),
        "tomo_net_save": (i32, [vp, C.c_char_p]),
        "tomo_net_load": (i32, [vp, C.c_char_p]),
        "tomo_net_forward_device": (i32, [vp, vp, i32, i32, i32, vp]),
        "tomo_net_grad_device": (i32, [vp, vp, vp, vp, i32, i32, i32, FP, DP]),
        "tomo_net_train_step_device": (i32, [vp, vp, vp, vp, i32, i32, i32, f32, DP]),
        "tomo_features_device": (i32, [vp, vp, vp, DP]),
        "tomo_set_learned_scale": (i32, [vp, C.c_double]),
        "tomo_set_learned_backtrack": (i32, [vp, i32]),
        "tomo_set_learned_resume": (i32, [vp, i32]),
        "tomo_iterate_learned": (i32, [vp, vp, C.POINTER(Schedule), i32, vp, vp, C.POINTER(IterStats), IP]),
        "tomo_run_learned": (i32, [vp, vp, C.POINTER(Schedule), vp, vp, C.c_double, i32, C.c_double, i32, DP, IP,
                                   IP, IP, C.POINTER(C.c_double)]),
        "tomo_iterate_batch": (i32, [C.POINTER(vp), i32, i32, C.POINTER(Schedule), i32, i32, C.POINTER(vp),
                                     C.POINTER(vp), DP, C.POINTER(C.c_double)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


class TomoError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"tomo status {status}: {msg}")
        self.status = status


def phantom_ref(nx=192, ny=192) -> np.ndarray:
    fo = np.zeros((ny, nx), np.float32)
    st = lib().tomo_phantom_ref(nx, ny, _fp(fo))
    if st:
        raise TomoError(st, "tomo_phantom_ref")
    return fo


def phantom_cfg(nx, ny, kind, n, rmin, rmax, vmax, noise_sigma, support, seed) -> np.ndarray:
    fo = np.zeros((ny, nx), np.float32)
    st = lib().tomo_phantom_cfg(nx, ny, kind, n, rmin, rmax, vmax, noise_sigma, support, seed, _fp(fo))
    if st:
        raise TomoError(st, "tomo_phantom_cfg")
    return fo


class Context:
    """Owns a tomo_ctx (device buffers and one CUDA stream)."""

    def __init__(self, cfg: Config):
        self.cfg = cfg
        h = C.c_void_p()
        st = lib().tomo_create(C.byref(cfg), C.byref(h))
        if st:
            raise TomoError(st, "tomo_create: " + (lib().tomo_last_error(None) or b"").decode())
        self.h = h
        info = Info()
        self._check(lib().tomo_get_info(self.h, C.byref(info)))
        self.info = info
        self.G = info.n_groups
        self.nch = info.n_channels

    def _check(self, st):
        if st:
            raise TomoError(st, (lib().tomo_last_error(self.h) or b"").decode())

    def close(self):
        if getattr(self, "h", None):
            lib().tomo_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def shape(self):
        return (self.cfg.ny, self.cfg.nx)

    def records_shape(self):
        return (self.G, self.cfg.nt, self.nch)

    def transducers(self):
        n = self.info.n_transducers
        ii = np.zeros(n, np.int32)
        jj = np.zeros(n, np.int32)
        self._check(lib().tomo_transducers(self.h, _ip(ii), _ip(jj)))
        return ii, jj

    def forward(self, f, u_last=False):
        f = np.ascontiguousarray(f, np.float32)
        rec = np.zeros(self.records_shape(), np.float32)
        ul = np.zeros((self.G,) + self.shape, np.float32) if u_last else None
        self._check(lib().tomo_forward(self.h, _fp(f), _fp(rec), _fp(ul)))
        return (rec, ul) if u_last else rec

    def generate_data(self, f_true, noise_level=0.0, seed=0, kind=1):
        """Forward records plus seeded noise (kind 1 additive Gaussian, 2/3 multiplicative uniform)."""
        f = np.ascontiguousarray(f_true, np.float32)
        rec = np.zeros(self.records_shape(), np.float32)
        nz = Noise(kind=kind if noise_level > 0 else 0, level=noise_level, seed=seed)
        self._check(lib().tomo_generate_data(self.h, _fp(f), _fp(rec), C.byref(nz)))
        return rec

    def set_residual_noise(self, kind=0, level=0.0, seed=0):
        """In-loop multiplicative record noise (kind 2 fresh per sweep, 3 fixed; 0 off)."""
        nz = Noise(kind=kind, level=level, seed=seed)
        self._check(lib().tomo_set_residual_noise(self.h, C.byref(nz)))

    def set_records(self, rec):
        rec = np.ascontiguousarray(rec, np.float32)
        self._check(lib().tomo_set_records(self.h, _fp(rec)))

    def gradient(self, f, rec, per_group=True):
        f = np.ascontiguousarray(f, np.float32)
        rec = np.ascontiguousarray(rec, np.float32)
        dfg = np.zeros((self.G,) + self.shape, np.float32) if per_group else None
        df = np.zeros(self.shape, np.float32)
        r2 = C.c_double()
        self._check(lib().tomo_gradient(self.h, _fp(f), _fp(rec), _fp(dfg), _fp(df), C.byref(r2)))
        return dfg, df, r2.value

    def iterate(self, method, sched: Schedule, it, f, rec=None, f_true=None):
        """One iteration in place on f (float32 array); returns IterStats."""
        assert f.dtype == np.float32 and f.flags.c_contiguous
        rp = None if rec is None else _fp(np.ascontiguousarray(rec, np.float32))
        ft = None if f_true is None else np.ascontiguousarray(f_true, np.float32)
        stats = IterStats()
        self._check(lib().tomo_iterate(self.h, method, C.byref(sched), it, _fp(f), rp, _fp(ft),
                                       C.byref(stats)))
        return stats

    def run(self, method, sched, f, rec, f_true, target_eps, max_iters):
        assert f.dtype == np.float32 and f.flags.c_contiguous
        log = np.zeros(max(max_iters, 1), np.float64)
        done = C.c_int32()
        st = lib().tomo_run(self.h, method, C.byref(sched), _fp(f),
                            _fp(np.ascontiguousarray(rec, np.float32)),
                            _fp(np.ascontiguousarray(f_true, np.float32)),
                            target_eps, max_iters, _dp(log), C.byref(done))
        if st not in (OK, ERR_DIVERGED):
            self._check(st)
        return log[: done.value], st

    def forward_device(self, d_f: int, d_rec: int):
        self._check(lib().tomo_forward_device(self.h, C.c_void_p(d_f), C.c_void_p(d_rec)))

    def iterate_device(self, method, sched, it, d_f: int, d_rec: int = 0, d_ftrue: int = 0):
        stats = IterStats()
        self._check(lib().tomo_iterate_device(self.h, method, C.byref(sched), it, C.c_void_p(d_f),
                                              C.c_void_p(d_rec or None), C.c_void_p(d_ftrue or None),
                                              C.byref(stats)))
        return stats

    def gradient_groups_device(self, d_f: int, g0: int, ng: int) -> float:
        """Gradient sweeps of groups g0 .. g0+ng-1 for the device field d_f; their correlations stay
        in the context.  Returns their squared record residual."""
        r2 = C.c_double()
        self._check(lib().tomo_gradient_groups_device(self.h, C.c_void_p(d_f), g0, ng, C.byref(r2)))
        return r2.value

    def get_correlations_device(self, g0: int, ng: int, d_out: int):
        self._check(lib().tomo_get_correlations_device(self.h, g0, ng, C.c_void_p(d_out)))

    def set_correlations_device(self, g0: int, ng: int, d_in: int):
        self._check(lib().tomo_set_correlations_device(self.h, g0, ng, C.c_void_p(d_in)))

    def update_device(self, method, sched, it, d_f: int, d_ftrue: int = 0):
        """The update rule of a SIRT method from the correlations held for all groups."""
        stats = IterStats()
        self._check(lib().tomo_update_device(self.h, method, C.byref(sched), it, C.c_void_p(d_f),
                                             C.c_void_p(d_ftrue or None), C.byref(stats)))
        return stats

    def time_kernel(self, which: int, steps: int):
        """(ms per launch, algorithmic bytes per launch) of the forward (0) or adjoint (1) step."""
        ms, by = C.c_double(), C.c_double()
        self._check(lib().tomo_time_kernel(self.h, which, steps, C.byref(ms), C.byref(by)))
        return ms.value, by.value

    def synchronize(self):
        self._check(lib().tomo_synchronize(self.h))

    def features_device(self, d_f: int, d_feat: int) -> float:
        """Writes the network features of the device field d_f into d_feat (3*ny*nx floats)."""
        r2 = C.c_double()
        self._check(lib().tomo_features_device(self.h, C.c_void_p(d_f), C.c_void_p(d_feat), C.byref(r2)))
        return r2.value

    def iterate_learned(self, net: "Net", fallback: Schedule, it: int, d_f: int, d_ftrue: int = 0):
        """One residual-checked learned iteration on the device field d_f; (stats, accepted)."""
        stats = IterStats()
        acc = C.c_int32()
        self._check(lib().tomo_iterate_learned(self.h, net.h, C.byref(fallback), it, C.c_void_p(d_f),
                                               C.c_void_p(d_ftrue or None), C.byref(stats), C.byref(acc)))
        return stats, bool(acc.value)

    def run_learned(self, net: "Net", fallback: Schedule, d_f: int, d_ftrue: int = 0,
                    target_eps: float = -1.0, max_iters: int = 50, min_decrease: float = LEARNED_MIN_DECREASE,
                    patience: int = LEARNED_PATIENCE):
        """Learned iterations on d_f until epsilon <= target_eps or max_iters:
        (epsilon per iteration, step kind per iteration [1 learned, 0 rejected, -1 plain],
        gradient sweeps, wall seconds)."""
        eps = np.full(max(max_iters, 1), np.nan)
        kind = np.zeros(max(max_iters, 1), np.int32)
        done, sweeps, secs = C.c_int32(), C.c_int32(), C.c_double()
        self._check(lib().tomo_run_learned(self.h, net.h, C.byref(fallback), C.c_void_p(d_f),
                                           C.c_void_p(d_ftrue or None), target_eps, max_iters, min_decrease,
                                           patience, _dp(eps), _ip(kind), C.byref(done), C.byref(sweeps),
                                           C.byref(secs)))
        n = done.value
        return eps[:n], kind[:n], sweeps.value, secs.value

    def set_learned_scale(self, scale: float):
        """Scale of the learned proposal f + scale * mask * net(features)."""
        self._check(lib().tomo_set_learned_scale(self.h, scale))

    def set_learned_backtrack(self, retries: int):
        """Retries of a rejected learned proposal at half the previous scale (run_learned)."""
        self._check(lib().tomo_set_learned_backtrack(self.h, int(retries)))

    def set_learned_resume(self, plain_steps: int):
        """Plain steps after which a paused learned run proposes again (0: never)."""
        self._check(lib().tomo_set_learned_resume(self.h, int(plain_steps)))

    @property
    def stream(self) -> int:
        return lib().tomo_stream(self.h) or 0


def iterate_batch(ctxs, method, sched: Schedule, iter0: int, iters: int, d_fs, d_ftrues=None):
    """Advance several contexts together (one host thread each, kernels overlapping on the GPU):
    (epsilon [n, iters] or NaN without d_ftrues, wall seconds)."""
    n = len(ctxs)
    hs = (C.c_void_p * n)(*[c.h for c in ctxs])
    fs = (C.c_void_p * n)(*d_fs)
    ts = (C.c_void_p * n)(*d_ftrues) if d_ftrues is not None else None
    eps = np.full((n, max(iters, 1)), np.nan)
    secs = C.c_double()
    st = lib().tomo_iterate_batch(hs, n, method, C.byref(sched), iter0, iters, fs, ts, _dp(eps), C.byref(secs))
    if st != OK:
        msgs = [lib().tomo_last_error(c.h) for c in ctxs]
        raise TomoError(st, "; ".join(m.decode() for m in msgs if m))
    return eps[:, :iters], secs.value


class Net:
    """The learned update network (tomo_net): 5 layers of 3x3 convolutions."""

    def __init__(self, device: int = 0, seed: int = 0):
        h = C.c_void_p()
        st = lib().tomo_net_create(device, seed, C.byref(h))
        if st:
            raise TomoError(st, "tomo_net_create")
        self.h = h
        self.n_params = int(lib().tomo_net_num_params())

    def _check(self, st):
        if st:
            raise TomoError(st, (lib().tomo_net_last_error(self.h) or b"").decode())

    def close(self):
        if getattr(self, "h", None):
            lib().tomo_net_destroy(self.h)
            self.h = None

    __del__ = close

    def params(self) -> np.ndarray:
        p = np.zeros(self.n_params, np.float32)
        self._check(lib().tomo_net_get_params(self.h, _fp(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        self._check(lib().tomo_net_set_params(self.h, _fp(p)))

    def save(self, path: str):
        self._check(lib().tomo_net_save(self.h, path.encode()))

    def load(self, path: str):
        self._check(lib().tomo_net_load(self.h, path.encode()))

    def forward_device(self, d_feat: int, B: int, H: int, W: int, d_out: int):
        self._check(lib().tomo_net_forward_device(self.h, C.c_void_p(d_feat), B, H, W, C.c_void_p(d_out)))

    def grad_device(self, d_feat: int, d_tgt: int, d_mask: int, B: int, H: int, W: int):
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_double()
        self._check(lib().tomo_net_grad_device(self.h, C.c_void_p(d_feat), C.c_void_p(d_tgt), C.c_void_p(d_mask),
                                               B, H, W, _fp(g), C.byref(loss)))
        return g, loss.value

    def train_step_device(self, d_feat: int, d_tgt: int, d_mask: int, B: int, H: int, W: int, lr: float) -> float:
        loss = C.c_double()
        self._check(lib().tomo_net_train_step_device(self.h, C.c_void_p(d_feat), C.c_void_p(d_tgt),
                                                     C.c_void_p(d_mask), B, H, W, lr, C.byref(loss)))
        return loss.value
