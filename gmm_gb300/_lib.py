"""ctypes binding of the C ABI in include/gmm_gb300.h.

The shared library is built in-tree by ``gmm_gb300.build`` (``gmm_gb300/_build``). If it is
missing, importing this module raises: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgmm_gb300.so")

OK, ERR_ARG, ERR_CUDA, ERR_STATE, ERR_MODEL, ERR_NOMEM, ERR_UNSUPPORTED, ERR_MLLR, ERR_TIMEOUT = range(9)
PREC_FP32, PREC_TC = 0, 1
ACC_MEAN, ACC_VAR, ACC_PROBS_ONLY = 1, 2, 4

# Every symbol the header declares, with (restype, argtypes).
_vp, _i, _ll, _f, _d, _sz = C.c_void_p, C.c_int, C.c_longlong, C.c_float, C.c_double, C.c_size_t
SIGNATURES = {
    "gmm_create": (_i, [_i, C.POINTER(_vp)]),
    "gmm_destroy": (_i, [_vp]),
    "gmm_last_error": (C.c_char_p, [_vp]),
    "gmm_set_options": (_i, [_vp, _f, _f, _f]),
    "gmm_set_precision": (_i, [_vp, _i]),
    "gmm_set_memory_budget": (_i, [_vp, _sz]),
    "gmm_get_stream": (_i, [_vp, C.POINTER(_vp)]),
    "gmm_upload_model": (_i, [_vp, _i, _i, _vp, _vp, _vp]),
    "gmm_upload_model_full": (_i, [_vp, _i, _i, _vp, _vp, _vp]),
    "gmm_fmllr_estimate": (_i, [_vp, _i, _vp]),
    "gmm_set_robust": (_i, [_vp, _i]),
    "gmm_accumulate_host": (_i, [_vp, _i, _vp, _ll, _i]),
    "gmm_mllr_estimate_full": (_i, [_vp, _i, _vp]),
    "gmm_mllr_apply_full": (_i, [_vp, _vp]),
    "gmm_read_aux": (_i, [_vp, _i, _vp, _vp, _vp]),
    "gmm_fmllr_apply": (_i, [_vp, _vp]),
    "gmm_fmllr_estimate_full": (_i, [_vp, _i, _vp]),
    "gmm_set_prior_full": (_i, [_vp, _vp, _vp, _vp]),
    "gmm_read_model_full": (_i, [_vp, _vp, _vp, _vp]),
    "gmm_accumulate_full": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp]),
    "gmm_accumulate_full_device": (_i, [_vp, _i]),
    "gmm_read_stats_full": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "gmm_loglikes_full": (_i, [_vp, _vp]),
    "gmm_em_update_full": (_i, [_vp, _i, _i, _i, _vp]),
    "gmm_map_update_full": (_i, [_vp, _i, _i, _i, _i]),
    "gmm_set_prior": (_i, [_vp, _vp, _vp, _vp]),
    "gmm_read_model": (_i, [_vp, _vp, _vp, _vp]),
    "gmm_upload_features": (_i, [_vp, _vp, _ll, _i]),
    "gmm_upload_features_device": (_i, [_vp, _vp, _ll, _i]),
    "gmm_accumulate": (_i, [_vp, _i, _vp, _vp, _vp, C.POINTER(_d), C.POINTER(_ll)]),
    "gmm_accumulate_device": (_i, [_vp, _i]),
    "gmm_read_stats": (_i, [_vp, _vp, _vp, _vp, C.POINTER(_d), C.POINTER(_ll)]),
    "gmm_loglikes": (_i, [_vp, _vp]),
    "gmm_em_update": (_i, [_vp, _i, _i, _i, C.POINTER(_i)]),
    "gmm_map_update": (_i, [_vp, _i, _i, _i, _i]),
    "gmm_em_iterate": (_i, [_vp, _i, _i, _i, _i, _vp, C.POINTER(_i)]),
    "gmm_map_batch": (_i, [_vp, _i, _vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp]),
    "gmm_map_batch_device": (_i, [_vp, _i, _vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp]),
    "gmm_mllr_batch": (_i, [_vp, _i, _vp, _i, _vp, _vp, _vp, _vp]),
    "gmm_map_batch_host": (_i, [_vp, _vp, C.c_longlong, _i, _i, _vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp]),
    "gmm_mllr_batch_host": (_i, [_vp, _vp, C.c_longlong, _i, _i, _vp, _i, _vp, _vp, _vp, _vp]),
    "gmm_mllr_estimate": (_i, [_vp, _i, _vp]),
    "gmm_mllr_apply": (_i, [_vp, _vp]),
    "gmm_profile_enable": (_i, [_vp, _i]),
    "gmm_profile_reset": (_i, [_vp]),
    "gmm_profile_read": (_i, [_vp, _i, C.POINTER(C.c_char_p), _vp, _vp]),
    "gmm_launch_count": (_ll, [_vp]),
    "gmm_accumulate_noalloc": (_i, [_vp, _ll, _i, _i, _vp, _vp, _vp, _f, _f, _f, _i, _vp, _vp]),
    "gmm_set_autotune": (_i, [_vp, _i]),
    "gmm_set_wait_limit": (_i, [_vp, _ll]),
    "gmm_set_tile_schedule": (_i, [_vp, _i]),
    "gmm_upload_model_slot": (_i, [_vp, _i, _i, _i, _vp, _vp, _vp]),
    "gmm_select_model": (_i, [_vp, _i]),
    "gmm_clear_model_slots": (_i, [_vp]),
    "gmm_autotune_choice": (_i, [_vp, C.POINTER(_i), _vp, _vp, _i]),
    "gmm_read_param": (_i, [C.c_char_p, _i, C.c_uint, _vp, _ll, C.POINTER(_ll), C.POINTER(_i)]),
    "gmm_accumulate_files": (_i, [_vp, _i, _i, C.POINTER(C.c_char_p), _i, C.c_uint, _d, C.POINTER(_i)]),
    "gmm_server_create": (_i, [_i, _i, _i, _i, _sz, C.POINTER(_vp)]),
    "gmm_server_destroy": (_i, [_vp]),
    "gmm_server_last_error": (C.c_char_p, [_vp]),
    "gmm_server_set_options": (_i, [_vp, _f, _f, _f, _i]),
    "gmm_server_add_model": (_i, [_vp, _vp, _vp, _vp, C.POINTER(_i)]),
    "gmm_server_submit": (_i, [_vp, _i, _i, _vp, _ll, _i, _i, _i, _i, _i, C.POINTER(_ll)]),
    "gmm_server_poll": (_i, [_vp, _ll, C.POINTER(_i)]),
    "gmm_server_wait": (_i, [_vp, _ll, _i]),
    "gmm_server_result": (_i, [_vp, _ll, C.POINTER(_d), _vp, _vp, _vp, _vp, C.POINTER(_d)]),
    "gmm_server_stats": (_i, [_vp, C.POINTER(_ll), C.POINTER(_ll), C.POINTER(_ll), C.POINTER(_sz)]),
}

PRM_SVES, PRM_HTK, PRM_RAW = 0, 1, 2
REQ_SCORE, REQ_MAP = 0, 1
REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3
SUBMIT_FRAME_LL, SUBMIT_NO_COPY = 1, 2

_lib = None


def load():
    """Load the library (once). Raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"gmm_gb300 CUDA library not found at {LIB_PATH}; build it with "
                "`python -m gmm_gb300.build` (there is no CPU fallback)")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class GMMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[gmm status {code}] {msg}")
        self.code = code


def ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


class Handle:
    """One engine handle (one stream on one device)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.gmm_create(device, C.byref(h))
        if rc:
            raise GMMError(rc, self.lib.gmm_last_error(None).decode())
        self.h = h
        self.M = self.D = 0
        self.N = 0

    def check(self, rc):
        if rc:
            raise GMMError(rc, self.lib.gmm_last_error(self.h).decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.lib.gmm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- configuration
    def set_options(self, min_loglike=-1e20, min_gamma=1e-4, min_var=1e-6):
        self.check(self.lib.gmm_set_options(self.h, min_loglike, min_gamma, min_var))

    def set_precision(self, mode):
        self.check(self.lib.gmm_set_precision(self.h, mode))

    def set_memory_budget(self, nbytes):
        self.check(self.lib.gmm_set_memory_budget(self.h, nbytes))

    def set_autotune(self, on: bool):
        self.check(self.lib.gmm_set_autotune(self.h, int(on)))

    def set_tile_schedule(self, mode):
        """Sparse tile schedule of the tensor-core statistics: 0 off (default), 1 on for large
        E-steps (>= 2048 frame tiles), 2 on always; True means 2, False 0."""
        self.check(self.lib.gmm_set_tile_schedule(self.h, 2 if mode is True else 0 if mode is False else int(mode)))

    def set_wait_limit(self, cycles: int):
        """Test hook: clock cycles a tensor-core pipeline wait may take (<= 0: the default)."""
        self.check(self.lib.gmm_set_wait_limit(self.h, int(cycles)))

    def autotune_choices(self) -> dict:
        n = C.c_int()
        self.check(self.lib.gmm_autotune_choice(self.h, C.byref(n), None, None, 0))
        keys = np.zeros(max(1, n.value), np.int64)
        waves = np.zeros(max(1, n.value), np.int32)
        self.check(self.lib.gmm_autotune_choice(self.h, C.byref(n), ptr(keys), ptr(waves), n.value))
        return {int(k): int(w) for k, w in zip(keys[:n.value], waves[:n.value])}

    def stream(self) -> int:
        s = C.c_void_p()
        self.check(self.lib.gmm_get_stream(self.h, C.byref(s)))
        return s.value or 0

    # -- model / features
    def upload_model(self, w, mu, var):
        w = np.ascontiguousarray(w, np.float32)
        mu = np.ascontiguousarray(mu, np.float32)
        var = np.ascontiguousarray(var, np.float32)
        M, D = mu.shape
        self.check(self.lib.gmm_upload_model(self.h, M, D, ptr(w), ptr(mu), ptr(var)))
        self.M, self.D = M, D

    def upload_model_slot(self, slot, w, mu, var):
        """Stores a model in a device-resident slot of the handle's group (the model in use is
        unchanged)."""
        w = np.ascontiguousarray(w, np.float32)
        mu = np.ascontiguousarray(mu, np.float32)
        var = np.ascontiguousarray(var, np.float32)
        M, D = mu.shape
        self.check(self.lib.gmm_upload_model_slot(self.h, int(slot), M, D, ptr(w), ptr(mu), ptr(var)))
        if not hasattr(self, "_slot_shapes"):
            self._slot_shapes = {}
        self._slot_shapes[int(slot)] = (M, D)

    def select_model(self, slot):
        """Makes the model of `slot` the resident model (device-to-device)."""
        self.check(self.lib.gmm_select_model(self.h, int(slot)))
        self.M, self.D = self._slot_shapes[int(slot)]

    def clear_model_slots(self):
        self.check(self.lib.gmm_clear_model_slots(self.h))
        self._slot_shapes = {}

    def set_prior(self, w=None, mu=None, var=None):
        if w is None:
            self.check(self.lib.gmm_set_prior(self.h, None, None, None))
            return
        w = np.ascontiguousarray(w, np.float32)
        mu = np.ascontiguousarray(mu, np.float32)
        var = np.ascontiguousarray(var, np.float32)
        self.check(self.lib.gmm_set_prior(self.h, ptr(w), ptr(mu), ptr(var)))

    def read_model(self):
        w = np.zeros(self.M, np.float32)
        mu = np.zeros((self.M, self.D), np.float32)
        var = np.zeros((self.M, self.D), np.float32)
        self.check(self.lib.gmm_read_model(self.h, ptr(w), ptr(mu), ptr(var)))
        return w, mu, var

    def upload_features(self, X):
        X = np.ascontiguousarray(X, np.float32)
        N, D = X.shape
        self.check(self.lib.gmm_upload_features(self.h, ptr(X), N, D))
        self.N, self.D = N, D

    def upload_features_device(self, dptr: int, N: int, D: int):
        self.check(self.lib.gmm_upload_features_device(self.h, dptr, N, D))
        self.N, self.D = N, D

    def accumulate_files(self, paths, prm_type, dwnsmp=1, buffer_gb=1.0, flags=ACC_MEAN | ACC_VAR):
        """File-by-file accumulation; returns the number of files that contributed frames. The
        statistics stay on the device (read_stats / the M-step entry points)."""
        arr = (C.c_char_p * max(1, len(paths)))(*[p.encode() for p in paths])
        used = C.c_int()
        self.check(self.lib.gmm_accumulate_files(self.h, flags, len(paths), arr, prm_type, dwnsmp,
                                                 buffer_gb, C.byref(used)))
        return used.value

    # -- E-step
    def accumulate(self, flags=ACC_MEAN | ACC_VAR):
        n = np.zeros(self.M)
        F = np.zeros((self.M, self.D))
        S = np.zeros((self.M, self.D))
        tl, tn = C.c_double(), C.c_longlong()
        self.check(self.lib.gmm_accumulate(self.h, flags, ptr(n), ptr(F), ptr(S),
                                           C.byref(tl), C.byref(tn)))
        return dict(n=n, F=F, S=S, totLL=tl.value, totN=tn.value)

    def accumulate_host(self, X, flags=ACC_MEAN | ACC_VAR):
        """E-step over host features (uploaded in chunks that overlap the E-step); statistics
        stay on the device."""
        X = np.ascontiguousarray(X, np.float32)
        N, D = X.shape
        self.check(self.lib.gmm_accumulate_host(self.h, flags, ptr(X), N, D))
        self.N = N

    def accumulate_device(self, flags=ACC_MEAN | ACC_VAR):
        self.check(self.lib.gmm_accumulate_device(self.h, flags))

    def read_stats(self):
        n = np.zeros(self.M)
        F = np.zeros((self.M, self.D))
        S = np.zeros((self.M, self.D))
        tl, tn = C.c_double(), C.c_longlong()
        self.check(self.lib.gmm_read_stats(self.h, ptr(n), ptr(F), ptr(S), C.byref(tl), C.byref(tn)))
        return dict(n=n, F=F, S=S, totLL=tl.value, totN=tn.value)

    def loglikes(self):
        out = np.zeros(self.N, np.float32)
        self.check(self.lib.gmm_loglikes(self.h, ptr(out)))
        return out

    # -- M-step
    def em_update(self, upW=True, upM=True, upV=True):
        a = C.c_int()
        self.check(self.lib.gmm_em_update(self.h, int(upW), int(upM), int(upV), C.byref(a)))
        self.last_alive = a.value
        return a.value

    def map_update(self, tau, upW=False, upM=True, upV=False):
        self.check(self.lib.gmm_map_update(self.h, int(tau), int(upW), int(upM), int(upV)))

    # -- --robust
    def set_robust(self, on=True):
        self.check(self.lib.gmm_set_robust(self.h, int(on)))

    def read_aux(self, full=False):
        M, D = (self.Mf, self.Df) if full else (self.M, self.D)
        aux, aux2, aux3 = np.zeros((M, D)), np.zeros(M), np.zeros(M)
        self.check(self.lib.gmm_read_aux(self.h, int(full), ptr(aux), ptr(aux2), ptr(aux3)))
        return dict(aux=aux, aux2=aux2, aux3=aux3)

    # -- fMLLR
    def fmllr_estimate(self, iters=20):
        """W [D, D+1] = [A | b] of the resident features against the resident diagonal model."""
        W = np.zeros((self.D, self.D + 1))
        self.check(self.lib.gmm_fmllr_estimate(self.h, int(iters), ptr(W)))
        return W

    def fmllr_estimate_full(self, iters=20):
        W = np.zeros((self.Df, self.Df + 1))
        self.check(self.lib.gmm_fmllr_estimate_full(self.h, int(iters), ptr(W)))
        return W

    def fmllr_apply(self, W):
        W = np.ascontiguousarray(W, np.float64)
        self.check(self.lib.gmm_fmllr_apply(self.h, ptr(W)))

    # -- full covariances (cov [M, D, D]; second-order statistics packed [M, D(D+1)/2])
    def upload_model_full(self, w, mu, cov):
        w = np.ascontiguousarray(w, np.float32)
        mu = np.ascontiguousarray(mu, np.float32)
        cov = np.ascontiguousarray(cov, np.float32)
        M, D = mu.shape
        if cov.shape != (M, D, D):
            raise ValueError("cov must be [M, D, D]")
        self.check(self.lib.gmm_upload_model_full(self.h, M, D, ptr(w), ptr(mu), ptr(cov)))
        self.Mf, self.Df = M, D

    def set_prior_full(self, w=None, mu=None, cov=None):
        if w is None:
            self.check(self.lib.gmm_set_prior_full(self.h, None, None, None))
            return
        w, mu, cov = (np.ascontiguousarray(a, np.float32) for a in (w, mu, cov))
        self.check(self.lib.gmm_set_prior_full(self.h, ptr(w), ptr(mu), ptr(cov)))

    def read_model_full(self):
        w = np.zeros(self.Mf, np.float32)
        mu = np.zeros((self.Mf, self.Df), np.float32)
        cov = np.zeros((self.Mf, self.Df, self.Df), np.float32)
        self.check(self.lib.gmm_read_model_full(self.h, ptr(w), ptr(mu), ptr(cov)))
        return w, mu, cov

    def _full_stats(self, fn, *args):
        P = self.Df * (self.Df + 1) // 2
        n, F, Sp = np.zeros(self.Mf), np.zeros((self.Mf, self.Df)), np.zeros((self.Mf, P))
        tl, tn = C.c_double(), C.c_longlong()
        self.check(fn(self.h, *args, ptr(n), ptr(F), ptr(Sp), C.byref(tl), C.byref(tn)))
        return dict(n=n, F=F, Sp=Sp, totLL=tl.value, totN=tn.value)

    def accumulate_full(self, flags=ACC_MEAN | ACC_VAR):
        return self._full_stats(self.lib.gmm_accumulate_full, flags)

    def accumulate_full_device(self, flags=ACC_MEAN | ACC_VAR):
        self.check(self.lib.gmm_accumulate_full_device(self.h, flags))

    def read_stats_full(self):
        return self._full_stats(self.lib.gmm_read_stats_full)

    def loglikes_full(self):
        out = np.zeros(self.N, np.float32)
        self.check(self.lib.gmm_loglikes_full(self.h, ptr(out)))
        return out

    def em_update_full(self, upW=True, upM=True, upV=True):
        a = C.c_int()
        self.check(self.lib.gmm_em_update_full(self.h, int(upW), int(upM), int(upV), C.byref(a)))
        self.last_alive = a.value
        return a.value

    def mllr_estimate_full(self, ubm_init=False):
        W = np.zeros((self.Df, self.Df + 1))
        self.check(self.lib.gmm_mllr_estimate_full(self.h, int(ubm_init), ptr(W)))
        return W

    def mllr_apply_full(self, W):
        W = np.ascontiguousarray(W, np.float64)
        self.check(self.lib.gmm_mllr_apply_full(self.h, ptr(W)))

    def map_update_full(self, tau, upW=False, upM=True, upV=False):
        self.check(self.lib.gmm_map_update_full(self.h, int(tau), int(upW), int(upM), int(upV)))

    def map_batch(self, offs, tau, upW=False, upM=True, upV=False):
        """One MAP iteration per speaker against the resident model (the UBM); speaker s owns the
        resident frames offs[s]:offs[s+1]. Returns (w [S,M], mu [S,M,D], var [S,M,D], ll [S])."""
        offs = np.ascontiguousarray(offs, np.int64)
        S = len(offs) - 1
        w = np.zeros((S, self.M), np.float32)
        mu = np.zeros((S, self.M, self.D), np.float32)
        var = np.zeros((S, self.M, self.D), np.float32)
        ll = np.zeros(S)
        self.check(self.lib.gmm_map_batch(self.h, S, ptr(offs), int(tau), int(upW), int(upM),
                                          int(upV), ptr(w), ptr(mu), ptr(var), ptr(ll)))
        return w, mu, var, ll

    def map_batch_device(self, offs, tau, upW, upM, upV, d_w=0, d_mu=0, d_var=0, d_ll=0):
        """map_batch into caller-owned device arrays (integer device pointers, 0 = not wanted)."""
        offs = np.ascontiguousarray(offs, np.int64)
        self.check(self.lib.gmm_map_batch_device(self.h, len(offs) - 1, ptr(offs), int(tau),
                                                 int(upW), int(upM), int(upV), d_w or None,
                                                 d_mu or None, d_var or None, d_ll or None))

    def mllr_batch(self, offs, ubm_init=False, means=True):
        """Global MLLR transform per speaker against the resident model (the UBM). Returns
        (W [S, D, D+1], status [S], adapted means [S, M, D] or None, ll [S])."""
        offs = np.ascontiguousarray(offs, np.int64)
        S = len(offs) - 1
        W = np.zeros((S, self.D, self.D + 1))
        st = np.zeros(S, np.int32)
        mu = np.zeros((S, self.M, self.D), np.float32) if means else None
        ll = np.zeros(S)
        self.check(self.lib.gmm_mllr_batch(self.h, S, ptr(offs), int(ubm_init), ptr(W), ptr(st),
                                           ptr(mu) if mu is not None else None, ptr(ll)))
        return W, st, mu, ll

    def map_batch_host(self, X, offs, tau, upW=False, upM=True, upV=False):
        """map_batch over frames in host memory (X [N, D] becomes the handle's features; on the
        tensor-core path the copy overlaps the E-step)."""
        X = np.ascontiguousarray(X, np.float32)
        offs = np.ascontiguousarray(offs, np.int64)
        S = len(offs) - 1
        w = np.zeros((S, self.M), np.float32)
        mu = np.zeros((S, self.M, self.D), np.float32)
        var = np.zeros((S, self.M, self.D), np.float32)
        ll = np.zeros(S)
        self.check(self.lib.gmm_map_batch_host(self.h, ptr(X), X.shape[0], X.shape[1], S, ptr(offs), int(tau),
                                               int(upW), int(upM), int(upV), ptr(w), ptr(mu), ptr(var), ptr(ll)))
        return w, mu, var, ll

    def mllr_batch_host(self, X, offs, ubm_init=False, means=True):
        """mllr_batch over frames in host memory (as map_batch_host)."""
        X = np.ascontiguousarray(X, np.float32)
        offs = np.ascontiguousarray(offs, np.int64)
        S = len(offs) - 1
        W = np.zeros((S, self.D, self.D + 1))
        st = np.zeros(S, np.int32)
        mu = np.zeros((S, self.M, self.D), np.float32) if means else None
        ll = np.zeros(S)
        self.check(self.lib.gmm_mllr_batch_host(self.h, ptr(X), X.shape[0], X.shape[1], S, ptr(offs), int(ubm_init),
                                                ptr(W), ptr(st), ptr(mu) if mu is not None else None, ptr(ll)))
        return W, st, mu, ll

    def em_iterate(self, iters, upW=True, upM=True, upV=True):
        ll = np.zeros(max(iters, 1))
        a = C.c_int()
        self.check(self.lib.gmm_em_iterate(self.h, iters, int(upW), int(upM), int(upV),
                                           ptr(ll), C.byref(a)))
        return ll[:iters], a.value

    def mllr_estimate(self, ubm_init=False):
        W = np.zeros((self.D, self.D + 1))
        self.check(self.lib.gmm_mllr_estimate(self.h, int(ubm_init), ptr(W)))
        return W

    def mllr_apply(self, W):
        W = np.ascontiguousarray(W, np.float64)
        self.check(self.lib.gmm_mllr_apply(self.h, ptr(W)))

    # -- profiling
    def profile(self, on=True):
        self.check(self.lib.gmm_profile_enable(self.h, int(on)))

    def profile_reset(self):
        self.check(self.lib.gmm_profile_reset(self.h))

    def profile_read(self):
        cap = 64
        names = (C.c_char_p * cap)()
        ms = np.zeros(cap)
        cnt = np.zeros(cap, np.int64)
        n = self.lib.gmm_profile_read(self.h, cap, names, ptr(ms), ptr(cnt))
        return {names[i].decode(): (float(ms[i]), int(cnt[i])) for i in range(min(n, cap))}

    def launch_count(self) -> int:
        return int(self.lib.gmm_launch_count(self.h))


class Server:
    """Continuous-batching request server (gmm_server_*): resident models, scoring and MAP
    requests. submit() returns a ticket; result() waits and returns the request's outputs."""

    def __init__(self, device: int, D: int, M: int, max_models: int, request_bytes: int):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.gmm_server_create(device, D, M, max_models, request_bytes, C.byref(h))
        if rc:
            raise GMMError(rc, self.lib.gmm_server_last_error(None).decode())
        self.h, self.D, self.M = h, D, M
        self._keep = {}

    def check(self, rc):
        if rc:
            raise GMMError(rc, self.lib.gmm_server_last_error(self.h).decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.lib.gmm_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_options(self, min_loglike=-1e20, min_gamma=1e-4, min_var=1e-6, max_batch=4096):
        self.check(self.lib.gmm_server_set_options(self.h, min_loglike, min_gamma, min_var, max_batch))

    def add_model(self, w, mu, var) -> int:
        w = np.ascontiguousarray(w, np.float32)
        mu = np.ascontiguousarray(mu, np.float32)
        var = np.ascontiguousarray(var, np.float32)
        mid = C.c_int()
        self.check(self.lib.gmm_server_add_model(self.h, ptr(w), ptr(mu), ptr(var), C.byref(mid)))
        return mid.value

    def submit(self, kind, model, X, tau=16, upW=0, upM=1, upV=0, frame_ll=False, no_copy=False) -> int:
        """no_copy: X must stay alive and unchanged until result() (the server keeps a reference)."""
        X = np.ascontiguousarray(X, np.float32)
        t = C.c_longlong()
        opts = (SUBMIT_FRAME_LL if frame_ll else 0) | (SUBMIT_NO_COPY if no_copy else 0)
        self.check(self.lib.gmm_server_submit(self.h, kind, model, ptr(X), len(X), tau, upW, upM, upV,
                                              opts, C.byref(t)))
        if no_copy:
            self._keep[t.value] = X
        self._n = getattr(self, "_n", {})
        self._n[t.value] = (kind, len(X), bool(frame_ll))
        return t.value

    def poll(self, ticket) -> int:
        st = C.c_int()
        self.check(self.lib.gmm_server_poll(self.h, ticket, C.byref(st)))
        return st.value

    def wait(self, ticket, timeout_ms=-1):
        self.check(self.lib.gmm_server_wait(self.h, ticket, timeout_ms))

    def result(self, ticket, timeout_ms=-1):
        """Waits for the request; returns dict(ll, latency_ms, frame_ll?, w/mu/var for MAP)."""
        self.wait(ticket, timeout_ms)
        kind, n, want_fll = self._n.pop(ticket)
        ll, lat = C.c_double(), C.c_double()
        out = {}
        fll = np.zeros(n, np.float32) if want_fll else None
        w = mu = var = None
        if kind == REQ_MAP:
            w = np.zeros(self.M, np.float32)
            mu = np.zeros((self.M, self.D), np.float32)
            var = np.zeros((self.M, self.D), np.float32)
        rc = self.lib.gmm_server_result(self.h, ticket, C.byref(ll), ptr(fll) if fll is not None else None,
                                        ptr(w) if w is not None else None, ptr(mu) if mu is not None else None,
                                        ptr(var) if var is not None else None, C.byref(lat))
        self._keep.pop(ticket, None)
        self.check(rc)
        out.update(ll=ll.value, latency_ms=lat.value)
        if fll is not None:
            out["frame_ll"] = fll
        if kind == REQ_MAP:
            out.update(w=w, mu=mu, var=var)
        return out

    def stats(self):
        b, c, f, p = C.c_longlong(), C.c_longlong(), C.c_longlong(), C.c_size_t()
        self.check(self.lib.gmm_server_stats(self.h, C.byref(b), C.byref(c), C.byref(f), C.byref(p)))
        return dict(batches=b.value, completed=c.value, failed=f.value, peak_batch_bytes=p.value)


def read_param(path: str, prm_type: int, dwnsmp: int = 1) -> np.ndarray:
    """One feature file through the library's reader (gmm_read_param)."""
    lib = load()
    N, D = C.c_longlong(), C.c_int()
    rc = lib.gmm_read_param(path.encode(), prm_type, dwnsmp, None, 0, C.byref(N), C.byref(D))
    if rc:
        raise GMMError(rc, f"gmm_read_param: cannot read {path}")
    out = np.zeros((N.value, D.value), np.float32)
    if out.size:
        rc = lib.gmm_read_param(path.encode(), prm_type, dwnsmp, ptr(out), N.value, C.byref(N), C.byref(D))
        if rc:
            raise GMMError(rc, f"gmm_read_param: cannot read {path}")
    return out
