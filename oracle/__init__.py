"""CPU checkers for the GMM hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may use
this package, and only as the checker (or, in bench.py, as the timed CPU baseline). The
product package ``gmm_gb300`` never imports it.

Two libraries, both built by ``oracle/Makefile``:

* ``_build/liboracle.so`` -- the C restatement in ``gmm_oracle.c``: ``*32`` functions follow
  the reference CPU estimator's float semantics operation by operation (the "port"), ``*64``
  functions are the FP64 oracle. Builds on any host.
* ``_ref/libgmmref.so`` -- the reference's own CPU estimator and ``CModelAdapt`` compiled from
  the reference sources (only where those sources are present). Used to pin the port.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libgmmref.so")
# The reference GMM project (its lib_bmssr sources and example/): $GMM_REF_ROOT, else the
# checkout named "reference" beside this repository. Absent on machines without it.
REF_ROOT = os.environ.get("GMM_REF_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                           "reference", "GMM")
REF_SRC = os.path.join(REF_ROOT, "lib_bmssr")

ACC_MEAN, ACC_VAR, ACC_PROBS_ONLY = 1, 2, 4


class _Opts(C.Structure):
    _fields_ = [("minLogLike", C.c_float), ("minGamma", C.c_float),
                ("min_var", C.c_float), ("threads", C.c_int)]


def build(ref: bool | None = None) -> None:
    """Compile the port (always) and the reference library (when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if ref is None:
        ref = os.path.isdir(REF_SRC)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={REF_SRC}"], check=True)


def build_adapter(engine_dir: str) -> None:
    """Compile the reference-side binding (ref/gb300_adapter.hpp) against the reference headers,
    linked against the engine in `engine_dir` and against the CPU stand-in of its C ABI
    (ref/fake_engine.c): _ref/libadapter_gb300.so and _ref/libadapter_fake.so."""
    subprocess.run(["make", "-s", "-C", HERE, "adapter", f"REF_ROOT={REF_SRC}", f"ENGINE_DIR={engine_dir}"],
                   check=True)


ADAPTER_FAKE = os.path.join(HERE, "_ref", "libadapter_fake.so")
ADAPTER_GB300 = os.path.join(HERE, "_ref", "libadapter_gb300.so")

_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        _lib = C.CDLL(LIB_PATH)
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        _ref = C.CDLL(REF_PATH)
        _ref.ref_last_error.restype = C.c_char_p
    return _ref


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _opts(threads=1, minLogLike=-1e20, minGamma=1e-4, min_var=1e-6):
    return _Opts(minLogLike, minGamma, min_var, threads)


def rearrange_order(w):
    w = _f32(w)
    order = np.zeros(len(w), np.int32)
    nz = lib().orc_rearrange_order(len(w), _p(w), _p(order))
    return order, nz


def loglikes32(X, w, mu, var, threads=1, **kw):
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    out = np.zeros(N, np.float32)
    trouble = C.c_int(0)
    o = _opts(threads, **kw)
    rc = lib().orc32_loglikes(_p(X), C.c_longlong(N), D, len(w), _p(w), _p(mu), _p(var),
                              C.byref(o), _p(out), C.byref(trouble))
    if rc:
        raise RuntimeError(f"orc32_loglikes failed ({rc})")
    return out


def accumulate32(X, w, mu, var, flags=ACC_MEAN | ACC_VAR, threads=1, **kw):
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    M = len(w)
    n, F, S = np.zeros(M), np.zeros((M, D)), np.zeros((M, D))
    tl, tn = C.c_double(0.0), C.c_longlong(0)
    o = _opts(threads, **kw)
    rc = lib().orc32_accumulate(_p(X), C.c_longlong(N), D, M, _p(w), _p(mu), _p(var),
                                C.byref(o), flags, _p(n), _p(F), _p(S), C.byref(tl), C.byref(tn))
    if rc:
        raise RuntimeError(f"orc32_accumulate failed ({rc})")
    return dict(n=n, F=F, S=S, totLL=tl.value, totN=tn.value)


def loglikes64(X, w, mu, var, **kw):
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    out = np.zeros(N)
    o = _opts(1, **kw)
    rc = lib().orc64_loglikes(_p(X), C.c_longlong(N), D, len(w), _p(w), _p(mu), _p(var),
                              C.byref(o), _p(out))
    if rc:
        raise RuntimeError(f"orc64_loglikes failed ({rc})")
    return out


def accumulate64(X, w, mu, var, flags=ACC_MEAN | ACC_VAR, threads=1, **kw):
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    M = len(w)
    n, F, S = np.zeros(M), np.zeros((M, D)), np.zeros((M, D))
    tl, tn = C.c_double(0.0), C.c_longlong(0)
    o = _opts(threads, **kw)
    rc = lib().orc64_accumulate(_p(X), C.c_longlong(N), D, M, _p(w), _p(mu), _p(var),
                                C.byref(o), flags, _p(n), _p(F), _p(S), C.byref(tl), C.byref(tn))
    if rc:
        raise RuntimeError(f"orc64_accumulate failed ({rc})")
    return dict(n=n, F=F, S=S, totLL=tl.value, totN=tn.value)


def em_update(w, mu, var, st, upW=True, upM=True, upV=True, min_var=1e-6):
    w, mu, var = _f32(w).copy(), _f32(mu).copy(), _f32(var).copy()
    M, D = mu.shape
    n, F, S = (np.ascontiguousarray(st[k], np.float64) for k in ("n", "F", "S"))
    alive = lib().orc_em_update(M, D, _p(w), _p(mu), _p(var), _p(n), _p(F), _p(S),
                                C.c_longlong(st["totN"]), int(upW), int(upM), int(upV),
                                C.c_float(min_var))
    return w, mu, var, alive


def em_update64(w, st, upW=True, upM=True, upV=True, min_var=1e-6):
    w = _f32(w)
    M, D = st["F"].shape
    n, F, S = (np.ascontiguousarray(st[k], np.float64) for k in ("n", "F", "S"))
    ow, omu, ovar = np.zeros(M), np.zeros((M, D)), np.zeros((M, D))
    alive = lib().orc64_em_update(M, D, _p(w), _p(n), _p(F), _p(S), C.c_longlong(st["totN"]),
                                  int(upW), int(upM), int(upV), C.c_double(min_var),
                                  _p(ow), _p(omu), _p(ovar))
    return ow, omu, ovar, alive


def map_update(ubm_w, ubm_mu, ubm_var, st, tau, w=None, mu=None, var=None,
               upW=False, upM=True, upV=False, min_var=1e-6):
    ubm_w, ubm_mu, ubm_var = map(_f32, (ubm_w, ubm_mu, ubm_var))
    w = (ubm_w if w is None else _f32(w)).copy()
    mu = (ubm_mu if mu is None else _f32(mu)).copy()
    var = (ubm_var if var is None else _f32(var)).copy()
    M, D = mu.shape
    n, F, S = (np.ascontiguousarray(st[k], np.float64) for k in ("n", "F", "S"))
    lib().orc_map_update(M, D, _p(w), _p(mu), _p(var), _p(ubm_w), _p(ubm_mu), _p(ubm_var),
                         _p(n), _p(F), _p(S), C.c_longlong(st["totN"]), int(tau),
                         int(upW), int(upM), int(upV), C.c_float(min_var))
    return w, mu, var


def mllr_w(mu, var, st, ubm_mu=None, ubm_var=None, ubm_init=False, min_var=1e-6):
    mu, var = _f32(mu), _f32(var)
    M, D = mu.shape
    ubm_mu = mu if ubm_mu is None else _f32(ubm_mu)
    ubm_var = var if ubm_var is None else _f32(ubm_var)
    n, F = (np.ascontiguousarray(st[k], np.float64) for k in ("n", "F"))
    W = np.zeros((D, D + 1))
    rc = lib().orc_mllr_w(M, D, _p(mu), _p(var), _p(ubm_mu), _p(ubm_var), _p(n), _p(F),
                          int(ubm_init), C.c_float(min_var), _p(W))
    if rc:
        raise RuntimeError(f"orc_mllr_w failed ({rc}): MLLR invertibility conditions not met")
    return W


def mllr_apply(mu, W):
    mu = _f32(mu)
    M, D = mu.shape
    W = np.ascontiguousarray(W, np.float64)
    out = np.zeros_like(mu)
    lib().orc_mllr_apply(M, D, _p(mu), _p(W), _p(out))
    return out


# ------------------------------------------------------------------ reference library

def ref_loglikes(X, w, mu, var, threads=1, sse=False):
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    out = np.zeros(N, np.float32)
    rc = ref().ref_loglikes(_p(X), C.c_long(N), D, len(w), _p(w), _p(mu), _p(var),
                            threads, int(sse), _p(out))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return out


def ref_accumulate(X, w, mu, var, flags=ACC_MEAN | ACC_VAR, threads=1, sse=False):
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    M = len(w)
    n, F, S = np.zeros(M), np.zeros((M, D)), np.zeros((M, D))
    tl, tn = C.c_double(0.0), C.c_uint(0)
    order = np.zeros(M, np.int32)
    rc = ref().ref_accumulate(_p(X), C.c_long(N), D, M, _p(w), _p(mu), _p(var), threads,
                              int(sse), flags, _p(n), _p(F), _p(S), C.byref(tl), C.byref(tn),
                              _p(order))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return dict(n=n, F=F, S=S, totLL=tl.value, totN=tn.value, order=order)


def ref_em(X, w, mu, var, iters, upW=True, upM=True, upV=True, threads=1, sse=False):
    X = _f32(X)
    w, mu, var = _f32(w).copy(), _f32(mu).copy(), _f32(var).copy()
    N, D = X.shape
    M = len(w)
    ll = np.zeros(iters)
    order = np.zeros(M, np.int32)
    rc = ref().ref_em(_p(X), C.c_long(N), D, M, _p(w), _p(mu), _p(var), iters, int(upW),
                      int(upM), int(upV), threads, int(sse), _p(ll), _p(order))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return w, mu, var, ll


def ref_map(X, w, mu, var, tau, iters=1, upW=False, upM=True, upV=False, threads=1, sse=False):
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    M = len(w)
    ow, omu, ovar = np.zeros_like(w), np.zeros_like(mu), np.zeros_like(var)
    ll = np.zeros(iters)
    rc = ref().ref_map(_p(X), C.c_long(N), D, M, _p(w), _p(mu), _p(var), int(tau), iters,
                       int(upW), int(upM), int(upV), threads, int(sse), _p(ow), _p(omu),
                       _p(ovar), _p(ll))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return ow, omu, ovar, ll


def ref_mllr(X, w, mu, var, iters=1, ubm_init=False, threads=1, sse=False):
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    M = len(w)
    W = np.zeros((D, D + 1))
    omu = np.zeros_like(mu)
    rc = ref().ref_mllr(_p(X), C.c_long(N), D, M, _p(w), _p(mu), _p(var), iters,
                        int(ubm_init), threads, int(sse), _p(W), _p(omu))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return W, omu


def ref_param_load(path, prm_type, dwnsmp=1):
    """The reference's Param::Load on one feature file (None when the file is missing)."""
    N, D = C.c_longlong(), C.c_int()
    f = ref().ref_param_load
    f.argtypes = [C.c_char_p, C.c_int, C.c_uint, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong),
                  C.POINTER(C.c_int)]
    rc = f(path.encode(), prm_type, dwnsmp, None, 0, C.byref(N), C.byref(D))
    if rc == -1:
        return None
    if rc:
        raise RuntimeError(f"reference Param::Load failed ({rc})")
    out = np.zeros((N.value, D.value), np.float32)
    rc = f(path.encode(), prm_type, dwnsmp, _p(out) if out.size else None, N.value, C.byref(N), C.byref(D))
    if rc:
        raise RuntimeError(f"reference Param::Load failed ({rc})")
    return out


def ref_train(X, nummix, iters_em=5, split_x=0.0, split_th=0.0, ll_th=0.0, verbosity=0, threads=1):
    """The reference's TrainFromScratch on X (diagonal covariances); returns (w, mu, var)."""
    X = _f32(X)
    N, D = X.shape
    w, mu, var = np.zeros(nummix, np.float32), np.zeros((nummix, D), np.float32), np.zeros((nummix, D), np.float32)
    f = ref().ref_train
    f.argtypes = [C.c_void_p, C.c_long, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                  C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    rc = f(_p(X), N, D, nummix, iters_em, split_x, split_th, ll_th, verbosity, threads, _p(w), _p(mu), _p(var))
    if rc:
        raise RuntimeError(f"reference TrainFromScratch failed: {ref().ref_last_error().decode()}")
    return w, mu, var

# ------------------------------------------------------------------ full covariances

def full64_loglikes(X, w, mu, cov):
    """FP64 per-frame log-likelihoods under a full-covariance model (cov: [M, D, D])."""
    X, w, mu, cov = map(_f32, (X, w, mu, cov))
    N, D = X.shape
    out = np.zeros(N)
    rc = lib().orc64_full_loglikes(_p(X), C.c_longlong(N), D, len(w), _p(w), _p(mu), _p(cov), _p(out))
    if rc:
        raise RuntimeError(f"orc64_full_loglikes failed ({rc})")
    return out


def full64_accumulate(X, w, mu, cov, flags=ACC_MEAN | ACC_VAR, **kw):
    """FP64 statistics: n [M], F [M, D], Sp [M, D(D+1)/2] (packed upper triangle, row order)."""
    X, w, mu, cov = map(_f32, (X, w, mu, cov))
    N, D = X.shape
    M = len(w)
    P = D * (D + 1) // 2
    n, F, Sp = np.zeros(M), np.zeros((M, D)), np.zeros((M, P))
    tl, tn = C.c_double(0.0), C.c_longlong(0)
    o = _opts(1, **kw)
    rc = lib().orc64_full_accumulate(_p(X), C.c_longlong(N), D, M, _p(w), _p(mu), _p(cov), C.byref(o),
                                     flags, _p(n), _p(F), _p(Sp), C.byref(tl), C.byref(tn))
    if rc:
        raise RuntimeError(f"orc64_full_accumulate failed ({rc})")
    return dict(n=n, F=F, Sp=Sp, totLL=tl.value, totN=tn.value)


def full_em_update(w, mu, cov, st, upW=True, upM=True, upV=True):
    w, mu, cov = _f32(w).copy(), _f32(mu).copy(), _f32(cov).copy()
    M, D = mu.shape
    n, F, Sp = (np.ascontiguousarray(st[k], np.float64) for k in ("n", "F", "Sp"))
    alive = lib().orc_full_em_update(M, D, _p(w), _p(mu), _p(cov), _p(n), _p(F), _p(Sp),
                                     C.c_longlong(int(st["totN"])), int(upW), int(upM), int(upV))
    return w, mu, cov, alive


def full_map_update(ubm_w, ubm_mu, ubm_cov, st, tau, upW=False, upM=True, upV=False):
    ubm_w, ubm_mu, ubm_cov = map(_f32, (ubm_w, ubm_mu, ubm_cov))
    w, mu, cov = ubm_w.copy(), ubm_mu.copy(), ubm_cov.copy()
    M, D = mu.shape
    n, F, Sp = (np.ascontiguousarray(st[k], np.float64) for k in ("n", "F", "Sp"))
    lib().orc_full_map_update(M, D, _p(w), _p(mu), _p(cov), _p(ubm_w), _p(ubm_mu), _p(ubm_cov), _p(n),
                              _p(F), _p(Sp), C.c_longlong(int(st["totN"])), int(tau), int(upW), int(upM),
                              int(upV))
    return w, mu, cov


def ref_full_loglikes(X, w, mu, cov, threads=1):
    X, w, mu, cov = map(_f32, (X, w, mu, cov))
    N, D = X.shape
    out = np.zeros(N, np.float32)
    rc = ref().ref_full_loglikes(_p(X), C.c_long(N), D, len(w), _p(w), _p(mu), _p(cov), threads, _p(out))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return out


def ref_full_accumulate(X, w, mu, cov, flags=ACC_MEAN | ACC_VAR, threads=1):
    X, w, mu, cov = map(_f32, (X, w, mu, cov))
    N, D = X.shape
    M = len(w)
    P = D * (D + 1) // 2
    n, F, Sp = np.zeros(M), np.zeros((M, D)), np.zeros((M, P))
    tl, tn = C.c_double(0.0), C.c_uint(0)
    order = np.zeros(M, np.int32)
    rc = ref().ref_full_accumulate(_p(X), C.c_long(N), D, M, _p(w), _p(mu), _p(cov), threads, flags,
                                   _p(n), _p(F), _p(Sp), C.byref(tl), C.byref(tn), _p(order))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return dict(n=n, F=F, Sp=Sp, totLL=tl.value, totN=tn.value, order=order)


def ref_full_adapt(X, w, mu, cov, tau, iters, upW=True, upM=True, upV=True, threads=1):
    """IterEM (tau = 0) or IterMAP (tau > 0) on a full-covariance model."""
    X = _f32(X)
    w, mu, cov = _f32(w).copy(), _f32(mu).copy(), _f32(cov).copy()
    N, D = X.shape
    ll = np.zeros(iters)
    rc = ref().ref_full_adapt(_p(X), C.c_long(N), D, len(w), _p(w), _p(mu), _p(cov), int(tau), iters,
                              int(upW), int(upM), int(upV), threads, _p(ll))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return w, mu, cov, ll


# ------------------------------------------------------------------ fMLLR

def accumulate64_fullstats(X, w, mu, var, **kw):
    """FP64 E-step of a diagonal model with packed full second-order statistics."""
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    M = len(w)
    P = D * (D + 1) // 2
    n, F, Sp = np.zeros(M), np.zeros((M, D)), np.zeros((M, P))
    tl, tn = C.c_double(0.0), C.c_longlong(0)
    o = _opts(1, **kw)
    rc = lib().orc64_accumulate_fullstats(_p(X), C.c_longlong(N), D, M, _p(w), _p(mu), _p(var), C.byref(o),
                                          _p(n), _p(F), _p(Sp), C.byref(tl), C.byref(tn))
    if rc:
        raise RuntimeError(f"orc64_accumulate_fullstats failed ({rc})")
    return dict(n=n, F=F, Sp=Sp, totLL=tl.value, totN=tn.value)


def fmllr_w(mu, var, st, iters=20):
    """ComputeW_fMLLR from statistics (n, F, Sp, totN): W [D, D+1]."""
    mu, var = _f32(mu), _f32(var)
    M, D = mu.shape
    n, F, Sp = (np.ascontiguousarray(st[k], np.float64) for k in ("n", "F", "Sp"))
    W = np.zeros((D, D + 1))
    rc = lib().orc_fmllr_w(M, D, _p(mu), _p(var), _p(n), _p(F), _p(Sp), C.c_longlong(int(st["totN"])),
                           int(iters), _p(W))
    if rc:
        raise RuntimeError(f"orc_fmllr_w failed ({rc})")
    return W


def ref_fmllr(X, w, mu, var, threads=1):
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    M = len(w)
    P = D * (D + 1) // 2
    W = np.zeros((D, D + 1))
    n, F, Sp = np.zeros(M), np.zeros((M, D)), np.zeros((M, P))
    tl = C.c_double(0.0)
    rc = ref().ref_fmllr(_p(X), C.c_long(N), D, M, _p(w), _p(mu), _p(var), threads, _p(W), _p(n), _p(F),
                         _p(Sp), C.byref(tl))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return W, dict(n=n, F=F, Sp=Sp, totLL=tl.value, totN=N)


def ref_adapt_model(X, w, mu, var, adapt_type, tau=16, it_em=0, it_map=1, it_mllr=1, mllr_init=False,
                    upW=False, upM=True, upV=False, threads=1):
    """CModelAdapt::AdaptModel of the reference build (2 = MAP, 4 = MLLR+MAP)."""
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    M = len(w)
    ow, omu, ovar = np.zeros_like(w), np.zeros_like(mu), np.zeros_like(var)
    rc = ref().ref_adapt_model(_p(X), C.c_long(N), D, M, _p(w), _p(mu), _p(var), int(adapt_type), int(tau),
                               int(it_em), int(it_map), int(it_mllr), int(mllr_init), int(upW), int(upM),
                               int(upV), threads,
                               _p(ow), _p(omu), _p(ovar))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return ow, omu, ovar


# ------------------------------------------------------------------ --robust

def aux64(X, w, mu, var, full=False, **kw):
    """FP64 auxiliary statistics of --robust: aux [M, D], aux2 [M], aux3 [M]."""
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    M = len(w)
    aux, aux2, aux3 = np.zeros((M, D)), np.zeros(M), np.zeros(M)
    o = _opts(1, **kw)
    rc = lib().orc64_aux_stats(_p(X), C.c_longlong(N), D, M, _p(w), _p(mu), _p(var), int(full), C.byref(o),
                               _p(aux), _p(aux2), _p(aux3))
    if rc:
        raise RuntimeError(f"orc64_aux_stats failed ({rc})")
    return dict(aux=aux, aux2=aux2, aux3=aux3)


def make_robust(st, aux, full=False):
    """GetNIndFrames + MakeRobustStats: returns (modified second-order statistics, nind)."""
    n, F = (np.ascontiguousarray(st[k], np.float64) for k in ("n", "F"))
    S = np.ascontiguousarray(st["Sp" if full else "S"], np.float64).copy()
    M, D = F.shape
    a, a2, a3 = (np.ascontiguousarray(aux[k], np.float64) for k in ("aux", "aux2", "aux3"))
    nind = np.zeros(M)
    rc = lib().orc_make_robust(M, D, int(full), _p(n), _p(F), _p(S), _p(a), _p(a2), _p(a3), _p(nind))
    if rc:
        raise RuntimeError(f"orc_make_robust failed ({rc})")
    return S, nind


def em_update_robust(w, mu, var, st, S, nind, upW=True, upM=True, upV=True, min_var=1e-6, full=False):
    """UpdateModelEM with robust statistics S and the kill rule on nind."""
    w, mu, var = _f32(w).copy(), _f32(mu).copy(), _f32(var).copy()
    M, D = mu.shape
    n, F = (np.ascontiguousarray(st[k], np.float64) for k in ("n", "F"))
    S = np.ascontiguousarray(S, np.float64)
    nind = np.ascontiguousarray(nind, np.float64)
    if full:
        alive = lib().orc_full_em_update_nind(M, D, _p(w), _p(mu), _p(var), _p(n), _p(F), _p(S),
                                              C.c_longlong(int(st["totN"])), int(upW), int(upM), int(upV), _p(nind))
    else:
        alive = lib().orc_em_update_nind(M, D, _p(w), _p(mu), _p(var), _p(n), _p(F), _p(S),
                                         C.c_longlong(int(st["totN"])), int(upW), int(upM), int(upV),
                                         C.c_float(min_var), _p(nind))
    return w, mu, var, alive


def ref_aux_accumulate(X, w, mu, var, full=False):
    X, w, mu, var = map(_f32, (X, w, mu, var))
    N, D = X.shape
    M = len(w)
    aux, aux2, aux3 = np.zeros((M, D)), np.zeros(M), np.zeros(M)
    order = np.zeros(M, np.int32)
    rc = ref().ref_aux_accumulate(_p(X), C.c_long(N), D, M, _p(w), _p(mu), _p(var), int(full), _p(aux), _p(aux2),
                                  _p(aux3), _p(order))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return dict(aux=aux, aux2=aux2, aux3=aux3, order=order)


def ref_robust_adapt(X, w, mu, var, tau, iters, full=False, upW=True, upM=True, upV=True):
    X = _f32(X)
    w, mu, var = _f32(w).copy(), _f32(mu).copy(), _f32(var).copy()
    N, D = X.shape
    ll = np.zeros(iters)
    rc = ref().ref_robust_adapt(_p(X), C.c_long(N), D, len(w), _p(w), _p(mu), _p(var), int(full), int(tau),
                                iters, int(upW), int(upM), int(upV), _p(ll))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return w, mu, var, ll


def ref_full_mllr(X, w, mu, cov, iters=1, ubm_init=False, threads=1):
    X, w, mu, cov = map(_f32, (X, w, mu, cov))
    N, D = X.shape
    M = len(w)
    W = np.zeros((D, D + 1))
    omu = np.zeros_like(mu)
    rc = ref().ref_full_mllr(_p(X), C.c_long(N), D, M, _p(w), _p(mu), _p(cov), iters, int(ubm_init), threads,
                             _p(W), _p(omu))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return W, omu


def ref_train_full(X, nummix, iters_em=5, split_x=0.0, split_th=0.0, ll_th=0.0, verbosity=0, threads=1):
    """TrainFromScratch with full covariances (the split along the leading eigenvector)."""
    X = _f32(X)
    N, D = X.shape
    w, mu, cov = np.zeros(nummix, np.float32), np.zeros((nummix, D), np.float32), np.zeros((nummix, D, D), np.float32)
    rc = ref().ref_train_full(_p(X), C.c_long(N), D, nummix, iters_em, C.c_float(split_x), C.c_float(split_th),
                              C.c_float(ll_th), verbosity, threads, 1, _p(w), _p(mu), _p(cov))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return w, mu, cov


def ref_fmllr_full(X, w, mu, cov):
    X, w, mu, cov = map(_f32, (X, w, mu, cov))
    N, D = X.shape
    W = np.zeros((D, D + 1))
    rc = ref().ref_fmllr_full(_p(X), C.c_long(N), D, len(w), _p(w), _p(mu), _p(cov), _p(W))
    if rc:
        raise RuntimeError(ref().ref_last_error().decode())
    return W
