"""The reference-side binding GMMStatsEstimator_GB300 (oracle/ref/gb300_adapter.hpp), compiled
against the reference's own headers and run inside the reference's own CModelAdapt.

* Selection: CModelAdapt::InitializeEstimator (OL_ModelAdapt.cpp:248-267), reached through its
  --CUDA switch, constructs the GB300 estimator; on a machine without a GPU the engine's
  gmm_create fails and the estimator's constructor throws std::runtime_error with the engine's
  message, as the reference's estimators report failures.
* Bookkeeping: linked against a CPU stand-in of the engine's C ABI (the oracle's single-thread
  port, bit-exact to the reference CPU estimator), CModelAdapt::IterEM through the adapter and
  through the reference's own CPU estimator must agree bit for bit -- per-iteration total
  log-likelihood and the final model -- and so must a model group switched with
  setModelToBeUsed. That checks the rearranged order, the GMMStats += semantics, the totals and
  the accumulation flags the adapter passes.

Needs the reference sources (they are read in place); skipped where they are absent."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.skipif(not os.path.isdir(oracle.REF_SRC), reason="reference sources not present")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def adapter_libs():
    from gmm_gb300 import build
    build.build()
    oracle.build(ref=False)
    oracle.build_adapter(os.path.join(ROOT, "gmm_gb300", "_build"))
    return oracle.ADAPTER_FAKE, oracle.ADAPTER_GB300


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def test_initialize_estimator_selects_gb300_and_fails_cleanly_without_gpu(adapter_libs):
    # in a child process: the engine library and the CPU stand-in export the same C names
    code = ("import ctypes as C, sys\n"
            f"a = C.CDLL({adapter_libs[1]!r})\n"
            "b = C.create_string_buffer(512)\n"
            "rc = a.adt_initialize(b, 512)\n"
            "print(rc); print(b.value.decode())\n")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    rc, msg = out.stdout.strip().split("\n", 1)
    if rc == "0":  # a GPU is present: the estimator was built
        assert msg == "GB300"
    else:
        assert rc == "1", msg  # std::runtime_error, not another exception type
        assert msg.startswith("GMMStatsEstimator_GB300: gmm_create: "), msg
        assert "no CUDA device" in msg


def test_fake_engine_selected_by_initialize(adapter_libs):
    a = C.CDLL(adapter_libs[0])
    b = C.create_string_buffer(512)
    assert a.adt_initialize(b, 512) == 0, b.value
    assert b.value == b"GB300"


def _em(lib, X, w, mu, var, iters, gb300):
    w, mu, var = w.copy(), mu.copy(), var.copy()
    N, D = X.shape
    ll = np.zeros(iters)
    t = C.create_string_buffer(64)
    rc = lib.adt_em(_p(X), C.c_long(N), D, len(w), _p(w), _p(mu), _p(var), iters, gb300, _p(ll), t, 64)
    assert rc == 0, lib.adt_last_error()
    return w, mu, var, ll, t.value.decode()


def test_iter_em_through_adapter_matches_reference_estimator(adapter_libs):
    from gmm_gb300 import synth
    lib = C.CDLL(adapter_libs[0])
    lib.adt_last_error.restype = C.c_char_p
    X, w, mu, var = synth.config_em(61, 3000, 39, 8, 24)
    w = w.copy()
    w[[3, 10]] = 0.0  # zero-weight components: moved behind the others by insertModel
    w /= w.sum()
    a = _em(lib, X, w, mu, var, 4, 1)
    b = _em(lib, X, w, mu, var, 4, 0)
    assert a[4] == "GB300" and b[4] != "GB300"
    assert np.array_equal(a[3], b[3]), (a[3], b[3])   # per-iteration total log-likelihood
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
    assert np.all(np.diff(a[3]) > 0)


def _group(lib, gb300, fresh, X, w, mu, var, sel):
    K, M, D = mu.shape
    n = np.zeros((len(sel), M))
    F = np.zeros((len(sel), M, D))
    S = np.zeros((len(sel), M, D))
    tl = np.zeros(len(sel))
    t = C.create_string_buffer(64)
    rc = lib.adt_group(gb300, fresh, _p(X), C.c_long(len(X)), D, M, K, _p(w), _p(mu), _p(var), len(sel),
                       _p(sel), _p(n), _p(F), _p(S), _p(tl), t, 64)
    assert rc == 0, lib.adt_last_error()
    assert (t.value == b"GB300") == bool(gb300)
    return n, F, S, tl


def _three_models(same_var):
    from gmm_gb300 import synth
    M, D = 16, 39
    X = synth.config_em(71, 2500, D, 8, M)[0]
    ws, mus, vs = [], [], []
    for k in range(3):
        _, w, mu, var = synth.config_em(72 + k, 2500, D, 8, M)
        w = w.copy()
        if k == 1:
            w[5] = 0.0
            w /= w.sum()
        ws.append(w)
        mus.append(mu)
        vs.append(vs[0] if (same_var and vs) else var)
    w, mu, var = (np.ascontiguousarray(np.stack(a), np.float32) for a in (ws, mus, vs))
    return X, w, mu, var


def test_model_group_through_adapter(adapter_libs):
    """setModelToBeUsed(n) through the adapter gives exactly what an estimator holding model n
    alone gives (reference CPU estimator, one model per estimator).

    The reference's own CPU estimator cannot serve as the group oracle in general: insertModel
    gives every model of a group a new _icov array (OL_GMMStatsEstimator.cpp:255-268) but keeps no
    per-model copy, and setModelToBeUsed (:318-325) does not switch it back, so a switch to an
    earlier model runs with the last model's inverse variances. With one shared variance set
    that cannot matter, and there the reference's group switching matches the adapter's too."""
    lib = C.CDLL(adapter_libs[0])
    lib.adt_last_error.restype = C.c_char_p
    sel = np.array([1, 0, 2, 1], np.int32)
    X, w, mu, var = _three_models(same_var=False)
    got = _group(lib, 1, 0, X, w, mu, var, sel)
    alone = _group(lib, 0, 1, X, w, mu, var, sel)
    for x, y in zip(got, alone):
        assert np.array_equal(x, y)
    M = w.shape[1]
    # model 1's zero-weight component sits last after the rearrangement and gets no statistics
    assert np.all(got[0][[0, 3], M - 1] == 0.0) and np.all(got[0][[1, 2], M - 1] > 0.0)
    X, w, mu, var = _three_models(same_var=True)
    got = _group(lib, 1, 0, X, w, mu, var, sel)
    ref_group = _group(lib, 0, 0, X, w, mu, var, sel)
    for x, y in zip(got, ref_group):
        assert np.array_equal(x, y)
