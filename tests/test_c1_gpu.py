"""Plain EM at its specified size on the GPU: D = 39 float32 features, N = 100k frames of a
seeded 64-component diagonal GMM, M = 64 fitted from the random-frame initialisation, 10 EM
iterations (weights, means and variances).

Plain FP32 path: the per-iteration total log-likelihood within 1e-6 relative of the reference
CPU algorithm (the oracle port, which is bit-identical to the reference build), and the final
model within 1e-4. Tensor-core path: each iteration's total log-likelihood within 1e-4 relative
of the FP64 oracle run over the same 10 iterations.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ITERS = 10


def _device_run(glib, prec, X, w, mu, var):
    h = glib.Handle(0)
    h.set_precision(prec)
    h.upload_model(w, mu, var)
    h.upload_features(X)
    ll, alive = h.em_iterate(ITERS)
    model = h.read_model()
    h.close()
    return ll, alive, model


def test_c1_plain_ten_iterations_match_reference(glib, oracle):
    from gmm_gb300 import synth
    X, w, mu, var = synth.c1(seed=1)
    ll, alive, (dw, dmu, dvar) = _device_run(glib, glib.PREC_FP32, X, w, mu, var)
    rw, rmu, rvar = w.copy(), mu.copy(), var.copy()
    ref_ll = []
    for _ in range(ITERS):
        st = oracle.accumulate32(X, rw, rmu, rvar, threads=4)
        ref_ll.append(st["totLL"])
        rw, rmu, rvar, _ = oracle.em_update(rw, rmu, rvar, st)
    ref_ll = np.array(ref_ll)
    rel = np.abs(ll - ref_ll) / np.abs(ref_ll)
    print("C1 plain: per-iteration LL rel", " ".join(f"{r:.1e}" for r in rel))
    assert np.all(rel <= 1e-6)
    assert np.all(np.diff(ll) > 0)  # EM increases the likelihood
    assert np.allclose(dw, rw, rtol=1e-4, atol=1e-7)
    assert np.allclose(dmu, rmu, rtol=1e-4, atol=1e-4)
    assert np.allclose(dvar, rvar, rtol=1e-4, atol=1e-6)


def test_c1_tensor_core_ten_iterations_against_fp64(glib, oracle):
    from gmm_gb300 import synth
    X, w, mu, var = synth.c1(seed=1)
    ll, alive, _ = _device_run(glib, glib.PREC_TC, X, w, mu, var)
    ow = w.copy()
    omu, ovar = mu.astype(np.float64), var.astype(np.float64)
    ref_ll = []
    for _ in range(ITERS):
        st = oracle.accumulate64(X, ow, omu, ovar, threads=8)
        ref_ll.append(st["totLL"])
        nw, nmu, nvar, _ = oracle.em_update64(ow, st)
        keep = (nw > 0)[:, None]  # a killed component keeps its old parameters (weight 0)
        omu, ovar = np.where(keep, nmu, omu), np.where(keep, nvar, ovar)
        ow = nw.astype(np.float32)
    ref_ll = np.array(ref_ll)
    rel = np.abs(ll - ref_ll) / np.abs(ref_ll)
    print("C1 tensor core: per-iteration LL rel vs FP64", " ".join(f"{r:.1e}" for r in rel))
    assert np.all(rel <= 1e-4)
