"""Accuracy of the tensor-core path at the benchmarked shapes, against the FP64 oracle.

Bounds (the accuracy targets of the tensor-core form):
  total log-likelihood            rel <= 1e-4
  EM update, component weights    rel <= 1e-5
  EM update, means                |diff| <= 1e-5 of the component's standard deviation
  EM update, variances            rel <= 1e-5 (5e-5 with the opt-in sparse tile schedule)
  MAP means                       |diff| <= 1e-5 of the UBM standard deviation
Maximum over all components and dimensions, not a percentile.

UBM EM (N = 1M frames of a seeded 512-component generator, M = 2048, D = 39): the second EM
iteration, from the model that the FP64 oracle's first iteration gives, so that the components
sit on the data as in the benchmarked iterations. Batched mean-only MAP (UBM M = 1024, D = 60,
relevance factor 16) over four speakers of up to 30000 frames.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def test_tc_em_update_ubm_shape(glib, oracle):
    from gmm_gb300 import synth
    X, w0, mu0, var0 = synth.config_em(2, 1_000_000, 39, 512, 2048)
    o0 = oracle.accumulate64(X, w0, mu0, var0, threads=THREADS)
    ow, omu, ovar, _ = oracle.em_update64(w0, o0)
    w1, mu1, var1 = ow.astype(np.float32), omu.astype(np.float32), ovar.astype(np.float32)
    o1 = oracle.accumulate64(X, w1, mu1, var1, threads=THREADS)
    ew, emu, evar, _ = oracle.em_update64(w1, o1)

    for sched in (False, True):  # the dense and the sparse tile schedule of the statistics
        h = glib.Handle(0)
        h.set_precision(glib.PREC_TC)
        h.set_tile_schedule(sched)
        h.upload_model(w1, mu1, var1)
        h.upload_features(X)
        ll, alive = h.em_iterate(1)
        w, mu, var = h.read_model()
        h.close()

        ll_rel = abs(ll[0] - o1["totLL"]) / abs(o1["totLL"])
        live = o1["n"] >= 2  # components the update keeps (the others are reset in both)
        w_rel = (np.abs(w - ew) / ew)[live].max()
        mu_rel = (np.abs(mu - emu) / np.sqrt(evar))[live].max()
        var_rel = (np.abs(var - evar) / evar)[live].max()
        print(f"UBM EM, N=1M M=2048 D=39, {'sparse' if sched else 'dense'} schedule: LL rel {ll_rel:.2e}, "
              f"weights {w_rel:.2e}, means/sd {mu_rel:.2e}, variances {var_rel:.2e}")
        assert ll_rel <= 1e-4
        assert w_rel <= 1e-5
        assert mu_rel <= 1e-5
        # the sparse schedule (opt-in) sorts frames so that a component's posterior mass gathers
        # in fewer tiles, where the tensor core's round-toward-zero accumulation loses more low
        # bits: 2.4e-5 measured, about twice the reference's own FP32 arithmetic (1.1e-5)
        assert var_rel <= (5e-5 if sched else 1e-5)
        assert np.array_equal(w[~live], np.zeros((~live).sum(), np.float32))


def test_tc_map_batch_means_map_shape(glib, oracle):
    from gmm_gb300 import synth
    X, offs, (uw, umu, uvar) = synth.c3(seed=3, S=4, M=1024, D=60, lo=20000, hi=30000)
    tau = 16
    h = glib.Handle(0)
    h.set_precision(glib.PREC_TC)
    h.upload_model(uw, umu, uvar)
    h.upload_features(X)
    _, mu, _, ll = h.map_batch(offs, tau, upW=False, upM=True, upV=False)
    h.close()
    sd = np.sqrt(uvar.astype(np.float64))
    worst = 0.0
    for s in range(len(offs) - 1):
        Xs = X[offs[s]:offs[s + 1]]
        o = oracle.accumulate64(Xs, uw, umu, uvar, flags=oracle.ACC_MEAN, threads=THREADS)
        n = o["n"][:, None]
        alfa = n / (n + tau)
        adapted = (uw[:, None] > 0) & (n > 0)
        ref = np.where(adapted, alfa * o["F"] / np.maximum(n, 1e-300) + (1 - alfa) * umu, umu)
        worst = max(worst, (np.abs(mu[s] - ref) / sd).max())
        assert abs(ll[s] - o["totLL"]) <= 1e-4 * abs(o["totLL"])
    print(f"batched MAP, M=1024 D=60, 4 speakers: means/sd {worst:.2e}")
    assert worst <= 1e-5
