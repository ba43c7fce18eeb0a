"""Tensor-core (tcgen05) path against the FP64 oracle.

The TC path evaluates the log-likelihood as a split-bf16 contraction with FP32 accumulation
and exact-in-FP32 operand splits, so it is compared with the FP64 oracle (not with the float
replica). Tolerances, written per quantity:
  per-frame log-likelihood   |diff| <= 2e-4 + 2e-6 |ll|
  total log-likelihood       rel <= 1e-6
  statistics                 |diff| <= 1e-4 * (scale of the component's statistic) -- posteriors
                             near the minGamma cut may land on the other side, which moves a
                             statistic by at most minGamma * |x| per frame
  EM update                  weights rel <= 1e-5, means |diff| <= 1e-5 of the standard deviation,
                             variances rel <= 1e-5 (as at the full UBM size,
                             tests/test_tc_accuracy_gpu.py)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def tc_handle(glib):
    h = glib.Handle(0)
    h.set_precision(glib.PREC_TC)
    return h


def check_stats(s, o, rel=1e-4):
    for k in ("n", "F", "S"):
        scale = np.maximum(np.abs(o[k]), np.abs(o["n"])[:, None] if k != "n" else 1.0) + 1.0
        err = np.abs(s[k] - o[k]) / scale
        assert err.max() <= rel, (k, err.max())


# K = 112 and 128 (D = 52, 55, 60) run the logits kernel's plane-granular W ring: with an even
# chunk count (M = 130, 256: two MMA-issuing threads) and an odd one (M = 300, 384: one)
@pytest.mark.parametrize("D,M,N", [(39, 16, 2048), (39, 200, 3000), (6, 8, 1000), (20, 4, 777),
                                   (60, 130, 2500), (1, 5, 640), (47, 64, 1536), (52, 300, 2000),
                                   (60, 384, 1800), (55, 256, 1500)])
def test_tc_matches_fp64(glib, oracle, D, M, N):
    from gmm_gb300 import synth
    X, w, mu, var = synth.config_em(100 + D, N, D, max(2, M // 2), M)
    h = tc_handle(glib)
    h.upload_model(w, mu, var)
    h.upload_features(X)
    ll = h.loglikes()
    o_ll = oracle.loglikes64(X, w, mu, var)
    assert np.all(np.abs(ll - o_ll) <= 2e-4 + 2e-6 * np.abs(o_ll)), np.abs(ll - o_ll).max()
    s = h.accumulate()
    o = oracle.accumulate64(X, w, mu, var)
    assert abs(s["totLL"] - o["totLL"]) <= 1e-6 * abs(o["totLL"])
    check_stats(s, o)
    h.close()


def test_tc_zero_weights_and_single_component(glib, oracle, golden):
    e = golden("edge.npz")
    h = tc_handle(glib)
    h.upload_model(e["zw_w"], e["zw_mu"], e["zw_var"])
    h.upload_features(e["zw_X"])
    s = h.accumulate()
    o = oracle.accumulate64(e["zw_X"], e["zw_w"], e["zw_mu"], e["zw_var"])
    check_stats(s, o)
    assert s["n"][1] == 0 and s["n"][5] == 0
    h.upload_model(np.ones(1, np.float32), e["zw_mu"][:1], e["zw_var"][:1])
    s = h.accumulate()
    assert np.allclose(s["n"], [len(e["zw_X"])])
    o = oracle.accumulate64(e["zw_X"], np.ones(1, np.float32), e["zw_mu"][:1], e["zw_var"][:1])
    check_stats(s, o, rel=1e-5)
    h.close()


def test_tc_outlier_frame(glib, oracle, golden):
    from gmm_gb300 import synth
    e = golden("edge.npz")
    w, mu, var = synth.generator_gmm(21, 8, 6)
    h = tc_handle(glib)
    h.upload_model(w, mu, var)
    h.upload_features(e["out_X"])
    ll = h.loglikes()
    assert ll[17] == np.float32(-1e20)
    s = h.accumulate()
    assert s["totLL"] == pytest.approx(float(e["out_totLL"]), rel=1e-9)
    h.close()


def test_tc_em_iteration_close_to_fp64(glib, oracle, golden):
    g = golden("em_small.npz")
    h = tc_handle(glib)
    h.upload_model(g["w"], g["mu"], g["var"])
    h.upload_features(g["X"])
    ll, alive = h.em_iterate(1)
    o = oracle.accumulate64(g["X"], g["w"], g["mu"], g["var"])
    ow, omu, ovar, _ = oracle.em_update64(g["w"], o)
    w, mu, var = h.read_model()
    assert abs(ll[0] - o["totLL"]) <= 1e-6 * abs(o["totLL"])
    live = ow > 0
    assert (np.abs(w - ow) / np.where(live, ow, 1.0))[live].max() <= 1e-5
    assert (np.abs(mu - omu) / np.sqrt(ovar))[live].max() <= 1e-5
    assert (np.abs(var - ovar) / ovar)[live].max() <= 1e-5
    h.close()


def test_tc_c1_full_size(glib, oracle):
    """Config C1 at full size through the TC path, against the FP64 oracle."""
    from gmm_gb300 import synth
    X, w, mu, var = synth.c1(seed=1)
    h = tc_handle(glib)
    h.upload_model(w, mu, var)
    h.upload_features(X)
    s = h.accumulate()
    o = oracle.accumulate64(X, w, mu, var)
    assert abs(s["totLL"] - o["totLL"]) <= 1e-6 * abs(o["totLL"])
    check_stats(s, o)
    # the kept posterior mass per frame never exceeds one
    assert s["n"].sum() <= len(X) * (1 + 1e-6)
    h.close()


def test_tc_em_iterate_graph_replays_eager_iterations(glib, golden):
    """gmm_em_iterate on the tensor-core path replays a captured CUDA graph of one iteration
    after an eager first one: five iterations in one call equal five one-iteration calls
    bit for bit (same kernels, same fixed shapes), including a component that dies."""
    from gmm_gb300 import synth
    X, w, mu, var = synth.config_em(17, 6000, 13, 8, 24)
    w = w.copy()
    w[3] = 1e-9  # a component with almost no support, killed by the first update
    w /= w.sum()
    h = tc_handle(glib)
    h.upload_model(w, mu, var)
    h.upload_features(X)
    ll5, a5 = h.em_iterate(5)
    m5 = h.read_model()
    h.upload_model(w, mu, var)
    lls = []
    for _ in range(5):
        l1, a1 = h.em_iterate(1)
        lls.append(l1[0])
    m1 = h.read_model()
    h.close()
    assert np.array_equal(ll5, np.array(lls)) and a5 == a1
    for x, y in zip(m5, m1):
        assert np.array_equal(x, y)
    assert a5 < 24  # the weak component died


def test_tc_autotune_choice_and_results(glib):
    """The autotuner picks a decomposition once per shape and keeps it; statistics with and
    without tuning agree to FP32 rounding: the decomposition decides which frame tiles share an
    FP32 period (64 tiles from each slice start) before the FP64 partial sums."""
    from gmm_gb300 import synth
    X, w, mu, var = synth.config_em(23, 200_000, 20, 16, 300)
    h = tc_handle(glib)
    h.set_tile_schedule(False)  # the autotuner decomposes the dense schedule
    h.upload_model(w, mu, var)
    h.upload_features(X)
    a = h.accumulate()
    ch = h.autotune_choices()
    assert len(ch) == 1 and list(ch.values())[0] in (1, 2, 3)
    h.accumulate()
    assert h.autotune_choices() == ch
    h.set_autotune(False)
    b = h.accumulate()
    h.close()
    for k in ("n", "F", "S"):
        assert np.allclose(a[k], b[k], rtol=1e-5, atol=1e-6 * np.abs(b[k]).max()), k


@pytest.mark.parametrize("N", [1000, 300_000])
def test_accumulate_host_streams_features(glib, N):
    """gmm_accumulate_host (chunked host-to-device copies overlapping the E-step) gives the same
    statistics as gmm_upload_features + gmm_accumulate: n, F, S bit-identical (the same
    statistics kernel over the same planes and the same decomposition -- the autotuner is off in
    both, as its choice regroups the FP32 sums), total LL within 1e-12 rel (the LL partials are
    grouped per chunk); the features stay resident for the next E-step."""
    from gmm_gb300 import synth
    X, w, mu, var = synth.config_em(5, N, 39, 32, 64)
    a = glib.Handle(0)
    a.set_precision(glib.PREC_TC)
    a.set_autotune(False)
    a.upload_model(w, mu, var)
    a.upload_features(X)
    ref = a.accumulate()
    a.close()
    b = glib.Handle(0)
    b.set_precision(glib.PREC_TC)
    b.set_autotune(False)
    b.upload_model(w, mu, var)
    b.accumulate_host(X)
    st = b.read_stats()
    again = b.accumulate()  # resident features
    b.close()
    for k in ("n", "F", "S"):
        assert np.array_equal(st[k], ref[k]), k
        assert np.array_equal(again[k], ref[k]), k
    assert abs(st["totLL"] - ref["totLL"]) <= 1e-12 * abs(ref["totLL"])
    assert st["totN"] == N
