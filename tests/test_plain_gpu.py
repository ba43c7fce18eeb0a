"""Parity of the plain FP32 CUDA path with the oracle (and through it with the reference).

The plain path replicates the reference CPU arithmetic; the only source of difference is the
last-ulp behaviour of expf/logf on the GPU versus glibc. Tolerances:
  per-frame log-likelihood        |diff| <= 2e-5 + 2e-6 |ll|
  total log-likelihood            rel <= 1e-6
  statistics n, F, S              rel <= 1e-5 of the component's scale (abs floor 1e-6 n)
  EM model after 3 iterations     rel <= 1e-4 (updates are bit-exact given equal statistics)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def close_stats(a, b, rtol=1e-5):
    for k in ("n", "F", "S"):
        scale = np.maximum(np.abs(b[k]), 1.0)
        assert np.all(np.abs(a[k] - b[k]) <= rtol * scale), (k, np.abs(a[k] - b[k]).max())


def test_loglikes_example(dev, golden):
    g = golden("example.npz")
    dev.upload_model(g["w"], g["mu"], g["var"])
    dev.upload_features(g["X"])
    ll = dev.loglikes()
    ref = g["ll_ref"]
    assert np.all(np.abs(ll - ref) <= 2e-5 + 2e-6 * np.abs(ref))
    assert np.abs(ll - g["ll_file"]).max() < 1e-4


def test_stats_example(dev, golden):
    g = golden("example.npz")
    dev.upload_model(g["w"], g["mu"], g["var"])
    dev.upload_features(g["X"])
    s = dev.accumulate()
    close_stats(s, dict(n=g["n4"], F=g["F4"], S=g["S4"]))
    assert abs(s["totLL"] - g["totLL4"]) <= 1e-6 * abs(g["totLL4"])
    assert s["totN"] == 1000


@pytest.mark.parametrize("flags", [1, 2, 3, 4])
def test_stats_flags(dev, golden, oracle, flags):
    g = golden("em_small.npz")
    dev.upload_model(g["w"], g["mu"], g["var"])
    dev.upload_features(g["X"])
    s = dev.accumulate(flags)
    o = oracle.accumulate32(g["X"], g["w"], g["mu"], g["var"], flags=flags, threads=1)
    close_stats(s, o)


def test_em_three_iterations_match_reference(dev, golden):
    g = golden("em_small.npz")
    dev.upload_model(g["w"], g["mu"], g["var"])
    dev.upload_features(g["X"])
    ll, alive = dev.em_iterate(3)
    assert np.all(np.abs(ll - g["em_ll"]) <= 1e-6 * np.abs(g["em_ll"]))
    w, mu, var = dev.read_model()
    assert np.allclose(w, g["em_w"], rtol=1e-4, atol=1e-7)
    assert np.allclose(mu, g["em_mu"], rtol=1e-4, atol=1e-5)
    assert np.allclose(var, g["em_var"], rtol=1e-4, atol=1e-6)
    assert alive == 16


def test_em_update_bit_exact_given_stats(dev, golden, oracle):
    """The device M-step reproduces the reference's float/double update exactly."""
    g = golden("em_small.npz")
    dev.upload_model(g["w"], g["mu"], g["var"])
    dev.upload_features(g["X"])
    dev.accumulate_device(3)
    s = dev.read_stats()
    alive = dev.em_update(True, True, True)
    w, mu, var = dev.read_model()
    ow, omu, ovar, oalive = oracle.em_update(g["w"], g["mu"], g["var"], s)
    assert alive == oalive
    assert np.array_equal(w, ow) and np.array_equal(mu, omu) and np.array_equal(var, ovar)


def test_edge_cases(dev, golden, oracle):
    from gmm_gb300 import synth
    e = golden("edge.npz")
    # zero-weight components are skipped in place
    dev.upload_model(e["zw_w"], e["zw_mu"], e["zw_var"])
    dev.upload_features(e["zw_X"])
    s = dev.accumulate()
    order = e["zw_order"]
    close_stats(dict(n=s["n"][order], F=s["F"][order], S=s["S"][order]),
                dict(n=e["zw_n"], F=e["zw_F"], S=e["zw_S"]))
    assert s["n"][1] == 0 and s["n"][5] == 0
    # single component
    dev.upload_model(np.ones(1, np.float32), e["zw_mu"][:1], e["zw_var"][:1])
    s = dev.accumulate()
    close_stats(s, dict(n=e["m1_n"], F=e["m1_F"], S=e["m1_S"]))
    w, mu, var = synth.generator_gmm(21, 8, 6)
    # N = 50
    dev.upload_model(w, mu, var)
    dev.upload_features(e["zw_X"][:50])
    s = dev.accumulate()
    close_stats(s, dict(n=e["n50_n"], F=e["n50_F"], S=e["n50_S"]))
    # outlier frame
    dev.upload_features(e["out_X"])
    s = dev.accumulate()
    assert s["totLL"] == pytest.approx(float(e["out_totLL"]), rel=1e-12)
    ll = dev.loglikes()
    assert ll[17] == np.float32(-1e20)
    # D = 1
    dev.upload_model(w, mu[:, :1], var[:, :1])
    dev.upload_features(e["zw_X"][:, :1])
    s = dev.accumulate()
    close_stats(s, dict(n=e["d1_n"], F=e["d1_F"], S=e["d1_S"]))
    # EM kills an under-occupied component; model comes back in the reference's order
    dev.upload_model(e["kill_w0"], e["kill_mu0"], e["kill_var0"])
    dev.upload_features(e["kill_X"])
    ll, _ = dev.em_iterate(2)
    assert np.allclose(ll, e["kill_ll"], rtol=1e-6)
    w2, mu2, var2 = dev.read_model()
    assert np.array_equal(w2 == 0, e["kill_w"] == 0)
    assert np.allclose(mu2, e["kill_mu"], rtol=1e-4, atol=1e-5)
    assert var2[-1].view(np.uint32)[0] == 0x01010101


def test_low_variance_rejected(dev, golden, glib):
    g = golden("em_small.npz")
    var = g["var"].copy()
    var[2, 7] = 1e-7
    with pytest.raises(glib.GMMError) as ei:
        dev.upload_model(g["w"], g["mu"], var)
    assert ei.value.code == glib.ERR_MODEL


def test_map_and_mllr_match_reference(dev, golden):
    g = golden("map_mllr.npz")
    dev.upload_model(g["w"], g["mu"], g["var"])
    dev.set_prior(g["w"], g["mu"], g["var"])
    dev.upload_features(g["X"])
    dev.accumulate_device(1)
    for init, W_ref in ((False, g["mllr_W0"]), (True, g["mllr_W1"])):
        W = dev.mllr_estimate(init)
        assert np.allclose(W, W_ref, rtol=1e-5, atol=1e-6)
    dev.map_update(16, False, True, False)
    w, mu, var = dev.read_model()
    assert np.allclose(mu, g["map_mu"], rtol=1e-5, atol=1e-6)
    assert np.array_equal(w, g["map_w"])
    dev.upload_model(g["w"], g["mu"], g["var"])
    dev.mllr_apply(g["mllr_W0"])
    _, mu2, _ = dev.read_model()
    assert np.allclose(mu2, g["mllr_mu0"], rtol=1e-6, atol=1e-6)


def test_c1_full_size_against_port(dev, oracle):
    """Config C1 at full size (100k frames, M = 64, D = 39): one E-step against the port."""
    from gmm_gb300 import synth
    X, w, mu, var = synth.c1(seed=1)
    dev.upload_model(w, mu, var)
    dev.upload_features(X)
    s = dev.accumulate()
    o = oracle.accumulate32(X, w, mu, var, threads=8)
    assert abs(s["totLL"] - o["totLL"]) <= 1e-6 * abs(o["totLL"])
    close_stats(s, o)
    # size-independent property: the kept posterior mass never exceeds the frame count
    assert s["n"].sum() <= len(X) * (1 + 1e-9)


def test_estimator_mirror(glib, golden):
    from gmm_gb300 import formats
    from gmm_gb300.estimator import GMMStats, GMMStatsEstimatorGB300
    g = golden("edge.npz")
    est = GMMStatsEstimatorGB300()
    model = formats.GMModel(g["zw_w"], g["zw_mu"], g["zw_var"])
    est.insertModel(model)
    assert model.w[-1] == 0 and model.w[-2] == 0   # moved behind the others, like the reference
    st = GMMStats()
    est.setAccFlags(False, True, True)
    X = g["zw_X"]
    est.accumulateStatsMT(X, len(X), X.shape[1], st)
    est.accumulateStatsMT(X, len(X), X.shape[1], st)   # += semantics
    assert np.allclose(st.n, 2 * g["zw_n"], rtol=1e-5)
    assert st.getTotAccSamples() == 2 * len(X)
    ll = est.compVecsLogLikeMT(X, len(X), X.shape[1])
    assert ll.shape == (len(X),)
