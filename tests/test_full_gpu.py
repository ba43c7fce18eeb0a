"""Full-covariance models on the GPU (gmm_*_full) against the reference build and the FP64 oracle.

tests/golden/full.npz holds the reference's outputs (make_golden.py full_fixture; the reference's
single-precision Cholesky / inverse go through the restated LAPACK routines of
oracle/ref/shim/acml.h). The device factors each covariance in FP64 and evaluates
|L^-1 (x - mu)|^2 with FP32 fused multiply-adds, so it sits closer to the FP64 oracle than the
reference's float inverse does. Tolerances, written per check:
  per-frame LL         vs FP64 oracle  |d| <= 2e-5 + 1e-6 |ll|;  vs reference |d| <= 1e-4
  statistics n, F, S   vs FP64 oracle  within 2e-5 of each statistic's scale (posterior
                       differences of ~1e-5 relative), total LL 1e-6 rel
  EM (3 iterations) / MAP (tau 16)  vs reference  rel 1e-4, abs 1e-5 (weights, means,
                       covariances)
  edge cases: zero-weight components skipped (their statistics 0), one component (posterior 1),
  D = 1, D = 60, an outlier frame (LL = minLogLike), a covariance that is not positive definite
  (GMM_ERR_MODEL)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def close_stats(a, b, rel=2e-5):
    for k in ("n", "F", "Sp"):
        scale = max(np.abs(b[k]).max(), 1e-30)
        assert np.abs(a[k] - b[k]).max() <= rel * scale, (k, np.abs(a[k] - b[k]).max() / scale)
    assert abs(a["totLL"] - b["totLL"]) <= 1e-6 * abs(b["totLL"])


def check_ll(ll, ref64):
    assert np.all(np.abs(ll - ref64) <= 2e-5 + 1e-6 * np.abs(ref64)), np.abs(ll - ref64).max()


def test_example_model_loglikes_and_stats(dev, golden, oracle):
    g = golden("full.npz")
    dev.upload_model_full(g["ex_w"], g["ex_mu"], g["ex_cov"])
    dev.upload_features(g["ex_X"])
    ll = dev.loglikes_full()
    check_ll(ll, oracle.full64_loglikes(g["ex_X"], g["ex_w"], g["ex_mu"], g["ex_cov"]))
    assert np.abs(ll - g["ex_ll"]).max() < 1e-4
    st = dev.accumulate_full()
    close_stats(st, oracle.full64_accumulate(g["ex_X"], g["ex_w"], g["ex_mu"], g["ex_cov"]))
    close_stats(st, dict(n=g["ex_n"], F=g["ex_F"], Sp=g["ex_Sp"], totLL=g["ex_totLL"]))
    assert st["totN"] == 1000


@pytest.mark.parametrize("flags", [1, 2, 3, 4])
def test_flags(dev, golden, oracle, flags):
    g = golden("full.npz")
    dev.upload_model_full(g["w"], g["mu"], g["cov"])
    dev.upload_features(g["X"])
    st = dev.accumulate_full(flags)
    ref = oracle.full64_accumulate(g["X"], g["w"], g["mu"], g["cov"], flags=flags)
    close_stats(st, ref)
    if flags & 4 or not flags & 2:
        assert not st["Sp"].any()
    if flags == 4 or flags == 2:
        assert not st["F"].any()


def test_em_and_map_match_reference(glib, golden):
    from gmm_gb300 import adapt, formats
    g = golden("full.npz")
    ubm = formats.GMModel(g["w"], g["mu"], g["cov"])
    ma = adapt.ModelAdapt(adapt.Options(adaptType=adapt.MAP, tau=0, iterCountEM=3, AdaptWeightBool=True,
                                        AdaptMeanBool=True, AdaptVarBool=True))
    ma.InsertData(g["X"])
    ma.AdaptModel(ubm)
    m = ma.PickUpClientModel()
    assert np.allclose(ma.ll_history, g["em_ll"], rtol=1e-6)
    assert np.allclose(m.w, g["em_w"], rtol=1e-4, atol=1e-5)
    assert np.allclose(m.mu, g["em_mu"], rtol=1e-4, atol=1e-5)
    assert np.allclose(m.var, g["em_cov"], rtol=1e-4, atol=1e-5)
    ma = adapt.ModelAdapt(adapt.Options(adaptType=adapt.MAP, tau=16, iterCountMAP=1, AdaptWeightBool=True,
                                        AdaptMeanBool=True, AdaptVarBool=True))
    ma.InsertData(g["X"])
    ma.AdaptModel(formats.GMModel(g["w"], g["mu"], g["cov"]))
    m = ma.PickUpClientModel()
    assert np.allclose(m.w, g["map_w"], rtol=1e-4, atol=1e-5)
    assert np.allclose(m.mu, g["map_mu"], rtol=1e-4, atol=1e-5)
    assert np.allclose(m.var, g["map_cov"], rtol=1e-4, atol=1e-5)


def test_update_kernels_given_statistics(dev, golden, oracle):
    """EM and MAP updates on the device against the reference's expressions (oracle port) for
    the same statistics: within one float rounding of the outputs."""
    g = golden("full.npz")
    dev.upload_model_full(g["w"], g["mu"], g["cov"])
    dev.set_prior_full()
    dev.upload_features(g["X"])
    dev.accumulate_full_device(3)
    st = dev.read_stats_full()
    alive = dev.em_update_full(True, True, True)
    w, mu, cov = dev.read_model_full()
    ow, omu, ocov, oalive = oracle.full_em_update(g["w"], g["mu"], g["cov"], st)
    assert alive == oalive
    assert np.allclose(w, ow, rtol=2e-7) and np.allclose(mu, omu, rtol=2e-7, atol=1e-7)
    assert np.allclose(cov, ocov, rtol=2e-7, atol=1e-7)
    dev.upload_model_full(g["w"], g["mu"], g["cov"])
    dev.accumulate_full_device(3)
    st = dev.read_stats_full()
    dev.map_update_full(16, True, True, True)
    w, mu, cov = dev.read_model_full()
    ow, omu, ocov = oracle.full_map_update(g["w"], g["mu"], g["cov"], st, 16, True, True, True)
    assert np.allclose(w, ow, rtol=2e-7) and np.allclose(mu, omu, rtol=2e-7, atol=1e-7)
    assert np.allclose(cov, ocov, rtol=2e-7, atol=1e-7)


@pytest.mark.parametrize("M,D,N", [(1, 5, 700), (5, 1, 900), (8, 60, 2000), (33, 24, 3000), (6, 8, 300_000)])
def test_shapes_against_oracle(dev, oracle, M, D, N):
    from gmm_gb300 import synth
    w, mu, cov = synth.generator_gmm_full(100 + D, M, D)
    X = synth.sample_gmm_full(200 + M, w, mu, cov, N)
    if M > 4:
        w[3] = 0.0  # skipped, as after GMModel::RearrangeMixtures
        w /= w.sum()
    dev.upload_model_full(w, mu, cov)
    dev.upload_features(X)
    check_ll(dev.loglikes_full(), oracle.full64_loglikes(X, w, mu, cov))
    st = dev.accumulate_full()
    close_stats(st, oracle.full64_accumulate(X, w, mu, cov))
    if M == 1:
        assert st["n"][0] == N
    if M > 4:
        assert st["n"][3] == 0 and not st["Sp"][3].any()


def test_outlier_and_bad_covariance(dev, glib, golden):
    g = golden("full.npz")
    X = g["X"][:300].copy()
    X[17] = 1e19
    dev.upload_model_full(g["w"], g["mu"], g["cov"])
    dev.upload_features(X)
    ll = dev.loglikes_full()
    assert ll[17] == np.float32(-1e20) and np.isfinite(ll[:17]).all()
    cov = g["cov"].copy()
    cov[2, 0, 1] = cov[2, 1, 0] = 10.0 * np.sqrt(cov[2, 0, 0] * cov[2, 1, 1])  # not positive definite
    with pytest.raises(glib.GMMError) as e:
        dev.upload_model_full(g["w"], g["mu"], cov)
    assert e.value.code == glib.ERR_MODEL


def test_estimator_interface(glib, golden, oracle):
    from gmm_gb300 import estimator, formats
    g = golden("full.npz")
    est = estimator.GMMStatsEstimatorGB300()
    model = formats.GMModel(g["ex_w"], g["ex_mu"], g["ex_cov"])
    est.insertModel(model)
    est.setAccFlags(False, True, True, True)
    st = estimator.GMMStats()
    est.accumulateStatsMT(g["ex_X"], 1000, 20, st)
    est.accumulateStatsMT(g["ex_X"], 1000, 20, st)
    assert st.hasFullCov() and st.S.shape == (4, 210)
    assert np.abs(st.S - 2 * g["ex_Sp"]).max() <= 2e-5 * np.abs(2 * g["ex_Sp"]).max()
    ll = est.compVecsLogLikeMT(g["ex_X"], 1000, 20)
    assert np.abs(ll - g["ex_ll"]).max() < 1e-4


@pytest.mark.parametrize("init", [False, True])
def test_mllr_of_full_model(glib, golden, init):
    """MLLR of a full-covariance UBM (the covariance diagonals in G and k) against the reference
    build (tests/golden/full_mllr.npz): W within 1e-4 abs (the E-step's LL arithmetic differs at
    ~1e-6), transformed means within 1e-4."""
    from gmm_gb300 import adapt, formats
    g = golden("full_mllr.npz")
    ma = adapt.ModelAdapt(adapt.Options(adaptType=adapt.MLLR, mllrUBMInit=init, applyTransforms=True))
    ma.InsertData(g["X"])
    ma.AdaptModel(formats.GMModel(g["w"], g["mu"], g["cov"]))
    key = "1" if init else "0"
    W = ma.PickUpTRNMatrix()
    assert np.abs(W - g[f"W{key}"]).max() < 1e-4, np.abs(W - g[f"W{key}"]).max()
    m = ma.PickUpClientModel()
    assert m.full and np.abs(m.mu - g[f"mu{key}"]).max() < 1e-4
    assert np.array_equal(m.var, g["cov"])


def test_fmllr_of_full_model(glib, golden):
    """fMLLR of a full-covariance UBM (full E-step statistics, covariance diagonals in G and k)
    against the reference build: W within 1e-4 abs."""
    from gmm_gb300 import adapt, formats
    g = golden("full_mllr.npz")
    ma = adapt.ModelAdapt(adapt.Options(adaptType=adapt.FMLLR))
    ma.InsertData(g["X"])
    ma.AdaptModel(formats.GMModel(g["w"], g["mu"], g["cov"]))
    W = ma.PickUpTRNMatrix()
    assert np.abs(W - g["fW"]).max() < 1e-4, np.abs(W - g["fW"]).max()
