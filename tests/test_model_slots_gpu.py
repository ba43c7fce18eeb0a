"""Device-resident model groups: gmm_upload_model_slot / gmm_select_model / gmm_clear_model_slots.

The reference keeps the precomputed terms of every model inserted with insertModel(model,
first = false) and switches between them with setModelToBeUsed (OL_GMMStatsEstimator.cpp:234-325).
Here the models of a group stay in device memory and a switch is a device-to-device copy. A
switch must give exactly what uploading that model from the host gives (bit-identical
statistics and log-likelihoods, plain FP32 and tensor-core paths)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _models(D=39):
    from gmm_gb300 import synth
    X, w0, mu0, var0 = synth.config_em(501, 4000, D, 8, 32)
    _, w1, mu1, var1 = synth.config_em(502, 4000, D, 8, 32)
    _, w2, mu2, var2 = synth.config_em(503, 4000, D, 8, 64)
    w1 = w1.copy()
    w1[3] = 0.0  # a zero-weight component (skipped by the E-step)
    w1 /= w1.sum()
    return X, [(w0, mu0, var0), (w1, mu1, var1), (w2, mu2, var2)]


@pytest.mark.parametrize("prec", ["fp32", "tc"])
def test_select_equals_upload(glib, prec):
    X, models = _models()
    mode = glib.PREC_TC if prec == "tc" else glib.PREC_FP32
    h = glib.Handle(0)
    h.set_precision(mode)
    h.set_autotune(False)
    h.upload_features(X)
    for i, m in enumerate(models):
        h.upload_model_slot(i, *m)
    ref = glib.Handle(0)
    ref.set_precision(mode)
    ref.set_autotune(False)
    ref.upload_features(X)
    for n in (1, 0, 2, 1):
        h.select_model(n)
        ref.upload_model(*models[n])
        a, b = h.accumulate(), ref.accumulate()
        assert a["totLL"] == b["totLL"]
        for k in ("n", "F", "S"):
            assert np.array_equal(a[k], b[k]), (n, k)
        assert np.array_equal(h.loglikes(), ref.loglikes())
    h.close()
    ref.close()


def test_slot_errors(glib):
    X, models = _models()
    h = glib.Handle(0)
    h.upload_model_slot(0, *models[0])
    with pytest.raises(glib.GMMError) as e:
        h.select_model(1)  # empty slot
    assert e.value.code == glib.ERR_ARG
    w, mu, var = models[0]
    with pytest.raises(glib.GMMError) as e:  # another dimension in the same group
        h.upload_model_slot(1, w, mu[:, :20], var[:, :20])
    assert e.value.code == glib.ERR_ARG
    bad = var.copy()
    bad[2, 5] = 1e-9  # below min_var: the check runs when the slot is selected
    h.upload_model_slot(2, w, mu, bad)
    with pytest.raises(glib.GMMError):
        h.select_model(2)
    h.clear_model_slots()
    with pytest.raises(glib.GMMError):
        h.select_model(0)
    h.close()


def test_estimator_group_switch(glib):
    """The Python mirror of the estimator: insertModel(first = False) keeps the group on the
    device; setModelToBeUsed(n) switches without a host upload."""
    from gmm_gb300 import formats
    from gmm_gb300.estimator import GMMStats, GMMStatsEstimatorGB300
    X, models = _models()
    est = GMMStatsEstimatorGB300()
    for i, m in enumerate(models):
        est.insertModel(formats.GMModel(*m), first=(i == 0))
    got = []
    for n in (0, 2, 1):
        est.setModelToBeUsed(n)
        st = GMMStats()
        est.setAccFlags(False, True, True)
        est.accumulateStatsMT(X, len(X), X.shape[1], st)
        got.append((n, st))
    for n, st in got:
        h = glib.Handle(0)
        g = formats.GMModel(*models[n])
        g.rearrange()
        h.upload_model(g.w, g.mu, g.var)
        h.upload_features(X)
        r = h.accumulate()
        h.close()
        assert np.array_equal(st.n, r["n"]), n
