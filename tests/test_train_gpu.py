"""Train from scratch (ModelAdapt.TrainFromScratch) against the reference's TrainFromScratch.

tests/golden/train.npz holds the reference build's models (make_golden.py): one split per
round, several splits per round (--split-X 0.5 --split-th 0.2), and the log-likelihood stop rule
(--ll-Th 0.01), quiet and verbose (the reference only tracks the likelihood when verbose, which
changes where it stops). The plain FP32 path reproduces the reference's E-step and M-step to
~1e-6 per iteration; after the rounds of EM and splitting the models agree within
  weights, means   1e-4 absolute + 1e-4 relative
  variances        1e-4 relative
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {"one": dict(nummix=6, iters_em=3),
         "multi": dict(nummix=8, iters_em=3, split_x=0.5, split_th=0.2),
         "llth_quiet": dict(nummix=8, iters_em=2, ll_th=0.01, verbosity=0),
         "llth_verbose": dict(nummix=8, iters_em=2, ll_th=0.01, verbosity=1)}


@pytest.mark.parametrize("name", list(CASES))
def test_train_from_scratch_matches_reference(glib, golden, name):
    from gmm_gb300 import adapt
    g = golden("train.npz")
    kw = CASES[name]
    opt = adapt.Options(adaptType=adapt.FROM_SCRATCH, iterCountEM=kw["iters_em"],
                        splitXpercAtOnce=kw.get("split_x", 0.0), splitTh=kw.get("split_th", 0.0),
                        llTh=kw.get("ll_th", 0.0), verbosity=kw.get("verbosity", 0))
    ma = adapt.ModelAdapt(opt)
    ma.InsertData(g["X"])
    model = ma.TrainFromScratch(kw["nummix"])
    w, mu, var = g[f"{name}_w"], g[f"{name}_mu"], g[f"{name}_var"]
    assert np.array_equal(model.w > 0, w > 0), (model.w, w)
    alive = w > 0
    assert np.allclose(model.w, w, rtol=1e-4, atol=1e-4), np.abs(model.w - w).max()
    assert np.allclose(model.mu[alive], mu[alive], rtol=1e-4, atol=1e-4), np.abs(model.mu - mu)[alive].max()
    assert np.allclose(model.var[alive], var[alive], rtol=1e-4), (np.abs(model.var - var)[alive] / var[alive]).max()


@pytest.mark.parametrize("name", ["one", "multi"])
def test_train_full_covariance_matches_reference(glib, golden, name):
    """Full covariances: splits along the leading eigenvector (sign: largest component positive,
    the convention of the reference build's restated ssyevr). Weights / means 1e-4 abs + rel,
    covariances 1e-4 abs + rel."""
    from gmm_gb300 import adapt
    g = golden("train_full.npz")
    kw = {"one": dict(nummix=4, iters_em=3), "multi": dict(nummix=6, iters_em=3, split_x=0.5, split_th=0.2)}[name]
    opt = adapt.Options(adaptType=adapt.FROM_SCRATCH, iterCountEM=kw["iters_em"],
                        splitXpercAtOnce=kw.get("split_x", 0.0), splitTh=kw.get("split_th", 0.0))
    ma = adapt.ModelAdapt(opt)
    ma.InsertData(g["X"])
    model = ma.TrainFromScratch(kw["nummix"], fullcov=True)
    assert model.full
    w, mu, cov = g[f"{name}_w"], g[f"{name}_mu"], g[f"{name}_cov"]
    assert np.array_equal(model.w > 0, w > 0)
    alive = w > 0
    assert np.allclose(model.w, w, rtol=1e-4, atol=1e-4)
    assert np.allclose(model.mu[alive], mu[alive], rtol=1e-4, atol=1e-4)
    assert np.allclose(model.var[alive], cov[alive], rtol=1e-4, atol=1e-4)
