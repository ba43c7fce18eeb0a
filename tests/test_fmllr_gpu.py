"""fMLLR on the GPU (gmm_fmllr_estimate / gmm_fmllr_apply) against the reference build.

tests/golden/fmllr.npz holds the reference's transform (ComputeW_fMLLR, 20 passes) and the
statistics it used. The device E-step keeps the reference's float log-likelihoods and products;
its statistics are summed in double-float instead of double, and the FP64 row passes follow the
reference's loop orders with explicit rounding. Tolerances, written per check:
  W vs the reference          |d| <= 1e-6
  W vs the oracle port fed the reference's statistics   |d| <= 1e-6
  gmm_fmllr_apply             x' = A x + b within 1e-6 relative (FP64 sums, float output)
  command line --type 3       the " fMLLR" file's %g values within 1e-5 relative + 1e-6
  too few components          GMM_ERR_MLLR (CheckInvertibility)
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_transform_matches_reference(dev, golden, oracle):
    g = golden("fmllr.npz")
    dev.upload_model(g["w"], g["mu"], g["var"])
    dev.upload_features(g["X"])
    W = dev.fmllr_estimate(20)
    assert np.abs(W - g["W"]).max() <= 1e-6, np.abs(W - g["W"]).max()
    Wo = oracle.fmllr_w(g["mu"], g["var"], dict(n=g["n"], F=g["F"], Sp=g["Sp"], totN=len(g["X"])))
    assert np.abs(W - Wo).max() <= 1e-6


@pytest.mark.parametrize("prec", ["PREC_FP32", "PREC_TC"])
def test_apply_and_precision_modes(glib, golden, prec):
    g = golden("fmllr.npz")
    h = glib.Handle(0)
    h.set_precision(getattr(glib, prec))  # the fMLLR E-step is the plain path in both modes
    h.upload_model(g["w"], g["mu"], g["var"])
    h.upload_features(g["X"])
    W = h.fmllr_estimate(20)
    assert np.abs(W - g["W"]).max() <= 1e-6
    h.fmllr_apply(W)
    # read the transformed frames back through a 1-component model's statistics: F = sum x'
    h.upload_model(np.ones(1, np.float32), np.zeros((1, g["X"].shape[1]), np.float32),
                   np.ones((1, g["X"].shape[1]), np.float32))
    st = h.accumulate(glib.ACC_MEAN)
    h.close()
    Xt = g["X"].astype(np.float64) @ W[:, :-1].T + W[:, -1]
    assert np.allclose(st["F"][0], Xt.sum(0), rtol=1e-6, atol=1e-3)


def test_model_adapt_and_command_line(glib, golden, tmp_path):
    from gmm_gb300 import adapt, build, formats
    g = golden("fmllr.npz")
    ma = adapt.ModelAdapt(adapt.Options(adaptType=adapt.FMLLR))
    ma.InsertData(g["X"])
    ma.AdaptModel(formats.GMModel(g["w"], g["mu"], g["var"]))
    assert np.abs(ma.PickUpTRNMatrix() - g["W"]).max() <= 1e-6
    feat = tmp_path / "spk.prm"
    formats.write_sves(str(feat), g["X"])
    ubm = tmp_path / "ubm.gmm"
    formats.write_gmm_bin(str(ubm), formats.GMModel(g["w"], g["mu"], g["var"]))
    r = subprocess.run([os.path.join(build.OUT_DIR, "gmm_adapt"), "-i", str(feat), "-u", str(ubm), "-o",
                        str(tmp_path / "spk.gmm"), "-t", "3"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    text = (tmp_path / "spk.mat").read_text()
    assert text.startswith(" fMLLR\n 1\t12 13\n")
    W = formats.read_trn(str(tmp_path / "spk.mat"))
    assert np.allclose(W, g["W"], rtol=1e-5, atol=1e-6)
    assert not (tmp_path / "spk.gmm").exists()


def test_invertibility_check(dev, glib, golden):
    g = golden("fmllr.npz")
    dev.upload_model(g["w"][:8] / g["w"][:8].sum(), g["mu"][:8], g["var"][:8])  # M = 8 < D + 1
    dev.upload_features(g["X"])
    with pytest.raises(glib.GMMError) as e:
        dev.fmllr_estimate(20)
    assert e.value.code == glib.ERR_MLLR


def test_mllr_map_matches_reference(glib, golden, tmp_path):
    """MLLR+MAP (--type 4): the MLLR-transformed UBM, then one MAP iteration against the original
    UBM; against the reference's AdaptModel (tests/golden/mllr_map.npz): means rel 1e-5 / abs
    1e-5, variances rel 1e-4 / abs 1e-5, through the Python driver and the command line."""
    from gmm_gb300 import adapt, build, formats
    g = golden("map_mllr.npz")
    want = golden("mllr_map.npz")
    ma = adapt.ModelAdapt(adapt.Options(adaptType=adapt.MLLR_MAP, tau=16, iterCountMAP=1, AdaptMeanBool=True,
                                        AdaptVarBool=True))
    ma.InsertData(g["X"])
    ma.AdaptModel(formats.GMModel(g["w"], g["mu"], g["var"]))
    m = ma.PickUpClientModel()
    assert np.allclose(m.mu, want["mu"], rtol=1e-5, atol=1e-5)
    assert np.allclose(m.var, want["var"], rtol=1e-4, atol=1e-5)
    feat = tmp_path / "s.prm"
    formats.write_sves(str(feat), g["X"])
    ubm = tmp_path / "ubm.gmm"
    formats.write_gmm_bin(str(ubm), formats.GMModel(g["w"], g["mu"], g["var"]))
    r = subprocess.run([os.path.join(build.OUT_DIR, "gmm_adapt"), "-i", str(feat), "-u", str(ubm), "-o",
                        str(tmp_path / "s.gmm"), "-t", "4", "--it-MAP", "1", "-r", "16", "-M", "-V",
                        "--precision", "fp32"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    c = formats.read_gmm_bin(str(tmp_path / "s.gmm"))
    assert np.allclose(c.mu, want["mu"], rtol=1e-5, atol=1e-5)
    assert np.allclose(c.var, want["var"], rtol=1e-4, atol=1e-5)
