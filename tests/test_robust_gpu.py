"""--robust on the GPU (gmm_set_robust) against the reference build (tests/golden/robust.npz).

Tolerances, written per check:
  auxiliary statistics, diagonal model   within 1e-7 of each statistic's scale (the same float
                                         posteriors and products; FP64 sums in another order)
  auxiliary statistics, full model       within 2e-5 of the scale (the device's log-likelihood
                                         arithmetic differs from the reference's float inverse)
  robust EM (2 iterations) / MAP         rel 1e-4, abs 1e-5 of the reference's models
  tensor-core precision mode             the same results as the plain mode (robust E-steps
                                         run on the plain kernels)
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def close(a, b, rel):
    return np.abs(a - b).max() <= rel * max(np.abs(b).max(), 1e-30)


def test_aux_statistics(glib, golden):
    r = golden("robust.npz")
    e = golden("em_small.npz")
    f = golden("full.npz")
    h = glib.Handle(0)
    h.set_robust(True)
    h.upload_model(e["w"], e["mu"], e["var"])
    h.upload_features(e["X"])
    h.accumulate()
    a = h.read_aux()
    for k in ("aux", "aux2", "aux3"):
        assert close(a[k], r[f"diag_{k}"], 1e-7), k
    h.upload_model_full(f["w"], f["mu"], f["cov"])
    h.upload_features(f["X"])
    h.accumulate_full()
    a = h.read_aux(full=True)
    for k in ("aux", "aux2", "aux3"):
        assert close(a[k], r[f"full_{k}"], 2e-5), k
    h.close()


@pytest.mark.parametrize("prec", ["PREC_FP32", "PREC_TC"])
def test_robust_em_and_map(glib, golden, prec):
    from gmm_gb300 import adapt, formats
    r = golden("robust.npz")
    e = golden("em_small.npz")
    f = golden("full.npz")
    mm = golden("map_mllr.npz")
    P = getattr(glib, prec)
    for key, X, model in (("diag", e["X"], formats.GMModel(e["w"], e["mu"], e["var"])),
                          ("full", f["X"], formats.GMModel(f["w"], f["mu"], f["cov"]))):
        ma = adapt.ModelAdapt(adapt.Options(adaptType=adapt.MAP, tau=0, iterCountEM=2, AdaptWeightBool=True,
                                            AdaptMeanBool=True, AdaptVarBool=True, robustCov=True, precision=P))
        ma.InsertData(X)
        ma.AdaptModel(model)
        m = ma.PickUpClientModel()
        vkey = "cov" if key == "full" else "var"
        assert np.allclose(m.w, r[f"{key}_em_w"], rtol=1e-4, atol=1e-5), key
        assert np.allclose(m.mu, r[f"{key}_em_mu"], rtol=1e-4, atol=1e-5), key
        assert np.allclose(m.var, r[f"{key}_em_{vkey}"], rtol=1e-4, atol=1e-5), key
    ma = adapt.ModelAdapt(adapt.Options(adaptType=adapt.MAP, tau=16, iterCountMAP=1, AdaptMeanBool=True,
                                        AdaptVarBool=True, robustCov=True, precision=P))
    ma.InsertData(mm["X"])
    ma.AdaptModel(formats.GMModel(mm["w"], mm["mu"], mm["var"]))
    m = ma.PickUpClientModel()
    assert np.allclose(m.mu, r["map_mu"], rtol=1e-4, atol=1e-5)
    assert np.allclose(m.var, r["map_var"], rtol=1e-4, atol=1e-5)


def test_command_line_robust(glib, golden, tmp_path):
    from gmm_gb300 import build, formats
    r = golden("robust.npz")
    e = golden("em_small.npz")
    feat = tmp_path / "x.raw"
    formats.write_raw(str(feat), e["X"])
    ubm = tmp_path / "ubm.gmm"
    formats.write_gmm_bin(str(ubm), formats.GMModel(e["w"], e["mu"], e["var"]))
    rr = subprocess.run([os.path.join(build.OUT_DIR, "gmm_adapt"), "-i", str(feat), "--data-T", "2", "-u", str(ubm),
                         "-o", str(tmp_path / "em.gmm"), "--it-EM", "2", "-W", "-M", "-V", "-R", "--precision",
                         "fp32"], capture_output=True, text=True, timeout=300)
    assert rr.returncode == 0, rr.stdout + rr.stderr
    m = formats.read_gmm_bin(str(tmp_path / "em.gmm"))
    keep = r["diag_em_w"] > 0
    assert np.allclose(m.mu, r["diag_em_mu"][keep], rtol=1e-4, atol=1e-5)
    assert np.allclose(m.var, r["diag_em_var"][keep], rtol=1e-4, atol=1e-5)
