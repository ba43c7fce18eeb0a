"""File-by-file accumulation (gmm_accumulate_files) against one E-step over the same frames.

Batches are accumulated one after another into the same FP64 statistics, so the result equals
the E-step over the concatenated frames up to the grouping of the sums:
  plain FP32 path   n, F, S and total LL within 1e-12 relative (FP64 sums of identical float
                    products, grouped by batch)
  tensor-core path  within 1e-6 of each statistic's scale (FP32 tile sums grouped by batch)
A missing file and an empty file are skipped, as the reference does.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def write_files(tmp_path, kind, lens, D, seed=3):
    from gmm_gb300 import formats, synth
    w, mu, var = synth.generator_gmm(seed, 32, D)
    paths, blocks = [], []
    for i, n in enumerate(lens):
        X = synth.sample_gmm(seed * 10 + i, w, mu, var, n) if n else np.zeros((0, D), np.float32)
        p = str(tmp_path / f"f{i}.{kind}")
        {"sves": formats.write_sves, "htk": formats.write_htk, "raw": formats.write_raw}[kind](p, X)
        paths.append(p)
        blocks.append(X)
    return paths, np.concatenate(blocks), (w, mu, var)


@pytest.mark.parametrize("prec_name", ["PREC_FP32", "PREC_TC"])
@pytest.mark.parametrize("kind,prm", [("sves", 0), ("htk", 1), ("raw", 2)])
def test_files_equal_one_shot(glib, tmp_path, prec_name, kind, prm):
    D = 20
    paths, X, model = write_files(tmp_path, kind, [500, 1200, 0, 64, 3000, 777], D)
    paths.insert(2, str(tmp_path / "missing.prm"))
    h = glib.Handle(0)
    h.set_precision(getattr(glib, prec_name))
    h.upload_model(*model)
    used = h.accumulate_files(paths, prm, dwnsmp=1, buffer_gb=2e3 * D * 4 / 2**30)  # ~2000-frame batches
    st = h.read_stats()
    h.upload_features(X)
    ref = h.accumulate()
    h.close()
    assert used == 5 and st["totN"] == len(X)
    tol = 1e-12 if prec_name == "PREC_FP32" else 1e-6
    assert abs(st["totLL"] - ref["totLL"]) <= tol * abs(ref["totLL"])
    for k in ("n", "F", "S"):
        scale = np.abs(ref[k]) + (np.abs(ref["n"])[:, None] if k != "n" else 0) + 1.0
        assert np.max(np.abs(st[k] - ref[k]) / scale) <= tol, k


def test_files_small_batches_and_downsampling(glib, tmp_path):
    D = 12
    paths, X, model = write_files(tmp_path, "htk", [300, 301, 302, 303], D, seed=9)
    h = glib.Handle(0)
    h.upload_model(*model)
    h.accumulate_files(paths, glib.PRM_HTK, dwnsmp=3, buffer_gb=1e-7)  # one batch per file
    st = h.read_stats()
    Xd = np.concatenate([X[0:300][::3], X[300:601][::3], X[601:903][::3], X[903:1206][::3]])
    h.upload_features(Xd)
    ref = h.accumulate()
    h.close()
    assert st["totN"] == len(Xd)
    assert abs(st["totLL"] - ref["totLL"]) <= 1e-12 * abs(ref["totLL"])
    assert np.allclose(st["S"], ref["S"], rtol=1e-12, atol=1e-9)


def test_files_dimension_mismatch(glib, tmp_path):
    from gmm_gb300 import formats
    paths, X, model = write_files(tmp_path, "raw", [100], 8)
    h = glib.Handle(0)
    h.upload_model(*model)
    bad = str(tmp_path / "bad.raw")
    formats.write_raw(bad, np.zeros((10, 9), np.float32))
    with pytest.raises(glib.GMMError) as e:
        h.accumulate_files(paths + [bad], glib.PRM_RAW)
    assert e.value.code == glib.ERR_ARG
    h.close()
