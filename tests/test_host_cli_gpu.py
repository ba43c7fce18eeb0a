"""The command lines gmm_adapt / gmm_loglike (C++ host layer over the C ABI) against the
reference's golden outputs and against the Python host API, on one GB300.

Tolerances, written per check (the plain FP32 path, --precision fp32, unless noted):
  gmm_loglike per-frame values  2e-5 + 2e-6 |ref| of the reference build's values (ll_ref), and
                                one unit of the 6th significant digit (<= 1.5e-5 rel) of the
                                reference's example/data.logL (both files hold %g values);
                                tensor-core path 1e-4 |ref| + 1e-4
  EM (3 iterations, W M V)      weights rel 1e-4 / atol 1e-7, means rel 1e-4 / atol 1e-5,
                                variances rel 1e-4 / atol 1e-6 of the reference's IterEM
  MAP (tau 16, means)           rel 1e-5 / atol 1e-6 of the reference's AdaptModelMAP
  MLLR transform file           rel 2e-5 / atol 2e-6 of the reference's W (the file holds 6
                                significant digits, as the reference's ostream output)
  train from scratch            weights / means 1e-4 abs + 1e-4 rel, variances 1e-4 rel
  modes (file-by-file, model-file, CLASS) equal the one-shot run within 1e-6 rel
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def exe(glib):
    from gmm_gb300 import build
    return lambda name: os.path.join(build.OUT_DIR, name)


def run(path, *args):
    r = subprocess.run([path, *map(str, args)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout, r.stderr)
    return r.stdout


def write_model(path, w, mu, var):
    from gmm_gb300 import formats
    formats.write_gmm_bin(str(path), formats.GMModel(w, mu, var))


def read_model(path):
    from gmm_gb300 import formats
    return formats.read_gmm_bin(str(path))


@pytest.mark.parametrize("prec", ["fp32", "tc"])
def test_loglike_for_each_matches_reference(exe, golden, tmp_path, prec):
    from gmm_gb300 import formats
    g = golden("example.npz")
    feat = tmp_path / "data.raw"
    formats.write_raw(str(feat), g["X"])
    mdl = tmp_path / "m.gmm"
    formats.write_gmm_txt(str(mdl), formats.GMModel(g["w"], g["mu"], g["var"]))
    out = tmp_path / "out"
    out.mkdir()
    run(exe("gmm_loglike"), "-i", feat, "-g", mdl, "-L", "--data-T", "2", "-f", "-o", out, "-T",
        "--precision", prec)
    text = (out / "data.logL").read_text()
    assert text.startswith("1 1000\n") and text.endswith(" \n\n")
    ll = formats.read_mat(str(out / "data.logL"), True)[0].astype(np.float64)
    ref = g["ll_ref"]
    if prec == "fp32":
        assert np.all(np.abs(ll - ref) <= 2e-5 + 2e-6 * np.abs(ref))
        assert np.all(np.abs(ll - g["ll_file"]) <= 1.5e-5 * np.abs(g["ll_file"]))
    else:
        assert np.all(np.abs(ll - ref) <= 1e-4 + 1e-4 * np.abs(ref))
    # binary saveMat and the mean-per-file mode
    run(exe("gmm_loglike"), "-i", feat, "-g", mdl, "-L", "--data-T", "2", "-f", "-o", out, "-x", ".bin",
        "--precision", prec)
    llb = formats.read_mat(str(out / "data.bin"), False)[0]
    assert np.allclose(llb, ll, rtol=1e-5, atol=1e-5)
    line = run(exe("gmm_loglike"), "-i", feat, "-g", mdl, "-L", "--data-T", "2", "--precision", prec)
    name, mean = line.strip("\r\n").split("\t")
    assert name == str(feat) and abs(float(mean) - ref.mean()) < 1e-3


def test_full_covariance_models(exe, golden, tmp_path):
    """gmm_loglike on the reference's example/myModelFC.gmm (text, full covariances) and gmm_adapt
    EM / MAP of a full-covariance model, against the reference build (tests/golden/full.npz);
    tolerances as tests/test_full_gpu.py (LL 1e-4 abs, models rel 1e-4 / abs 1e-5)."""
    from gmm_gb300 import formats
    g = golden("full.npz")
    feat = tmp_path / "data.raw"
    formats.write_raw(str(feat), g["ex_X"])
    mdl = tmp_path / "fc.gmm"
    formats.write_gmm_txt(str(mdl), formats.GMModel(g["ex_w"], g["ex_mu"], g["ex_cov"]))
    out = tmp_path / "out"
    out.mkdir()
    run(exe("gmm_loglike"), "-i", feat, "-g", mdl, "-L", "--data-T", "2", "-f", "-o", out)
    ll = formats.read_mat(str(out / "data.logL"), False)[0]
    assert np.abs(ll - g["ex_ll"]).max() < 1e-4
    xs = tmp_path / "x.prm"
    formats.write_sves(str(xs), g["X"])
    ubm = tmp_path / "ubm.gmm"
    formats.write_gmm_bin(str(ubm), formats.GMModel(g["w"], g["mu"], g["cov"]))
    run(exe("gmm_adapt"), "-i", xs, "-u", ubm, "-o", tmp_path / "em.gmm", "--it-EM", "3", "-W", "-M", "-V")
    m = formats.read_gmm_bin(str(tmp_path / "em.gmm"))
    assert m.full
    assert np.allclose(m.w, g["em_w"], rtol=1e-4, atol=1e-5) and np.allclose(m.mu, g["em_mu"], rtol=1e-4, atol=1e-5)
    assert np.allclose(m.var, g["em_cov"], rtol=1e-4, atol=1e-5)
    run(exe("gmm_adapt"), "-i", xs, "-u", ubm, "-o", tmp_path / "map.gmm", "--it-MAP", "1", "-r", "16",
        "-W", "-M", "-V")
    m = formats.read_gmm_bin(str(tmp_path / "map.gmm"))
    assert np.allclose(m.w, g["map_w"], rtol=1e-4, atol=1e-5) and np.allclose(m.mu, g["map_mu"], rtol=1e-4, atol=1e-5)
    assert np.allclose(m.var, g["map_cov"], rtol=1e-4, atol=1e-5)


def test_em_matches_reference(exe, golden, tmp_path):
    from gmm_gb300 import formats
    g = golden("em_small.npz")
    feat = tmp_path / "x.raw"
    formats.write_raw(str(feat), g["X"])
    write_model(tmp_path / "ubm.gmm", g["w"], g["mu"], g["var"])
    run(exe("gmm_adapt"), "-i", feat, "--data-T", "2", "-u", tmp_path / "ubm.gmm", "-o", tmp_path / "em.gmm",
        "-t", "2", "--it-EM", "3", "-W", "-M", "-V", "--precision", "fp32")
    m = read_model(tmp_path / "em.gmm")
    assert np.allclose(m.w, g["em_w"], rtol=1e-4, atol=1e-7)
    assert np.allclose(m.mu, g["em_mu"], rtol=1e-4, atol=1e-5)
    assert np.allclose(m.var, g["em_var"], rtol=1e-4, atol=1e-6)
    # file by file (two files, small batches) equals the resident run
    half = len(g["X"]) // 2
    formats.write_raw(str(tmp_path / "a.raw"), g["X"][:half])
    formats.write_raw(str(tmp_path / "b.raw"), g["X"][half:])
    run(exe("gmm_adapt"), "-i", tmp_path / "a.raw", "-i", tmp_path / "b.raw", "--data-T", "2", "-u",
        tmp_path / "ubm.gmm", "-o", tmp_path / "fbf.gmm", "-t", "2", "--it-EM", "3", "-W", "-M", "-V",
        "--precision", "fp32", "-f", "--prm-buffer", "0.0002")
    f = read_model(tmp_path / "fbf.gmm")
    assert np.allclose(f.w, m.w, rtol=1e-6) and np.allclose(f.mu, m.mu, rtol=1e-6, atol=1e-7)
    assert np.allclose(f.var, m.var, rtol=1e-6)


def test_map_and_mllr_match_reference(exe, golden, tmp_path):
    from gmm_gb300 import formats
    g = golden("map_mllr.npz")
    feat = tmp_path / "s.prm"
    formats.write_sves(str(feat), g["X"])
    ubm = tmp_path / "ubm.gmm"
    write_model(ubm, g["w"], g["mu"], g["var"])
    run(exe("gmm_adapt"), "-i", feat, "-u", ubm, "-o", tmp_path / "map.gmm", "-t", "2", "--it-MAP", "1",
        "-r", "16", "-M", "--precision", "fp32")
    m = read_model(tmp_path / "map.gmm")
    assert np.allclose(m.mu, g["map_mu"], rtol=1e-5, atol=1e-6)
    assert np.array_equal(m.w, g["map_w"])
    for init, key in (([], "0"), (["--mllr-init"], "1")):
        out = tmp_path / f"mllr{key}.gmm"
        run(exe("gmm_adapt"), "-i", feat, "-u", ubm, "-o", out, "-t", "1", "-a", "-s", "--precision", "fp32", *init)
        W = formats.read_trn(str(tmp_path / f"mllr{key}.mat"))
        assert np.allclose(W, g[f"mllr_W{key}"], rtol=2e-5, atol=2e-6)
        a = read_model(out)
        assert np.allclose(a.mu, g[f"mllr_mu{key}"], rtol=1e-5, atol=1e-5)
    # --save-in-stat-form: the model and the transform in the GMMStats<float> layout
    run(exe("gmm_adapt"), "-i", feat, "-u", ubm, "-o", tmp_path / "map.st", "-t", "2", "--it-MAP", "1",
        "-r", "16", "-M", "--precision", "fp32", "--save-in-stat-form")
    n, F, S = formats.read_gmm_stats(str(tmp_path / "map.st"), False, np.float32)
    assert np.array_equal(n, m.w) and np.array_equal(F, m.mu) and np.array_equal(S, m.var)
    run(exe("gmm_adapt"), "-i", feat, "-u", ubm, "-o", tmp_path / "w.st", "-t", "1", "--precision", "fp32",
        "--save-in-stat-form", "-T")
    n, F, S = formats.read_gmm_stats(str(tmp_path / "w.st"), True)
    D = g["X"].shape[1]
    assert S is None and np.all(n == 1) and F.shape == (D, D + 1)
    assert np.allclose(F, g["mllr_W0"], rtol=2e-5, atol=2e-6)
    # without --apply-trn only the transform is written
    out = tmp_path / "only.gmm"
    run(exe("gmm_adapt"), "-i", feat, "-u", ubm, "-o", out, "-t", "1", "-X", ".trn")
    assert (tmp_path / "only.trn").exists() and not out.exists()


def test_train_from_scratch_matches_reference(exe, golden, tmp_path):
    from gmm_gb300 import formats
    g = golden("train.npz")
    feat = tmp_path / "t.htk"
    formats.write_htk(str(feat), g["X"])
    out = tmp_path / "t.gmm"
    run(exe("gmm_adapt"), "-i", feat, "--data-T", "1", "-g", "8", "--it-EM", "3", "--split-X", "0.5",
        "--split-th", "0.2", "-o", out, "-T", "--precision", "fp32")
    m = formats.read_gmm_txt(str(out))
    w, mu, var = g["multi_w"], g["multi_mu"], g["multi_var"]
    alive = w > 0
    assert m.M == alive.sum()
    assert np.allclose(m.w, w[alive], rtol=1e-4, atol=1e-4)
    assert np.allclose(m.mu, mu[alive], rtol=1e-4, atol=1e-4)
    assert np.allclose(m.var, var[alive], rtol=1e-4)


def test_model_file_and_class_modes(exe, glib, tmp_path):
    from gmm_gb300 import adapt, formats, synth
    D, M = 12, 32
    w, mu, var = synth.generator_gmm(41, M, D)
    ubm = tmp_path / "ubm.gmm"
    write_model(ubm, w, mu, var)
    feats = tmp_path / "feats"
    feats.mkdir()
    X = {}
    for i, n in enumerate((900, 1500, 700)):
        X[f"s{i}"] = synth.sample_gmm(50 + i, w, mu + 0.2 * i, var, n)
        formats.write_sves(str(feats / f"s{i}.prm"), X[f"s{i}"])
    out = tmp_path / "models"
    out.mkdir()
    common = ["-u", ubm, "-t", "2", "--it-MAP", "1", "-r", "16", "-M", "-V", "-D", out]
    run(exe("gmm_adapt"), "-I", feats, "-e", ".prm", "--model-file-mode", *common)
    classes = tmp_path / "classes.txt"
    classes.write_text("spkA s0, s2\nspkB s1\n")
    run(exe("gmm_adapt"), "-S", classes, "-I", feats, "-e", ".prm", "-x", ".cls", *common)

    def python_map(x):
        ma = adapt.ModelAdapt(adapt.Options(adaptType=adapt.MAP, tau=16, iterCountMAP=1, AdaptMeanBool=True,
                                            AdaptVarBool=True, precision=glib.PREC_TC))
        ma.InsertData(x)
        ma.AdaptModel(formats.GMModel(w, mu, var))
        return ma.PickUpClientModel()

    for name, x in (("s0.gmm", X["s0"]), ("s1.gmm", X["s1"]), ("s2.gmm", X["s2"]),
                    ("spkA.cls", np.concatenate([X["s0"], X["s2"]])), ("spkB.cls", X["s1"])):
        got = read_model(out / name)
        want = python_map(x)
        assert np.allclose(got.mu, want.mu, rtol=1e-6, atol=1e-7), name
        assert np.allclose(got.var, want.var, rtol=1e-6), name


def test_train_full_covariance_command_line(exe, golden, tmp_path):
    """gmm_adapt --full-cov -g 6 --split-X 0.5 --split-th 0.2 against the reference build's
    full-covariance TrainFromScratch (tests/golden/train_full.npz); 1e-4 abs + rel."""
    from gmm_gb300 import formats
    g = golden("train_full.npz")
    feat = tmp_path / "t.raw"
    formats.write_raw(str(feat), g["X"])
    out = tmp_path / "t.gmm"
    run(exe("gmm_adapt"), "-i", feat, "--data-T", "2", "-g", "6", "--it-EM", "3", "--split-X", "0.5",
        "--split-th", "0.2", "--full-cov", "-o", out)
    m = formats.read_gmm_bin(str(out))
    w, mu, cov = g["multi_w"], g["multi_mu"], g["multi_cov"]
    alive = w > 0
    assert m.full and m.M == alive.sum()
    assert np.allclose(m.w, w[alive], rtol=1e-4, atol=1e-4)
    assert np.allclose(m.mu, mu[alive], rtol=1e-4, atol=1e-4)
    assert np.allclose(m.var, cov[alive], rtol=1e-4, atol=1e-4)
