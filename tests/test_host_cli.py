"""The C++ host layer (gmm_gb300/host) without a GPU: model files written by GMModel::Save are
byte-identical to formats.py's writers (which follow GMModel::WriteTXT / WriteBIN), the
command-line plumbing follows the reference tools' rules (option syntax, configuration files,
file lists, output naming, saveMat layout), and the two command lines reject bad arguments with
the reference's messages before they touch a device."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "gmm_gb300", "host")

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include "gmm_cli.hpp"
#include "gmm_host.hpp"
int main(int argc, char** argv) {
  const std::string cmd = argv[1];
  if (cmd == "model") {            // model IN TXT_IN OUT TXT_OUT
    gmmgb::GMModel g;
    g.Load(argv[2], std::atoi(argv[3]));
    const int z = g.RearrangeMixtures();
    g.Save(argv[4], std::atoi(argv[5]));
    std::printf("%d %d %d\n", g.GetDimension(), g.GetNumberOfMixtures(), z);
  } else if (cmd == "stats") {     // stats IN TXT_IN OUT TXT_OUT
    gmmgb::GMMStats st;
    st.load(argv[2], std::atoi(argv[3]));
    st.save(argv[4], std::atoi(argv[5]));
    std::printf("%d %d\n", st.M, st.D);
  } else if (cmd == "newpath") {   // newpath FILE DIR EXT
    std::printf("%s\n", gmmgb::cli::new_path(argv[2], argv[3], argv[4]).c_str());
  } else if (cmd == "list") {      // list PATH EXT
    std::vector<std::string> v;
    gmmgb::cli::read_list(argv[2], argv[3], &v);
    for (auto& s : v) std::printf("%s\n", s.c_str());
  } else if (cmd == "savemat") {   // savemat PATH TXT v...
    std::vector<float> v;
    for (int a = 4; a < argc; ++a) v.push_back(std::strtof(argv[a], nullptr));
    gmmgb::cli::save_mat(argv[2], std::atoi(argv[3]), v.data(), 1, (unsigned)v.size());
  } else if (cmd == "opts") {      // opts ARGS... : the parsed values
    gmmgb::cli::Parser P({{"config", 'c', gmmgb::cli::STR, "", ""}, {"in-file", 'i', gmmgb::cli::MULTI, "", ""},
                          {"tau", 'r', gmmgb::cli::STR, "0", ""}, {"mean", 'M', gmmgb::cli::FLAG, "0", ""},
                          {"var", 'V', gmmgb::cli::FLAG, "0", ""}});
    P.parse(argc - 1, argv + 1);
    std::printf("tau=%d mean=%d var=%d files=", P.get_int("tau"), (int)P.get_bool("mean"), (int)P.get_bool("var"));
    for (auto& f : P.all("in-file")) std::printf("%s,", f.c_str());
    std::printf("\n");
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def built():
    from gmm_gb300 import build
    build.build()
    return build


@pytest.fixture(scope="module")
def driver(built, tmp_path_factory):
    d = tmp_path_factory.mktemp("drv")
    src = d / "drv.cpp"
    src.write_text(DRIVER)
    exe = str(d / "drv")
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-I" + HOST, str(src),
                        os.path.join(HOST, "gmm_host.cpp"), "-o", exe, "-L" + built.OUT_DIR, "-lgmm_gb300",
                        "-Wl,-rpath," + built.OUT_DIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def run(*args):
        p = subprocess.run([exe, *map(str, args)], capture_output=True, text=True)
        assert p.returncode == 0, p.stderr
        return p.stdout
    return run


def model_with_zeros():
    from gmm_gb300 import synth
    w, mu, var = synth.generator_gmm(7, 9, 5)
    w[[1, 4]] = 0.0
    return w, mu, var


@pytest.mark.parametrize("txt_in", [0, 1])
@pytest.mark.parametrize("txt_out", [0, 1])
def test_model_files_match_python_writers(driver, tmp_path, txt_in, txt_out):
    from gmm_gb300 import formats
    g = formats.GMModel(*model_with_zeros())
    g.norm = np.linspace(0.5, 1.5, g.D).astype(np.float32)
    src = tmp_path / ("in.txt" if txt_in else "in.bin")
    # zero-weight components are dropped by both writers; the loaded model has 7 components
    (formats.write_gmm_txt if txt_in else formats.write_gmm_bin)(str(src), g)
    out = tmp_path / "out"
    D, M, z = map(int, driver("model", src, txt_in, out, txt_out).split())
    assert (D, M, z) == (5, 7, 0)
    ref = (formats.read_gmm_txt if txt_in else formats.read_gmm_bin)(str(src))
    want = tmp_path / "want"
    (formats.write_gmm_txt if txt_out else formats.write_gmm_bin)(str(want), ref)
    assert out.read_bytes() == want.read_bytes()


@pytest.mark.parametrize("txt_in", [0, 1])
@pytest.mark.parametrize("txt_out", [0, 1])
def test_full_model_files_match_python_writers(driver, tmp_path, txt_in, txt_out):
    from gmm_gb300 import formats, synth
    w, mu, cov = synth.generator_gmm_full(8, 5, 6)
    w[1] = 0.0
    g = formats.GMModel(w, mu, cov)
    src = tmp_path / ("in.txt" if txt_in else "in.bin")
    (formats.write_gmm_txt if txt_in else formats.write_gmm_bin)(str(src), g)
    out = tmp_path / "out"
    assert driver("model", src, txt_in, out, txt_out).split() == ["6", "4", "0"]
    ref = (formats.read_gmm_txt if txt_in else formats.read_gmm_bin)(str(src))
    assert ref.full
    want = tmp_path / "want"
    (formats.write_gmm_txt if txt_out else formats.write_gmm_bin)(str(want), ref)
    assert out.read_bytes() == want.read_bytes()


def test_full_stats_files(driver, tmp_path):
    from gmm_gb300 import estimator, formats
    rng = np.random.default_rng(9)
    D, M = 5, 3
    n, F, Sp = rng.uniform(1, 9, M), rng.standard_normal((M, D)), rng.standard_normal((M, D * (D + 1) // 2))
    src = tmp_path / "full.st"
    formats.write_gmm_stats(str(src), False, n, F, Sp)
    out = tmp_path / "o.st"
    assert driver("stats", src, 0, out, 0).split() == ["3", "5"]
    assert out.read_bytes() == src.read_bytes()
    st = estimator.GMMStats()
    st.load(str(out), False)
    assert st.hasFullCov() and np.array_equal(st.S, Sp)


def test_rearrange_matches_reference_rule(driver, tmp_path):
    """A text model that keeps zero-weight components (hand-written file) is rearranged as
    GMModel::RearrangeMixtures does, and Save drops the zero-weight ones."""
    from gmm_gb300 import formats
    w, mu, var = model_with_zeros()
    p = tmp_path / "z.txt"
    with open(p, "w") as f:  # the text layout, zero weights included
        f.write("5\n" + "1\n" * 5 + "9\n")
        for m in range(9):
            f.write("%15e\n\n" % w[m] + "".join("%15e\n" % v for v in mu[m]) + "\n" +
                    "".join("%15e\n" % v for v in var[m]) + "\n")
    out = tmp_path / "o.bin"
    D, M, z = map(int, driver("model", p, 1, out, 0).split())
    assert (M, z) == (9, 2)
    g = formats.read_gmm_txt(str(p))
    order = g.rearrange()
    r = formats.read_gmm_bin(str(out))
    keep = order[:7]
    assert np.array_equal(r.w, g.w[:7]) and np.array_equal(r.mu, formats.read_gmm_txt(str(p)).mu[keep])


@pytest.mark.parametrize("txt_in", [0, 1])
@pytest.mark.parametrize("txt_out", [0, 1])
def test_stats_files_match_python_writer(driver, tmp_path, txt_in, txt_out):
    from gmm_gb300 import estimator, formats
    rng = np.random.default_rng(4)
    n = rng.uniform(0, 500, 6)
    F = rng.standard_normal((6, 4)) * 100
    S = rng.uniform(1, 1e4, (6, 4))
    if txt_in:  # the text file holds 6 digits: start from values it represents exactly
        n, F, S = (np.array(["%g" % v for v in a.ravel()], float).reshape(a.shape) for a in (n, F, S))
    src = tmp_path / "in.st"
    formats.write_gmm_stats(str(src), txt_in, n, F, S)
    out = tmp_path / "out.st"
    assert driver("stats", src, txt_in, out, txt_out).split() == ["6", "4"]
    want = tmp_path / "want.st"
    formats.write_gmm_stats(str(want), txt_out, n, F, S)
    assert out.read_bytes() == want.read_bytes()
    st = estimator.GMMStats()
    st.load(str(out), txt_out)
    tol = 1e-5 if txt_out else 0
    assert np.allclose(st.n, n, rtol=tol, atol=0) and np.allclose(st.F, F, rtol=tol) and np.allclose(st.S, S, rtol=tol)
    st.save(str(tmp_path / "again.st"), txt_out)
    assert (tmp_path / "again.st").read_bytes() == out.read_bytes()


def test_output_naming_and_lists(driver, tmp_path):
    assert driver("newpath", "a/b/spk1.prm", "out", ".logL").strip() == "out/spk1.logL"
    assert driver("newpath", "spk1", "", ".gmm").strip() == "spk1.gmm"
    assert driver("newpath", "a/b.c/spk1", "o", ".x").strip() == "o/spk1.x"
    assert driver("newpath", "a/spk1.prm", "o", ".*").strip() == "o/spk1.prm"
    d = tmp_path / "feats"
    d.mkdir()
    for n in ("b.prm", "a.prm", "c.txt"):
        (d / n).write_bytes(b"x")
    assert driver("list", d, ".prm").split() == [str(d / "a.prm"), str(d / "b.prm")]
    assert len(driver("list", d, ".*").split()) == 3
    lst = tmp_path / "list.txt"
    lst.write_text("x1.prm\r\n\ny/x2.prm\n")
    assert driver("list", lst, ".*").split() == ["x1.prm", "y/x2.prm"]


def test_save_mat_layout(driver, tmp_path):
    from gmm_gb300 import formats
    vals = np.array([-27.2761, -1.5, 3.25e-7], np.float32)
    p = tmp_path / "m.txt"
    driver("savemat", p, 1, *vals)
    want = tmp_path / "w.txt"
    formats.write_loglikes_txt(str(want), vals)
    assert p.read_text() == want.read_text() == "1 3\n-27.2761 -1.5 3.25e-07 \n\n"
    b = tmp_path / "m.bin"
    driver("savemat", b, 0, *vals)
    assert np.array_equal(formats.read_mat(str(b), False)[0], vals)


def test_option_syntax_and_config(driver, tmp_path):
    out = driver("opts", "-i", "a", "--in-file=b", "-r", "16", "-M", "--var=0")
    assert out.strip() == "tau=16 mean=1 var=0 files=a,b,"
    cfg = tmp_path / "c.ini"
    cfg.write_text("tau = 3   # relevance\nvar = true\nin-file = z\n")
    assert driver("opts", "-c", cfg).strip() == "tau=3 mean=0 var=1 files=z,"
    # the command line wins over the file
    assert driver("opts", "-c", cfg, "--tau", "5", "-i", "q").strip() == "tau=5 mean=0 var=1 files=q,"


def cli(built, name, *args):
    return subprocess.run([os.path.join(built.OUT_DIR, name), *map(str, args)], capture_output=True, text=True)


def test_command_lines_check_arguments(built, tmp_path):
    r = cli(built, "gmm_adapt", "-h")
    assert r.returncode == 0
    for opt in ("--in-file", "--in-list", "--in-UBM", "--outFile", "--nummix", "--it-EM", "--it-MAP", "--tau",
                "--mean", "--apply-trn", "--save-trn", "--mllr-init", "--it-mllr", "--data-T", "--dwnsmp",
                "--file-by-file", "--model-file-mode", "--in-classes"):
        assert opt in r.stdout, opt
    r = cli(built, "gmm_adapt", "-o", "x.gmm", "-u", "ubm.gmm")
    assert r.returncode == 1 and "input not specified" in r.stdout
    r = cli(built, "gmm_adapt", "-i", "f.prm", "-u", "ubm.gmm")
    assert r.returncode == 1 and '"outFile" not specified' in r.stdout
    r = cli(built, "gmm_adapt", "-i", "f.prm", "-o", "x.gmm")
    assert r.returncode == 1 and "None input model" in r.stdout
    r = cli(built, "gmm_adapt", "--bogus")
    assert r.returncode == 1 and "unrecognised option" in r.stdout
    r = cli(built, "gmm_loglike", "-h")
    assert r.returncode == 0 and "--in-GMM" in r.stdout and "--for-each" in r.stdout
    r = cli(built, "gmm_loglike", "-i", "f.prm")
    assert r.returncode == 1 and '"in-GMM" not specified' in r.stderr
    feat = tmp_path / "f.prm"
    feat.write_bytes(b"x")
    cfg = tmp_path / "ll.ini"
    cfg.write_text(f"in-file = {feat}\nin-GMM = {tmp_path / 'missing.gmm'}\n")
    r = cli(built, "gmm_loglike", "-c", cfg)  # configuration read; the model is missing
    assert r.returncode == 1 and "missing.gmm] not found" in r.stderr
