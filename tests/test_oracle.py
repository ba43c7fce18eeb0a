"""The oracle is pinned against the reference: its golden file and its own outputs.

The port (float semantics of the reference CPU estimator) must reproduce the fixtures in
tests/golden bit for bit; those fixtures were produced by the reference compiled from its
sources (tests/golden/make_golden.py). The FP64 oracle must agree with the port to float
accuracy."""
import numpy as np
import pytest


def test_port_matches_reference_logfile(oracle, golden):
    g = golden("example.npz")
    ll = oracle.loglikes32(g["X"], g["w"], g["mu"], g["var"], threads=4)
    # example/data.logL holds 6 significant digits
    assert np.abs(ll - g["ll_file"]).max() < 6e-5
    assert np.array_equal(ll, g["ll_ref"])


@pytest.mark.parametrize("threads", [1, 4])
def test_port_stats_bit_exact(oracle, golden, threads):
    g = golden("example.npz")
    s = oracle.accumulate32(g["X"], g["w"], g["mu"], g["var"], threads=threads)
    t = str(threads)
    assert np.array_equal(s["n"], g["n" + t])
    assert np.array_equal(s["F"], g["F" + t])
    assert np.array_equal(s["S"], g["S" + t])
    assert s["totLL"] == g["totLL" + t]


def test_port_em_iterations_bit_exact(oracle, golden):
    g = golden("em_small.npz")
    s = oracle.accumulate32(g["X"], g["w"], g["mu"], g["var"], threads=4)
    for k in "nFS":
        assert np.array_equal(s[k], g[k])
    w, mu, var = g["w"], g["mu"], g["var"]
    for it in range(3):
        st = oracle.accumulate32(g["X"], w, mu, var, threads=4)
        assert st["totLL"] == g["em_ll"][it]
        w, mu, var, _ = oracle.em_update(w, mu, var, st)
    assert np.array_equal(w, g["em_w"]) and np.array_equal(mu, g["em_mu"]) and np.array_equal(var, g["em_var"])


def test_port_edge_cases(oracle, golden):
    e = golden("edge.npz")
    # zero-weight components: the reference reorders them behind the others; the port skips
    # them in place, so compare through the reported order
    s = oracle.accumulate32(e["zw_X"], e["zw_w"], e["zw_mu"], e["zw_var"], threads=3)
    order = e["zw_order"]
    assert np.array_equal(s["n"][order], e["zw_n"])
    assert np.array_equal(s["F"][order], e["zw_F"])
    assert np.array_equal(s["S"][order], e["zw_S"])
    assert s["totLL"] == e["zw_totLL"]
    # single component: gamma = 1 for every frame
    s = oracle.accumulate32(e["zw_X"], np.ones(1, np.float32), e["zw_mu"][:1], e["zw_var"][:1], threads=2)
    assert np.array_equal(s["n"], e["m1_n"]) and s["totLL"] == e["m1_totLL"]
    assert np.array_equal(s["S"], e["m1_S"])
    # N < 100: single-thread path
    gw = golden("edge.npz")
    from gmm_gb300 import synth
    w, mu, var = synth.generator_gmm(21, 8, 6)
    s = oracle.accumulate32(e["zw_X"][:50], w, mu, var, threads=4)
    assert np.array_equal(s["F"], e["n50_F"]) and s["totLL"] == e["n50_totLL"]
    # outlier frame: numerical-stability branch (frame LL = minLogLike, no statistics)
    s = oracle.accumulate32(e["out_X"], w, mu, var, threads=2)
    assert s["totLL"] == e["out_totLL"] and np.array_equal(s["n"], e["out_n"])
    ll = oracle.loglikes32(e["out_X"], w, mu, var, threads=2)
    assert np.array_equal(ll, e["out_ll"]) and ll[17] == np.float32(-1e20)
    # D = 1
    s = oracle.accumulate32(e["zw_X"][:, :1], w, mu[:, :1], var[:, :1], threads=2)
    assert np.array_equal(s["S"], e["d1_S"]) and s["totLL"] == e["d1_totLL"]
    # EM kills an under-occupied component (weight 0, mean 0, variance bytes 0x01)
    w, mu, var = e["kill_w0"], e["kill_mu0"], e["kill_var0"]
    for it in range(2):
        st = oracle.accumulate32(e["kill_X"], w, mu, var, threads=2)
        assert st["totLL"] == e["kill_ll"][it]
        w, mu, var, _ = oracle.em_update(w, mu, var, st)
    # the reference's model comes back rearranged (killed component last)
    order, _ = oracle.rearrange_order(w)
    assert np.array_equal(w[order], e["kill_w"])
    assert np.array_equal(mu[order], e["kill_mu"]) and np.array_equal(var[order], e["kill_var"])
    assert (e["kill_w"] == 0).sum() >= 1
    assert e["kill_var"][-1].view(np.uint32)[0] == 0x01010101


def test_port_map_mllr_bit_exact(oracle, golden):
    g = golden("map_mllr.npz")
    st = oracle.accumulate32(g["X"], g["w"], g["mu"], g["var"], flags=oracle.ACC_MEAN, threads=2)
    w, mu, var = oracle.map_update(g["w"], g["mu"], g["var"], st, 16)
    assert np.array_equal(mu, g["map_mu"]) and np.array_equal(w, g["map_w"])
    for init, W_ref, mu_ref in ((False, g["mllr_W0"], g["mllr_mu0"]), (True, g["mllr_W1"], g["mllr_mu1"])):
        W = oracle.mllr_w(g["mu"], g["var"], st, ubm_init=init)
        assert np.array_equal(W, W_ref)
        assert np.array_equal(oracle.mllr_apply(g["mu"], W), mu_ref)


def test_fp64_oracle_agrees_with_port(oracle, golden):
    g = golden("em_small.npz")
    s32 = oracle.accumulate32(g["X"], g["w"], g["mu"], g["var"], threads=1)
    s64 = oracle.accumulate64(g["X"], g["w"], g["mu"], g["var"])
    assert abs(s64["totLL"] - s32["totLL"]) / abs(s64["totLL"]) < 1e-6
    assert np.allclose(s64["n"], s32["n"], rtol=1e-4, atol=1e-3)
    ll32 = oracle.loglikes32(g["X"], g["w"], g["mu"], g["var"])
    ll64 = oracle.loglikes64(g["X"], g["w"], g["mu"], g["var"])
    assert np.abs(ll32 - ll64).max() < 1e-3


def test_oracle_rejects_low_variance(oracle, golden):
    g = golden("em_small.npz")
    var = g["var"].copy()
    var[3, 5] = 1e-7
    with pytest.raises(RuntimeError):
        oracle.accumulate32(g["X"], g["w"], g["mu"], var)


def test_rearrange_order(oracle):
    from gmm_gb300.formats import GMModel
    w = np.array([0.2, 0.0, 0.3, 0.0, 0.5], np.float32)
    order, nz = oracle.rearrange_order(w)
    assert nz == 3 and list(order) == [0, 2, 4, 3, 1]
    g = GMModel(w, np.arange(10, dtype=np.float32).reshape(5, 2), np.ones((5, 2)))
    assert list(g.rearrange()) == [0, 2, 4, 3, 1]


def test_full_oracle_against_reference(oracle, golden):
    """Full covariances: the FP64 restatement against the reference build (single-precision
    Cholesky / inverse through the restated LAPACK routines): per-frame LL within 5e-5 abs,
    statistics within 2e-6 of each statistic's scale; three EM iterations and one MAP iteration
    of the oracle (FP64 E-step, the reference's update expressions) within 1e-4 rel."""
    g = golden("full.npz")
    ll = oracle.full64_loglikes(g["ex_X"], g["ex_w"], g["ex_mu"], g["ex_cov"])
    assert np.abs(ll - g["ex_ll"]).max() < 5e-5
    st = oracle.full64_accumulate(g["ex_X"], g["ex_w"], g["ex_mu"], g["ex_cov"])
    for k, ref in (("n", g["ex_n"]), ("F", g["ex_F"]), ("Sp", g["ex_Sp"])):
        assert np.abs(st[k] - ref).max() <= 2e-6 * np.abs(ref).max(), k
    assert abs(st["totLL"] - g["ex_totLL"]) <= 1e-6 * abs(g["ex_totLL"])
    w, mu, cov = g["w"].copy(), g["mu"].copy(), g["cov"].copy()
    for it in range(3):
        st = oracle.full64_accumulate(g["X"], w, mu, cov)
        assert abs(st["totLL"] - g["em_ll"][it]) <= 1e-6 * abs(g["em_ll"][it])
        w, mu, cov, alive = oracle.full_em_update(w, mu, cov, st)
    assert np.allclose(w, g["em_w"], rtol=1e-4) and np.allclose(mu, g["em_mu"], rtol=1e-4, atol=1e-5)
    assert np.allclose(cov, g["em_cov"], rtol=1e-4, atol=1e-5)
    st = oracle.full64_accumulate(g["X"], g["w"], g["mu"], g["cov"])
    mw, mmu, mcov = oracle.full_map_update(g["w"], g["mu"], g["cov"], st, 16, True, True, True)
    assert np.allclose(mw, g["map_w"], rtol=1e-5) and np.allclose(mmu, g["map_mu"], rtol=1e-5, atol=1e-6)
    assert np.allclose(mcov, g["map_cov"], rtol=1e-5, atol=1e-6)


def test_full_model_files(tmp_path):
    from gmm_gb300 import formats, synth
    w, mu, cov = synth.generator_gmm_full(3, 5, 7)
    w[2] = 0
    g = formats.GMModel(w, mu, cov)
    for ext, wr, rd in (("txt", formats.write_gmm_txt, formats.read_gmm_txt),
                        ("bin", formats.write_gmm_bin, formats.read_gmm_bin)):
        p = str(tmp_path / f"m.{ext}")
        wr(p, g)
        r = rd(p)
        keep = w > 0
        assert r.full and r.var.shape == (4, 7, 7)
        tol = 1e-6 if ext == "txt" else 0
        assert np.allclose(r.var, cov[keep], rtol=tol) and np.allclose(r.mu, mu[keep], rtol=tol, atol=1e-7)


def test_fmllr_oracle_against_reference(oracle, golden):
    """fMLLR: the restatement is bit-identical to the reference given the reference's own
    statistics; from the FP64 oracle's statistics W agrees within 1e-6 (abs) of the
    reference's W."""
    g = golden("fmllr.npz")
    st = dict(n=g["n"], F=g["F"], Sp=g["Sp"], totN=len(g["X"]))
    assert np.array_equal(oracle.fmllr_w(g["mu"], g["var"], st), g["W"])
    s64 = oracle.accumulate64_fullstats(g["X"], g["w"], g["mu"], g["var"])
    for k in ("n", "F", "Sp"):
        assert np.abs(s64[k] - g[k]).max() <= 1e-6 * np.abs(g[k]).max(), k
    assert np.abs(oracle.fmllr_w(g["mu"], g["var"], s64) - g["W"]).max() < 1e-6


def test_mllr_map_oracle_against_reference(oracle, golden):
    """MLLR+MAP: MLLR of the UBM (no UBM initialisation, the command-line default), then MAP of
    the transformed model against the original UBM -- the port reproduces the reference's
    AdaptModel bit for bit."""
    g = golden("map_mllr.npz")
    want = golden("mllr_map.npz")
    X, w, mu, var = g["X"], g["w"], g["mu"], g["var"]
    st = oracle.accumulate32(X, w, mu, var, flags=oracle.ACC_MEAN, threads=2)
    mu2 = oracle.mllr_apply(mu, oracle.mllr_w(mu, var, st))
    st2 = oracle.accumulate32(X, w, mu2, var, flags=oracle.ACC_MEAN | oracle.ACC_VAR, threads=2)
    _, omu, ovar = oracle.map_update(w, mu, var, st2, 16, w=w.copy(), mu=mu2.copy(), var=var.copy(),
                                     upM=True, upV=True)
    assert np.array_equal(omu, want["mu"]) and np.array_equal(ovar, want["var"])


def test_robust_oracle_against_reference(oracle, golden):
    """--robust: FP64 auxiliary statistics within 1e-6 of the reference's scale, and two robust
    EM iterations (FP64 E-step, the reference's MakeRobustStats / UpdateModelEM expressions)
    within 1e-4 rel / 1e-4 abs of the reference's models (diagonal and full covariances)."""
    r = golden("robust.npz")
    e = golden("em_small.npz")
    f = golden("full.npz")
    for key, X, w, mu, var, full in (("diag", e["X"], e["w"], e["mu"], e["var"], False),
                                      ("full", f["X"], f["w"], f["mu"], f["cov"], True)):
        a = oracle.aux64(X, w, mu, var, full=full)
        for k in ("aux", "aux2", "aux3"):
            ref = r[f"{key}_{k}"]
            assert np.abs(a[k] - ref).max() <= 1e-6 * np.abs(ref).max(), (key, k)
        ww, mm, vv = w.copy(), mu.copy(), var.copy()
        for _ in range(2):
            order, _ = oracle.rearrange_order(ww)  # insertModel moves killed components to the end
            ww, mm, vv = ww[order], mm[order], vv[order]
            st = oracle.full64_accumulate(X, ww, mm, vv) if full else oracle.accumulate64(X, ww, mm, vv)
            ax = oracle.aux64(X, ww, mm, vv, full=full)
            S, nind = oracle.make_robust(st, ax, full=full)
            ww, mm, vv, _ = oracle.em_update_robust(ww, mm, vv, st, S, nind, full=full)
        vkey = "cov" if full else "var"
        assert np.allclose(ww, r[f"{key}_em_w"], rtol=1e-4, atol=1e-6), key
        assert np.allclose(mm, r[f"{key}_em_mu"], rtol=1e-4, atol=1e-4), key
        assert np.allclose(vv, r[f"{key}_em_{vkey}"], rtol=1e-4, atol=1e-4), key
