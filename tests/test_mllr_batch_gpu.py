"""Batched global MLLR (gmm_mllr_batch) against the oracle, per speaker.

The batched path forms the G and k sums over components as FP32-operand GEMMs with FP64
accumulation, so it is compared with the oracle's FP64 MLLR (orc_mllr_w: the reference's
ComputeKiGi_MLLR + pivot-free Gauss-Jordan) on the oracle's own statistics. Tolerances:
  W                       |dW| <= 2e-4 * (1 + |W|) for the FP32 path, 1e-3 * (1 + |W|) for the
                          tensor-core path (its statistics are FP32-level, see test_tc_gpu.py)
  adapted means           |d mu'| <= 1e-3 * (1 + |mu'|)
  too few frames          status GMM_ERR_MLLR, W zero, means unchanged
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def c4_small(D=13, M=96, lens=(600, 5, 1500, 3000, 900), seed=8):
    from gmm_gb300 import synth
    uw, umu, uvar = synth.generator_gmm(seed, M, D)
    r = np.random.default_rng(seed)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    X = np.empty((int(offs[-1]), D), np.float32)
    for s, n in enumerate(lens):
        A = np.eye(D) + 0.1 * r.standard_normal((D, D))
        b = r.standard_normal(D) * np.sqrt(0.5)
        Z = synth.sample_gmm(seed * 1000 + s, uw, umu, uvar, n)
        X[offs[s]:offs[s + 1]] = (Z @ A.T + b).astype(np.float32)
    return X, offs, (uw, umu, uvar)


@pytest.mark.parametrize("prec_name,tol", [("PREC_FP32", 2e-4), ("PREC_TC", 1e-3)])
@pytest.mark.parametrize("ubm_init", [False, True])
def test_mllr_batch_matches_oracle(glib, oracle, prec_name, tol, ubm_init):
    X, offs, ubm = c4_small()
    h = glib.Handle(0)
    h.set_precision(getattr(glib, prec_name))
    h.upload_model(*ubm)
    h.upload_features(X)
    W, st, mu, ll = h.mllr_batch(offs, ubm_init=ubm_init)
    h.close()
    for s in range(len(offs) - 1):
        Xs = X[offs[s]:offs[s + 1]]
        o = oracle.accumulate64(Xs, *ubm, flags=oracle.ACC_MEAN)
        assert abs(ll[s] - o["totLL"]) <= 1e-6 * abs(o["totLL"])
        try:
            oW = oracle.mllr_w(ubm[1], ubm[2], o, ubm_init=ubm_init)
        except RuntimeError:
            assert st[s] == glib.ERR_MLLR, s
            assert not W[s].any() and np.array_equal(mu[s], ubm[1])
            continue
        assert st[s] == glib.OK, s
        assert np.all(np.abs(W[s] - oW) <= tol * (1 + np.abs(oW))), (s, np.abs(W[s] - oW).max())
        omu = oracle.mllr_apply(ubm[1], oW)
        assert np.all(np.abs(mu[s] - omu) <= 10 * tol * (1 + np.abs(omu))), s


def test_mllr_batch_single_speaker_close_to_exact_path(glib):
    """One speaker through gmm_mllr_batch and through gmm_accumulate + gmm_mllr_estimate (the
    reference's FP64 sequence) on the plain path."""
    X, offs, ubm = c4_small(lens=(2500,))
    h = glib.Handle(0)
    h.upload_model(*ubm)
    h.upload_features(X)
    W, st, _, _ = h.mllr_batch(offs, means=False)
    h.accumulate(glib.ACC_MEAN)
    We = h.mllr_estimate()
    h.close()
    assert st[0] == glib.OK
    assert np.all(np.abs(W[0] - We) <= 2e-4 * (1 + np.abs(We)))


def test_mllr_batch_tc_tiles_match_fp32_path(glib, oracle):
    """The tensor-core G term over several speaker tiles (140 speakers), component chunks
    (M = 300: three 128-component accumulator readouts, the last one partial) and column tiles
    (D = 24: 325 upper-triangle pairs in two tiles of 176) agrees with the FP32 GEMM path and,
    for a few speakers, with the oracle's FP64 MLLR."""
    D, M, S = 24, 300, 140
    lens = [250 + 7 * (s % 11) for s in range(S)]
    X, offs, ubm = c4_small(D=D, M=M, lens=lens, seed=11)
    res = {}
    for prec in ("PREC_FP32", "PREC_TC"):
        h = glib.Handle(0)
        h.set_precision(getattr(glib, prec))
        h.upload_model(*ubm)
        h.upload_features(X)
        res[prec] = h.mllr_batch(offs, means=False)
        h.close()
    Wf, stf = res["PREC_FP32"][0], res["PREC_FP32"][1]
    Wt, stt = res["PREC_TC"][0], res["PREC_TC"][1]
    assert np.array_equal(stf, stt)
    ok = stf == glib.OK
    assert ok.sum() > S // 2
    assert np.all(np.abs(Wt[ok] - Wf[ok]) <= 1e-3 * (1 + np.abs(Wf[ok]))), np.abs(Wt[ok] - Wf[ok]).max()
    for s in (0, 77, S - 1):
        if not ok[s]:
            continue
        o = oracle.accumulate64(X[offs[s]:offs[s + 1]], *ubm, flags=oracle.ACC_MEAN)
        oW = oracle.mllr_w(ubm[1], ubm[2], o, ubm_init=False)
        assert np.all(np.abs(Wt[s] - oW) <= 1e-3 * (1 + np.abs(oW))), (s, np.abs(Wt[s] - oW).max())
