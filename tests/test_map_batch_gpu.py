"""Batched MAP adaptation (gmm_map_batch) against the oracle and the one-speaker path.

The reference adapts one speaker at a time (Model_ADAPT's loop around CModelAdapt::AdaptModel):
for each speaker, statistics over the UBM, then UpdateModelMAP against the UBM. gmm_map_batch
does the same for S speakers in one call. Tolerances, written per quantity:
  FP32 path     bit-identical to the one-speaker FP32 path (same kernels on the same frames),
                and within 1e-5 rel of the float oracle port
  TC path       adapted means/vars/weights rel <= 1e-4 (atol 1e-4) of the FP64 oracle, speaker
                log-likelihood rel <= 1e-6; against the one-speaker TC path the same per-frame
                log-likelihoods (exact speaker totals) and means within 1e-5, variances within
                1e-4 rel: the FP32 accumulators group frames differently (one speaker run vs
                one slice per CTA), and the variance update S/n - mu^2 magnifies that
                rounding difference by (mu^2 + var) / var
Speaker lengths cover the tile edges (0, 1, 127, 128, 129 frames) and a speaker range that
does not start at frame 0.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LENS = [300, 0, 1, 127, 128, 129, 700, 2000, 5, 0, 256, 1100]


def workload(D=60, M=160, seed=31, lens=LENS, lead=37):
    from gmm_gb300 import synth
    uw, umu, uvar = synth.generator_gmm(seed, M, D)
    total = lead + int(np.sum(lens))
    X = synth.sample_gmm(seed + 1, uw, umu + 0.3, uvar, total)
    offs = lead + np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    return X, offs, (uw, umu, uvar)


def one_speaker(glib, prec, X, ubm, tau, upW, upM, upV):
    """The reference's per-speaker sequence through the one-model entry points."""
    uw, umu, uvar = ubm
    h = glib.Handle(0)
    h.set_precision(prec)
    h.upload_model(uw, umu, uvar)
    h.set_prior(uw, umu, uvar)
    if len(X) == 0:
        return uw.copy(), umu.copy(), uvar.copy(), 0.0
    h.upload_features(X)
    flags = (glib.ACC_MEAN if upM else 0) | (glib.ACC_VAR if upV else 0)
    if upW and not upM and not upV:
        flags = glib.ACC_PROBS_ONLY
    st = h.accumulate(flags)
    h.map_update(tau, upW, upM, upV)
    w, mu, var = h.read_model()
    h.close()
    return w, mu, var, st["totLL"]


def oracle_speaker(oracle, X, ubm, tau, upW, upM, upV, fp64):
    uw, umu, uvar = ubm
    if len(X) == 0:
        return uw.copy(), umu.copy(), uvar.copy(), 0.0
    st = (oracle.accumulate64 if fp64 else oracle.accumulate32)(X, uw, umu, uvar)
    w, mu, var = oracle.map_update(uw, umu, uvar, st, tau, upW=upW, upM=upM, upV=upV)
    return w, mu, var, st["totLL"]


@pytest.mark.parametrize("upW,upM,upV", [(0, 1, 0), (1, 1, 1)])
def test_fp32_batch_equals_one_speaker_path(glib, oracle, upW, upM, upV):
    X, offs, ubm = workload()
    h = glib.Handle(0)
    h.set_precision(glib.PREC_FP32)
    h.upload_model(*ubm)
    h.upload_features(X)
    w, mu, var, ll = h.map_batch(offs, 16, upW, upM, upV)
    for s in range(len(offs) - 1):
        Xs = X[offs[s]:offs[s + 1]]
        rw, rmu, rvar, rll = one_speaker(glib, glib.PREC_FP32, Xs, ubm, 16, upW, upM, upV)
        assert np.array_equal(w[s], rw) and np.array_equal(mu[s], rmu) and np.array_equal(var[s], rvar), s
        assert ll[s] == rll, s
        ow, omu, ovar, oll = oracle_speaker(oracle, Xs, ubm, 16, upW, upM, upV, fp64=False)
        assert np.allclose(mu[s], omu, rtol=1e-5, atol=1e-6), s
        assert np.allclose(var[s], ovar, rtol=1e-5), s
        assert np.allclose(w[s], ow, rtol=1e-5), s
    h.close()


@pytest.mark.parametrize("D,M", [(60, 160), (39, 300), (13, 64)])
def test_tc_batch_matches_fp64(glib, oracle, D, M):
    X, offs, ubm = workload(D=D, M=M, seed=40 + D)
    h = glib.Handle(0)
    h.set_precision(glib.PREC_TC)
    h.upload_model(*ubm)
    h.upload_features(X)
    w, mu, var, ll = h.map_batch(offs, 16, 1, 1, 1)
    for s in range(len(offs) - 1):
        Xs = X[offs[s]:offs[s + 1]]
        ow, omu, ovar, oll = oracle_speaker(oracle, Xs, ubm, 16, 1, 1, 1, fp64=True)
        assert np.allclose(mu[s], omu, rtol=1e-4, atol=1e-4), (s, np.abs(mu[s] - omu).max())
        assert np.allclose(var[s], ovar, rtol=1e-4, atol=1e-5), (s, np.abs(var[s] - ovar).max())
        assert np.allclose(w[s], ow, rtol=1e-4, atol=1e-7), s
        assert abs(ll[s] - oll) <= 1e-6 * abs(oll) + 1e-9, (s, ll[s], oll)
        if len(Xs) == 0:
            assert np.array_equal(mu[s], ubm[1]) and ll[s] == 0.0
        tw, tmu, tvar, tll = one_speaker(glib, glib.PREC_TC, Xs, ubm, 16, 1, 1, 1)
        assert np.allclose(mu[s], tmu, rtol=1e-5, atol=1e-5), s
        assert np.allclose(var[s], tvar, rtol=1e-4), s
        assert abs(ll[s] - tll) <= 1e-9 * abs(tll) + 1e-9, s
    # the resident model and features are unchanged and still usable
    st = h.accumulate()
    o = oracle.accumulate64(X, *ubm)
    assert abs(st["totLL"] - o["totLL"]) <= 1e-6 * abs(o["totLL"])
    h.close()


def test_batch_mean_only_two_calls_repeat(glib):
    """Two calls in a row give the same result (no state leaks between calls)."""
    X, offs, ubm = workload(seed=55)
    h = glib.Handle(0)
    h.set_precision(glib.PREC_TC)
    h.upload_model(*ubm)
    h.upload_features(X)
    a = h.map_batch(offs, 16, 0, 1, 0)
    b = h.map_batch(offs, 16, 0, 1, 0)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    # mean-only: weights and variances stay the UBM's
    assert np.array_equal(a[0], np.broadcast_to(ubm[0], a[0].shape))
    assert np.array_equal(a[2], np.broadcast_to(ubm[2], a[2].shape))
    h.close()


@pytest.mark.parametrize("upW,upM,upV", [(0, 1, 0), (1, 1, 1)])
def test_batch_graph_replay_equals_eager(glib, upW, upM, upV):
    """Over the resident frames a batch layout that comes twice in a row is captured (after the
    second call's eager run) and replayed by later calls with the same layout. Replays with the
    same offsets, and with other speaker lengths of the same padded layout (same speaker count,
    tiles and work items; the offsets, pieces and work items are uploaded every call), equal the
    eager calls bit for bit, and every call adds the same number of kernel launches."""
    X, offs, ubm = workload(seed=57)
    lens = np.diff(offs)
    # other lengths of the same tile layout: move frames within each speaker's last tile
    lens2 = lens.copy()
    for s in range(len(lens2)):
        if lens2[s] % 128 not in (0, 1):
            lens2[s] -= 1
    offs2 = offs[0] + np.concatenate([[0], np.cumsum(lens2)]).astype(np.int64)

    def fresh(o):
        h = glib.Handle(0)
        h.set_precision(glib.PREC_TC)
        h.upload_model(*ubm)
        h.upload_features(X)
        r = h.map_batch(o, 16, upW, upM, upV)
        h.close()
        return r

    h = glib.Handle(0)
    h.set_precision(glib.PREC_TC)
    h.upload_model(*ubm)
    h.upload_features(X)
    counts = [h.launch_count()]
    results = []
    for o in (offs, offs, offs2, offs):  # eager, eager + capture, replay, replay
        results.append(h.map_batch(o, 16, upW, upM, upV))
        counts.append(h.launch_count())
    h.close()
    first, again, other, last = results
    for x, y, z in zip(first, again, last):
        assert np.array_equal(x, y)
        assert np.array_equal(x, z)
    for x, y in zip(other, fresh(offs2)):
        assert np.array_equal(x, y)
    steps = np.diff(counts)
    assert steps[0] > 0 and np.all(steps == steps[0]), steps


def test_batch_bad_offsets_are_errors(glib):
    X, offs, ubm = workload(seed=56)
    h = glib.Handle(0)
    h.upload_model(*ubm)
    h.upload_features(X)
    for bad in (np.array([0, 10, 5]), np.array([0, len(X) + 1]), np.array([-1, 3])):
        with pytest.raises(glib.GMMError) as e:
            h.map_batch(bad, 16)
        assert e.value.code == glib.ERR_ARG
    with pytest.raises(glib.GMMError) as e:
        h.map_batch(offs, 0)
    assert e.value.code == glib.ERR_ARG
    h.close()


def test_batch_scratch_reuse_across_sizes(glib):
    """The batched calls keep their device buffers between calls (grow-only scratch): a small
    batch after a large one, a large one after a small one and a MAP call after an MLLR call on
    the same handle give what a fresh handle gives for each batch."""
    X, offs, ubm = workload(seed=57)
    small = offs[3:7] - 0  # a few speakers, a sub-range of the frames
    calls = [("map", offs, (16, 1, 1, 1)), ("map", small, (8, 0, 1, 0)), ("mllr", offs, ()),
             ("map", offs, (16, 0, 1, 1)), ("map", small, (8, 1, 1, 0))]

    def run(h, kind, o, args):
        if kind == "map":
            return h.map_batch(o, *args)
        W, st, _, ll = h.mllr_batch(o, means=False)
        return W, st, ll

    h = glib.Handle(0)
    h.set_precision(glib.PREC_TC)
    h.upload_model(*ubm)
    h.upload_features(X)
    shared = [run(h, *c) for c in calls]
    h.close()
    for c, got in zip(calls, shared):
        f = glib.Handle(0)
        f.set_precision(glib.PREC_TC)
        f.upload_model(*ubm)
        f.upload_features(X)
        want = run(f, *c)
        f.close()
        for x, y in zip(got, want):
            assert np.array_equal(x, y), c[0]


@pytest.mark.parametrize("D", [60, 24])
def test_batch_host_frames_match_resident(glib, D):
    """gmm_map_batch_host / gmm_mllr_batch_host (frames copied in chunks of whole speakers, each
    chunk's log-likelihood kernels starting when its frames land) give the results of
    gmm_upload_features + the resident-frame calls, bit for bit. D = 60 builds the feature planes
    in a separate pass (K = 128), D = 24 inside the logits kernel (K = 64)."""
    X, offs, ubm = workload(D=D, seed=58)
    h = glib.Handle(0)
    h.set_precision(glib.PREC_TC)
    h.upload_model(*ubm)
    h.upload_features(X)
    a = h.map_batch(offs, 16, 1, 1, 1)
    m = h.mllr_batch(offs)
    h.close()
    g = glib.Handle(0)
    g.set_precision(glib.PREC_TC)
    g.upload_model(*ubm)
    b = g.map_batch_host(X, offs, 16, 1, 1, 1)
    n = g.mllr_batch_host(X, offs)
    b2 = g.map_batch_host(X, offs, 16, 1, 1, 1)  # again on the same handle: buffers reused
    g.close()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    for x, y in zip(a, b2):
        assert np.array_equal(x, y)
    for x, y in zip(m, n):
        assert np.array_equal(x, y)
