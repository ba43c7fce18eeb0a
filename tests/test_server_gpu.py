"""Request server (gmm_server_*): results against the one-request entry points, alone vs in a mix.

Tolerances, written per check:
  scoring request     per-frame log-likelihoods bit-identical to gmm_loglikes on the tensor-core
                      path (same kernels, same model planes); total = FP64 sum of those, within
                      1e-12 rel of numpy's sum of the same values
  MAP request         bit-identical to gmm_map_batch (tensor-core path) for the same speaker: the
                      server cuts a request into 8192-frame pieces whose FP64 sums are added in
                      the same order as the one-call path's periodic flushes
  alone vs mix        bit-identical (a request's arithmetic does not depend on its batch)
  against the oracle  MAP means rel 1e-4 / atol 1e-4 of the FP64 oracle (as gmm_map_batch)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

D, M = 20, 160


def models(n, seed=5):
    from gmm_gb300 import synth
    return [synth.generator_gmm(seed + i, M, D) for i in range(n)]


def frames(model, n, seed):
    from gmm_gb300 import synth
    w, mu, var = model
    return synth.sample_gmm(seed, w, mu + 0.2, var, n)


@pytest.fixture
def server(glib):
    s = glib.Server(0, D, M, 8, 256 << 20)
    yield s
    s.close()


def test_scoring_matches_one_model_path(glib, server):
    ms = models(3)
    ids = [server.add_model(*m) for m in ms]
    X = frames(ms[1], 1500, 11)
    t = server.submit(glib.REQ_SCORE, ids[1], X, frame_ll=True)
    r = server.result(t)
    h = glib.Handle(0)
    h.set_precision(glib.PREC_TC)
    h.upload_model(*ms[1])
    h.upload_features(X)
    ll = h.loglikes()
    h.close()
    assert np.array_equal(r["frame_ll"], ll)
    assert abs(r["ll"] - ll.astype(np.float64).sum()) <= 1e-12 * abs(r["ll"])


@pytest.mark.parametrize("n", [1, 700, 9000, 20000])
def test_map_matches_map_batch(glib, server, n):
    ms = models(2, seed=20)
    ids = [server.add_model(*m) for m in ms]
    X = frames(ms[0], n, 30 + n)
    t = server.submit(glib.REQ_MAP, ids[0], X, tau=16, upW=1, upM=1, upV=1)
    r = server.result(t)
    h = glib.Handle(0)
    h.set_precision(glib.PREC_TC)
    h.upload_model(*ms[0])
    h.upload_features(X)
    w, mu, var, ll = h.map_batch(np.array([0, n]), 16, 1, 1, 1)
    h.close()
    assert np.array_equal(r["w"], w[0]) and np.array_equal(r["mu"], mu[0]) and np.array_equal(r["var"], var[0])
    assert r["ll"] == pytest.approx(ll[0], rel=1e-12)


def test_alone_and_in_mix_are_identical(glib, server):
    ms = models(6, seed=40)
    ids = [server.add_model(*m) for m in ms]
    rng = np.random.default_rng(3)
    probe_map = frames(ms[2], 5000, 99)
    probe_score = frames(ms[4], 3000, 98)
    a_map = server.result(server.submit(glib.REQ_MAP, ids[2], probe_map, upM=1))
    a_score = server.result(server.submit(glib.REQ_SCORE, ids[4], probe_score, frame_ll=True))
    tickets = []
    for i in range(40):
        k = int(rng.integers(0, 2))
        mdl = int(rng.integers(0, len(ids)))
        n = int(rng.integers(1, 12000))
        tickets.append(server.submit(k, ids[mdl], frames(ms[mdl], n, 200 + i), upM=1))
        if i == 17:
            tm = server.submit(glib.REQ_MAP, ids[2], probe_map, upM=1)
            ts = server.submit(glib.REQ_SCORE, ids[4], probe_score, frame_ll=True)
    for t in tickets:
        server.result(t)
    b_map = server.result(tm)
    b_score = server.result(ts)
    assert np.array_equal(a_map["mu"], b_map["mu"]) and a_map["ll"] == b_map["ll"]
    assert np.array_equal(a_score["frame_ll"], b_score["frame_ll"]) and a_score["ll"] == b_score["ll"]
    st = server.stats()
    assert st["failed"] == 0 and st["completed"] >= 44


def test_map_against_oracle(glib, oracle, server):
    ms = models(1, seed=60)
    mid = server.add_model(*ms[0])
    X = frames(ms[0], 3000, 61)
    r = server.result(server.submit(glib.REQ_MAP, mid, X, tau=16, upW=1, upM=1, upV=1))
    st = oracle.accumulate64(X, *ms[0])
    ow, omu, ovar = oracle.map_update(*ms[0], st, 16, upW=True, upM=True, upV=True)
    assert np.allclose(r["mu"], omu, rtol=1e-4, atol=1e-4)
    assert np.allclose(r["var"], ovar, rtol=1e-4, atol=1e-5)
    assert np.allclose(r["w"], ow, rtol=1e-4, atol=1e-7)
    assert abs(r["ll"] - st["totLL"]) <= 1e-6 * abs(st["totLL"])


def test_errors(glib, server):
    ms = models(1, seed=70)
    mid = server.add_model(*ms[0])
    with pytest.raises(glib.GMMError) as e:
        server.submit(glib.REQ_SCORE, mid + 5, frames(ms[0], 10, 1))
    assert e.value.code == glib.ERR_ARG
    # a request larger than a request arena is refused when it is admitted
    t = server.submit(glib.REQ_SCORE, mid, np.zeros((400_000, D), np.float32))
    with pytest.raises(glib.GMMError) as e:
        server.result(t)
    assert e.value.code == glib.ERR_NOMEM
    bad = (ms[0][0], ms[0][1], np.full_like(ms[0][2], 1e-9))
    with pytest.raises(glib.GMMError) as e:
        server.add_model(*bad)
    assert e.value.code == glib.ERR_MODEL
    # the server keeps serving
    r = server.result(server.submit(glib.REQ_SCORE, mid, frames(ms[0], 100, 2)))
    assert np.isfinite(r["ll"])
