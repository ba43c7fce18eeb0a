"""Sparse tile schedule of the tensor-core statistics against the dense schedule.

The schedule skips the (128-frame tile, 128-component chunk) pairs whose posteriors are all
pruned at minGamma, after grouping the components into spatially coherent chunks and sorting
the frames by the chunks they keep posteriors in. The skipped pairs contribute nothing in the
dense schedule either; the sums differ only in rounding. In sorted tiles a component gathers
more posterior mass per tile than in the given frame order (its frames sit together), so the
tensor core's round-toward-zero accumulation of a tile's sums loses more low bits: the two
schedules agree to 1e-4 of each statistic's scale and each agrees with the FP64 oracle within
the usual tensor-core tolerance (1e-4). The total log-likelihood (the grouped components
change the order of the log-sum-exp's chunks) agrees within 1e-9 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _handle(glib, sched):
    h = glib.Handle(0)
    h.set_precision(glib.PREC_TC)
    h.set_autotune(False)
    h.set_tile_schedule(sched)
    return h


def _close(a, b, rel, rel_S=None):
    for k in ("n", "F", "S"):
        scale = np.maximum(np.abs(b[k]), np.abs(b["n"])[:, None] if k != "n" else 1.0) + 1.0
        err = (np.abs(a[k] - b[k]) / scale).max()
        assert err <= (rel_S if (k == "S" and rel_S) else rel), (k, err)


@pytest.mark.parametrize("D,M,N,flags", [
    (39, 2048, 60_000, 3),   # 16 chunks: the UBM shape, second-order statistics
    (39, 2048, 60_000, 1),   # mean-only statistics
    (20, 300, 7_777, 3),     # 3 chunks, a ragged last chunk and a ragged last tile
    (39, 64, 5_000, 3),      # one chunk
    (6, 1, 3_000, 3),        # one component: every frame keeps it
    (39, 4096, 20_000, 3),   # 32 chunks: the largest schedule (four sort passes)
])
def test_schedule_matches_dense(glib, oracle, D, M, N, flags):
    from gmm_gb300 import synth
    X, w, mu, var = synth.config_em(700 + M + D, N, D, max(2, min(M, 64) // 2), M)
    out = []
    for sched in (True, False):
        h = _handle(glib, sched)
        h.upload_model(w, mu, var)
        h.upload_features(X)
        out.append(h.accumulate(flags))
        out.append(h.accumulate(flags))  # again on the same handle (planes resident)
        h.close()
    a, a2, b, _ = out
    # the grouped component order changes the order of the log-sum-exp's chunks
    assert abs(a["totLL"] - b["totLL"]) <= 1e-9 * abs(b["totLL"])
    assert a["totLL"] == a2["totLL"]
    for k in ("n", "F", "S"):
        assert np.array_equal(a[k], a2[k]), k  # deterministic
    _close(a, b, 1e-4, 3e-4)
    o = oracle.accumulate64(X, w, mu, var, flags=flags)
    _close(a, o, 1e-4, 3e-4)


def test_schedule_em_iterations_and_streamed(glib):
    """Captured EM iterations (static shapes: the active count lives on the device) and the
    E-step over host frames use the schedule too."""
    from gmm_gb300 import synth
    X, w, mu, var = synth.config_em(91, 80_000, 39, 64, 512)
    res = []
    for sched in (True, False):
        h = _handle(glib, sched)
        h.upload_model(w, mu, var)
        h.upload_features(X)
        ll, _ = h.em_iterate(4)
        res.append((ll, h.read_model()))
        h.close()
    (la, ma), (lb, mb) = res
    assert np.allclose(la, lb, rtol=1e-7, atol=0), (la, lb)
    for x, y in zip(ma, mb):
        assert np.allclose(x, y, rtol=1e-4, atol=1e-5)
    out = []
    for sched in (True, False):
        h = _handle(glib, sched)
        h.upload_model(w, mu, var)
        h.accumulate_host(X)
        out.append(h.read_stats())
        h.close()
    _close(out[0], out[1], 1e-4)
