"""Bounded device waits of the tensor-core kernels: expiry is reported, and the handle recovers.

Every mbarrier wait of the tensor-core pipeline roles gives up after a limit (about 2 s by
default), raises the CTA's abort flag, lets the copies and MMAs still in flight finish, frees its
tensor memory and leaves an error flag that the host turns into GMM_ERR_TIMEOUT. The test hook
gmm_set_wait_limit shortens the limit to a few hundred clock cycles -- shorter than any TMA copy
from HBM takes -- so the first wait on data gives up: no fault, no hang, just the expiry path.
Afterwards, with the default limit, the same handle must give exactly the statistics of a fresh
handle (same decomposition: autotuning off in both), i.e. nothing half-built survives."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _handle(glib, X, w, mu, var, sched=False):
    h = glib.Handle(0)
    h.set_precision(glib.PREC_TC)
    h.set_autotune(False)
    h.set_tile_schedule(sched)
    h.upload_model(w, mu, var)
    h.upload_features(X)
    return h


# D = 39: the dense statistics kernel (K = 80), in the given frame order and over the sparse
# tile schedule (work items on a fixed grid); D = 60: the sparse one (K = 128, second order)
@pytest.mark.parametrize("D,M,N,sched", [(39, 64, 3000, False), (39, 300, 3000, True), (60, 40, 2000, False)])
def test_tc_wait_expiry_reports_timeout_then_recovers(glib, D, M, N, sched):
    from gmm_gb300 import synth
    X, w, mu, var = synth.config_em(300 + D, N, D, 8, M)
    fresh = _handle(glib, X, w, mu, var, sched)
    ref = fresh.accumulate(glib.ACC_MEAN | glib.ACC_VAR)
    ref_mean = fresh.accumulate(glib.ACC_MEAN)
    fresh.close()

    h = _handle(glib, X, w, mu, var, sched)
    h.set_wait_limit(300)
    for flags in (glib.ACC_MEAN | glib.ACC_VAR, glib.ACC_MEAN):
        with pytest.raises(glib.GMMError) as e:
            h.accumulate(flags)
        assert e.value.code == glib.ERR_TIMEOUT, str(e.value)
        assert "bounded device wait" in str(e.value)
    h.set_wait_limit(0)  # back to the default
    got = h.accumulate(glib.ACC_MEAN | glib.ACC_VAR)
    got_mean = h.accumulate(glib.ACC_MEAN)
    h.close()
    for a, b in ((got, ref), (got_mean, ref_mean)):
        assert a["totLL"] == b["totLL"]
        for k in ("n", "F", "S"):
            assert np.array_equal(a[k], b[k]), k
