"""The allocation-free entry point (gmm_accumulate_noalloc) against the regular one.

Callers that cannot let the library allocate device memory -- a framework that owns the device
memory pool, or a loop where a cudaMalloc/cudaFree is not allowed once it runs -- pass their own
device inputs and outputs and get the same statistics as gmm_accumulate, computed in a fixed
scratch array compiled into the library. This file is collected last so that a failure here
leaves every other test already run. Tolerance: the same float arithmetic per frame; only the
grouping of FP64 partial sums differs (different frame chunks), so 1e-12 relative."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run_noalloc(glib, torch, X, w, mu, var, flags, stream=None):
    lib = glib.load()
    dev = torch.device("cuda:0")
    dX = torch.from_numpy(X).to(dev)
    dw, dmu, dvar = (torch.from_numpy(a).to(dev) for a in (w, mu, var))
    M, D = mu.shape
    out = torch.full((M * (1 + 2 * D) + 1,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = lib.gmm_accumulate_noalloc(dX.data_ptr(), X.shape[0], D, M, dw.data_ptr(), dmu.data_ptr(),
                                    dvar.data_ptr(), -1e20, 1e-4, 1e-6, flags, out.data_ptr(), stream)
    assert rc == 0, lib.gmm_last_error(None)
    o = out.cpu().numpy()
    return dict(n=o[:M], F=o[M:M + M * D].reshape(M, D), S=o[M + M * D:M + 2 * M * D].reshape(M, D),
                totLL=o[-1])


def test_noalloc_matches_accumulate_twice(glib):
    torch = pytest.importorskip("torch")
    from gmm_gb300 import synth
    X, w, mu, var = synth.config_em(41, 50_000, 39, 32, 256)
    h = glib.Handle(0)
    h.upload_model(w, mu, var)
    h.upload_features(X)
    ref = h.accumulate(glib.ACC_MEAN | glib.ACC_VAR)
    h.close()
    for _ in range(2):  # two calls in a row share (and must re-initialise) the scratch
        got = run_noalloc(glib, torch, X, w, mu, var, glib.ACC_MEAN | glib.ACC_VAR)
        assert abs(got["totLL"] - ref["totLL"]) <= 1e-12 * abs(ref["totLL"])
        for k in ("n", "F", "S"):
            assert np.allclose(got[k], ref[k], rtol=1e-12, atol=1e-9), k


@pytest.mark.parametrize("M,D,N", [(4096, 64, 5000), (2048, 128, 5000), (4096, 128, 6000),
                                   (4096, 128, 300)])
def test_noalloc_largest_models(glib, M, D, N):
    """The largest models the scratch takes: the per-slice partial statistics are sized from
    M * (1 + 2D), so at M = 4096, D = 128 one slice fills 8.4 MB and a frame chunk holds about
    1300 frames -- N = 6000 runs several chunks through the same scratch, N = 300 one short
    chunk. Two calls in a row, against gmm_accumulate on the same inputs."""
    torch = pytest.importorskip("torch")
    from gmm_gb300 import synth
    X, w, mu, var = synth.config_em(43 + D, N, D, 16, M)
    h = glib.Handle(0)
    h.upload_model(w, mu, var)
    h.upload_features(X)
    ref = h.accumulate(glib.ACC_MEAN | glib.ACC_VAR)
    h.close()
    for _ in range(2):
        got = run_noalloc(glib, torch, X, w, mu, var, glib.ACC_MEAN | glib.ACC_VAR)
        assert abs(got["totLL"] - ref["totLL"]) <= 1e-12 * abs(ref["totLL"])
        for k in ("n", "F", "S"):
            assert np.all(np.isfinite(got[k])), k
            assert np.allclose(got[k], ref[k], rtol=1e-12, atol=1e-9), k


def test_noalloc_rejects_oversize(glib):
    torch = pytest.importorskip("torch")
    lib = glib.load()
    d = torch.zeros(16, device="cuda:0")
    rc = lib.gmm_accumulate_noalloc(d.data_ptr(), 1, 200, 2, d.data_ptr(), d.data_ptr(), d.data_ptr(),
                                    -1e20, 1e-4, 1e-6, 3, d.data_ptr(), None)
    assert rc == glib.ERR_UNSUPPORTED
    assert b"128" in lib.gmm_last_error(None)
