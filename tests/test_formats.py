import numpy as np

from gmm_gb300 import formats, synth


def test_gmm_txt_roundtrip(tmp_path, golden):
    g = golden("example.npz")
    m = formats.GMModel(g["w"], g["mu"], g["var"])
    p = tmp_path / "m.gmm"
    formats.write_gmm_txt(str(p), m)
    r = formats.read_gmm_txt(str(p))
    assert np.allclose(r.w, m.w, rtol=1e-6) and np.allclose(r.mu, m.mu, rtol=1e-6)
    assert np.allclose(r.var, m.var, rtol=1e-6)


def test_gmm_bin_roundtrip_drops_zero_weights(tmp_path):
    w, mu, var = synth.generator_gmm(5, 6, 4)
    w[2] = 0
    m = formats.GMModel(w, mu, var)
    p = tmp_path / "m.bin"
    formats.write_gmm_bin(str(p), m)
    r = formats.read_gmm_bin(str(p))
    keep = w > 0
    assert r.M == 5 and np.array_equal(r.mu, mu[keep]) and np.array_equal(r.var, var[keep])


def test_raw_roundtrip_and_truncation(tmp_path):
    X = synth.rng(1).standard_normal((17, 3)).astype(np.float32)
    p = tmp_path / "x.bin"
    formats.write_raw(str(p), X)
    assert np.array_equal(formats.read_raw(str(p)), X)
    p.write_bytes(p.read_bytes()[:-8])
    import pytest
    with pytest.raises(ValueError):
        formats.read_raw(str(p))


def test_synth_is_seeded():
    a = synth.c1(seed=3, N=1000)
    b = synth.c1(seed=3, N=1000)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    X, w, mu, var = a
    assert X.shape == (1000, 39) and mu.shape == (64, 39) and abs(w.sum() - 1) < 1e-6
