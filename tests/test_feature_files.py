"""Feature-file readers (gmm_read_param) for the reference's three formats.

The library's reader is checked bit-exactly against the numpy restatement in
gmm_gb300/formats.py and, where the reference build is available (oracle/_ref), against the
reference's own Param::Load on the same files: SVES, HTK (big-endian) and RAW, with and without
down-sampling, an empty file, a RAW file whose frame count is 0 ("read to the end").
"""
import os

import numpy as np
import pytest

from gmm_gb300 import formats


@pytest.fixture
def files(tmp_path):
    r = np.random.default_rng(1)
    X = r.standard_normal((37, 13)).astype(np.float32) * 5
    paths = {}
    paths["sves"] = str(tmp_path / "a.prm")
    formats.write_sves(paths["sves"], X, cf=np.linspace(0, 1, len(X)))
    paths["htk"] = str(tmp_path / "a.htk")
    formats.write_htk(paths["htk"], X)
    paths["raw"] = str(tmp_path / "a.raw")
    formats.write_raw(paths["raw"], X)
    paths["raw0"] = str(tmp_path / "b.raw")
    with open(paths["raw0"], "wb") as f:  # frame count 0: the reader takes the rest of the file
        f.write(np.array([0, 13], "<i4").tobytes())
        f.write(X.astype("<f4").tobytes())
    paths["empty"] = str(tmp_path / "e.prm")
    formats.write_sves(paths["empty"], np.zeros((0, 13), np.float32))
    return X, paths


@pytest.mark.parametrize("dwn", [1, 2, 3, 5])
def test_readers_match_numpy_and_reference(glib, oracle, files, dwn):
    X, p = files
    cases = [("sves", glib.PRM_SVES, formats.read_sves), ("htk", glib.PRM_HTK, formats.read_htk),
             ("raw", glib.PRM_RAW, formats.read_raw), ("raw0", glib.PRM_RAW, formats.read_raw)]
    for key, kind, np_read in cases:
        got = glib.read_param(p[key], kind, dwn)
        assert np.array_equal(got, X[::dwn]), key
        assert np.array_equal(got, np_read(p[key], dwn)), key
        if oracle.ref_available():
            assert np.array_equal(got, oracle.ref_param_load(p[key], kind, dwn)), key


def test_empty_and_missing(glib, oracle, files):
    _, p = files
    assert glib.read_param(p["empty"], glib.PRM_SVES).shape[0] == 0
    with pytest.raises(glib.GMMError):
        glib.read_param(p["empty"] + ".missing", glib.PRM_SVES)
    if oracle.ref_available():
        assert oracle.ref_param_load(p["empty"] + ".missing", glib.PRM_SVES) is None
    with pytest.raises(glib.GMMError):  # an HTK file is not an SVES file
        glib.read_param(p["htk"], glib.PRM_SVES)
