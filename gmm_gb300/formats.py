"""Host-side file formats of the reference (diagonal models and RAW features).

* GMM text format, as written by ``GMModel::WriteTXT`` / read by ``GMModel::ReadTXT``
  (lib_bmssr/model/OL_GMModel.cpp:475-547, 627-753): dimension, D normalisation
  coefficients, number of components, then per component a weight line (optionally
  ``<MIX_OCCUP> value``), a blank line, D means, a blank line, D variances, a blank line.
  Components with zero weight are not written.
* GMM binary format ``GMModel::WriteBIN`` / ``ReadBIN`` (OL_GMModel.cpp:551-624, 757-853):
  ``"GMM-DB-VN"``, int16 dimension (negative for full covariance), D float normalisation
  coefficients, int16 M, M float weights, then per component D means and D variances.
* RAW features (``Param::LoadRaw``, lib_bmssr/param/OL_Param.cpp:358-463):
  int32 nsamples, int32 dimension, float32 data.

Only diagonal covariances are in scope; a full-covariance file raises ``ValueError``.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np


@dataclass
class GMModel:
    """Diagonal GMM: ``w[M]``, ``mu[M, D]``, ``var[M, D]`` (float32), plus the file's
    normalisation coefficients (carried through, never used by the estimator)."""
    w: np.ndarray
    mu: np.ndarray
    var: np.ndarray
    norm: np.ndarray = field(default=None)

    def __post_init__(self):
        self.w = np.ascontiguousarray(self.w, np.float32)
        self.mu = np.ascontiguousarray(self.mu, np.float32)
        self.var = np.ascontiguousarray(self.var, np.float32)
        if self.norm is None:
            self.norm = np.ones(self.mu.shape[1], np.float32)

    @property
    def M(self) -> int:
        return int(self.w.shape[0])

    @property
    def D(self) -> int:
        return int(self.mu.shape[1])

    def copy(self) -> "GMModel":
        return GMModel(self.w.copy(), self.mu.copy(), self.var.copy(), self.norm.copy())

    def rearrange(self) -> np.ndarray:
        """Move zero-weight components behind the others, in place, exactly as
        ``GMModel::RearrangeMixtures`` (OL_GMModel.cpp:857-885): the non-zero ones keep
        their order; the k-th zero-weight component goes to slot M-1-k. Returns the
        permutation (slot -> original index)."""
        M = self.M
        order = np.empty(M, np.int64)
        nz, z = 0, 1
        for m in range(M):
            if self.w[m] > 0:
                order[nz] = m
                nz += 1
            else:
                order[M - z] = m
                z += 1
        self.w = np.ascontiguousarray(self.w[order])
        self.mu = np.ascontiguousarray(self.mu[order])
        self.var = np.ascontiguousarray(self.var[order])
        return order


def read_gmm_txt(path: str) -> GMModel:
    with open(path) as f:
        lines = [ln.strip() for ln in f]
    i = 0
    D = int(lines[i]); i += 1
    norm = np.array([float(lines[i + k]) for k in range(D)], np.float32); i += D
    M = int(lines[i]); i += 1
    w, mu, var = [], [], []
    for _ in range(M):
        head = lines[i].split()
        if len(head) > 1 and head[1] == "F":
            raise ValueError("full-covariance models are outside the diagonal hot path")
        w.append(float(head[0])); i += 2
        mu.append([float(lines[i + k]) for k in range(D)]); i += D + 1
        var.append([float(lines[i + k]) for k in range(D)]); i += D + 1
    return GMModel(np.array(w), np.array(mu), np.array(var), norm)


def write_gmm_txt(path: str, g: GMModel) -> None:
    with open(path, "w") as f:
        f.write(f"{g.D}\n")
        for v in g.norm:
            f.write("%15e\n" % v)
        keep = [m for m in range(g.M) if g.w[m] != 0]
        f.write(f"{len(keep)}\n")
        for m in keep:
            f.write("%15e\n\n" % g.w[m])
            for v in g.mu[m]:
                f.write("%15e\n" % v)
            f.write("\n")
            for v in g.var[m]:
                f.write("%15e\n" % v)
            f.write("\n")


def read_gmm_bin(path: str) -> GMModel:
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:9] != b"GMM-DB-VN":
        raise ValueError("not a GMM-DB-VN file")
    (D,) = struct.unpack_from("<h", buf, 9)
    if D < 0:
        raise ValueError("full-covariance models are outside the diagonal hot path")
    off = 11
    norm = np.frombuffer(buf, "<f4", D, off); off += 4 * D
    (M,) = struct.unpack_from("<h", buf, off); off += 2
    w = np.frombuffer(buf, "<f4", M, off); off += 4 * M
    body = np.frombuffer(buf, "<f4", 2 * M * D, off).reshape(M, 2, D)
    return GMModel(w.copy(), body[:, 0].copy(), body[:, 1].copy(), norm.copy())


def write_gmm_bin(path: str, g: GMModel) -> None:
    keep = [m for m in range(g.M) if g.w[m] > 0]
    with open(path, "wb") as f:
        f.write(b"GMM-DB-VN")
        f.write(struct.pack("<h", g.D))
        f.write(np.asarray(g.norm, "<f4").tobytes())
        f.write(struct.pack("<h", len(keep)))
        f.write(np.asarray(g.w[keep], "<f4").tobytes())
        for m in keep:
            f.write(np.asarray(g.mu[m], "<f4").tobytes())
            f.write(np.asarray(g.var[m], "<f4").tobytes())


def read_raw(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        buf = f.read()
    N, D = struct.unpack_from("<ii", buf, 0)
    if N < 0 or D <= 0 or 8 + 4 * N * D > len(buf):
        raise ValueError(f"truncated or malformed RAW feature file (N={N}, D={D})")
    return np.frombuffer(buf, "<f4", N * D, 8).reshape(N, D).copy()


def write_raw(path: str, X: np.ndarray) -> None:
    X = np.ascontiguousarray(X, "<f4")
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", X.shape[0], X.shape[1]))
        f.write(X.tobytes())


def write_loglikes_txt(path: str, ll: np.ndarray) -> None:
    """Per-frame log-likelihoods in the text layout of ``saveMat`` (IOMats.h:204-220):
    header "1 N", then the values on one line."""
    with open(path, "w") as f:
        f.write(f"1 {len(ll)}\n")
        f.write(" ".join("%g" % v for v in ll))
        f.write("\n")
