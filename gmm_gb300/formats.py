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

Full-covariance models (``GMModel(dim, nummix, true)``: Var holds D x D per component) carry
``var`` as [M, D, D]: text weight lines end in " F" and each covariance row is written as its
diagonal element followed by the D row values; the binary dimension is stored negated.
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

    @property
    def full(self) -> bool:
        """Full covariances (var is [M, D, D])."""
        return self.var.ndim == 3

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
    full = False
    for _ in range(M):
        head = lines[i].split()
        full = len(head) > 1 and head[1] == "F"
        w.append(float(head[0])); i += 2
        mu.append([float(lines[i + k]) for k in range(D)]); i += D + 1
        if full:  # each row: the diagonal element, then the D values of the row
            var.append([[float(v) for v in lines[i + k].split()[1:D + 1]] for k in range(D)])
        else:
            var.append([float(lines[i + k]) for k in range(D)])
        i += D + 1
    return GMModel(np.array(w), np.array(mu), np.array(var), norm)


def write_gmm_txt(path: str, g: GMModel) -> None:
    with open(path, "w") as f:
        f.write(f"{g.D}\n")
        for v in g.norm:
            f.write("%15e\n" % v)
        keep = [m for m in range(g.M) if g.w[m] != 0]
        f.write(f"{len(keep)}\n")
        for m in keep:
            f.write(("%15e F\n\n" if g.full else "%15e\n\n") % g.w[m])
            for v in g.mu[m]:
                f.write("%15e\n" % v)
            f.write("\n")
            if g.full:
                for k in range(g.D):
                    f.write("%15e" % g.var[m, k, k] + "".join(" %15e" % v for v in g.var[m, k]) + "\n")
            else:
                for v in g.var[m]:
                    f.write("%15e\n" % v)
            f.write("\n")


def read_gmm_bin(path: str) -> GMModel:
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:9] != b"GMM-DB-VN":
        raise ValueError("not a GMM-DB-VN file")
    (D,) = struct.unpack_from("<h", buf, 9)
    full = D < 0
    D = abs(D)
    V = D * D if full else D
    off = 11
    norm = np.frombuffer(buf, "<f4", D, off); off += 4 * D
    (M,) = struct.unpack_from("<h", buf, off); off += 2
    w = np.frombuffer(buf, "<f4", M, off); off += 4 * M
    body = np.frombuffer(buf, "<f4", M * (D + V), off).reshape(M, D + V)
    var = body[:, D:].reshape(M, D, D) if full else body[:, D:]
    return GMModel(w.copy(), body[:, :D].copy(), var.copy(), norm.copy())


def write_gmm_bin(path: str, g: GMModel) -> None:
    keep = [m for m in range(g.M) if g.w[m] > 0]
    with open(path, "wb") as f:
        f.write(b"GMM-DB-VN")
        f.write(struct.pack("<h", -g.D if g.full else g.D))
        f.write(np.asarray(g.norm, "<f4").tobytes())
        f.write(struct.pack("<h", len(keep)))
        f.write(np.asarray(g.w[keep], "<f4").tobytes())
        for m in keep:
            f.write(np.asarray(g.mu[m], "<f4").tobytes())
            f.write(np.asarray(g.var[m], "<f4").tobytes())


def _downsample(X: np.ndarray, dwnsmp: int) -> np.ndarray:
    """Param's down-sampling: frames 0, d, 2d, ... (N / d + (N % d > 0) frames)."""
    return X[::dwnsmp].copy() if dwnsmp > 1 else X


def read_raw(path: str, dwnsmp: int = 1) -> np.ndarray:
    """RAW_PRM_IN (Param::LoadRaw, param/OL_Param.cpp:345-450): int32 frames, int32 dim, floats;
    frames < 1 means the rest of the file."""
    with open(path, "rb") as f:
        buf = f.read()
    N, D = struct.unpack_from("<ii", buf, 0)
    if D > 0 and N < 1:
        N = (len(buf) - 8) // D // 4
    if N < 0 or D <= 0 or 8 + 4 * N * D > len(buf):
        raise ValueError(f"truncated or malformed RAW feature file (N={N}, D={D})")
    return _downsample(np.frombuffer(buf, "<f4", N * D, 8).reshape(N, D).copy(), dwnsmp)


def write_raw(path: str, X: np.ndarray) -> None:
    X = np.ascontiguousarray(X, "<f4")
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", X.shape[0], X.shape[1]))
        f.write(X.tobytes())


def write_sves(path: str, X: np.ndarray, cf: np.ndarray | None = None) -> None:
    """SVES_PRM_IN (Param::Save / Param::Load, param/OL_Param.cpp:245-340): "SV-ES-PARAM",
    int32 dim, int32 frames, float CF[frames], float frames[frames][dim]."""
    X = np.ascontiguousarray(X, "<f4")
    N, D = X.shape
    cf = np.ones(N, "<f4") if cf is None else np.ascontiguousarray(cf, "<f4")
    with open(path, "wb") as f:
        f.write(b"SV-ES-PARAM")
        f.write(struct.pack("<ii", D, N))
        f.write(cf.tobytes())
        f.write(X.tobytes())


def read_sves(path: str, dwnsmp: int = 1) -> np.ndarray:
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:11] != b"SV-ES-PARAM":
        raise ValueError(f"{path}: format different from SV-ES-PARAM")
    D, N = struct.unpack_from("<ii", buf, 11)
    if N <= 0 or D <= 0:
        return np.zeros((0, 0), np.float32)
    off = 19 + 4 * N
    return _downsample(np.frombuffer(buf, "<f4", N * D, off).reshape(N, D).copy(), dwnsmp)


def write_htk(path: str, X: np.ndarray, sample_period: int = 100000, parm_kind: int = 9) -> None:
    """HTK_PRM_IN (Param::LoadHTK, param/OL_Param.cpp:474-560): big-endian int32 frames, int32
    sample period, int16 bytes per frame, int16 parameter kind, big-endian float frames."""
    X = np.ascontiguousarray(X, ">f4")
    N, D = X.shape
    with open(path, "wb") as f:
        f.write(struct.pack(">iihh", N, sample_period, 4 * D, parm_kind))
        f.write(X.tobytes())


def read_htk(path: str, dwnsmp: int = 1) -> np.ndarray:
    with open(path, "rb") as f:
        buf = f.read()
    N, _, nb, _ = struct.unpack_from(">iihh", buf, 0)
    D = nb // 4
    if N <= 0 or D <= 0:
        return np.zeros((0, 0), np.float32)
    return _downsample(np.frombuffer(buf, ">f4", N * D, 12).reshape(N, D).astype(np.float32), dwnsmp)


def write_gmm_stats(path: str, txt: bool, n, F=None, S=None, dtype=np.float64) -> None:
    """``GMMStats<T>::save`` (model/OL_GMMStats.cpp:657-778), diagonal statistics: seven int32
    (mixProb saved, means saved, vars saved, full vars saved, dim, varsize, nummix), then per
    component n, F[dim], S[dim] as ``dtype``; the text layout has the same header line, a blank
    line, then per component "n", " F ...", " S ...", blank, in ostream's default format (%g)."""
    n = np.asarray(n, dtype)
    M = len(n)
    D = np.asarray(F).shape[1] if F is not None else (np.asarray(S).shape[1] if S is not None else 0)
    varsize = np.asarray(S).shape[1] if S is not None else 0
    full = int(S is not None and varsize != D)  # packed full second-order statistics
    hdr = [1, int(F is not None), int(S is not None), full, D, varsize, M]
    if txt:
        with open(path, "w") as f:
            f.write(" ".join(map(str, hdr)) + "\n\n")
            for m in range(M):
                f.write("%g\n" % n[m])
                if F is not None:
                    f.write("".join(" %g" % v for v in np.asarray(F, dtype)[m]) + "\n")
                if S is not None:
                    f.write("".join(" %g" % v for v in np.asarray(S, dtype)[m]) + "\n")
                f.write("\n")
        return
    with open(path, "wb") as f:
        f.write(np.asarray(hdr, "<i4").tobytes())
        for m in range(M):
            f.write(np.asarray(n[m], dtype).tobytes())
            if F is not None:
                f.write(np.asarray(F, dtype)[m].tobytes())
            if S is not None:
                f.write(np.asarray(S, dtype)[m].tobytes())


def read_gmm_stats(path: str, txt: bool, dtype=np.float64):
    """``GMMStats<T>::load`` (OL_GMMStats.cpp:493-655): returns (n, F or None, S or None); S is
    [M, varsize] (the packed upper triangle for full-covariance statistics)."""
    if txt:
        with open(path) as f:
            tok = f.read().split()
        hdr = [int(v) for v in tok[:7]]
        vals = np.array(tok[7:], np.float64)
    else:
        with open(path, "rb") as f:
            buf = f.read()
        hdr = list(np.frombuffer(buf, "<i4", 7))
        vals = np.frombuffer(buf, dtype, offset=28).astype(np.float64)
    mp, mean, var, full, D, varsize, M = hdr
    rec = int(mp) + int(mean) * D + int(var) * varsize
    body = vals[:M * rec].reshape(M, rec)
    n = body[:, 0] if mp else None
    F = body[:, int(mp):int(mp) + D] if mean else None
    S = body[:, int(mp) + int(mean) * D:] if var else None
    return n, F, S


def write_loglikes_txt(path: str, ll: np.ndarray) -> None:
    """Per-frame log-likelihoods in the text layout of ``saveMat`` (IOMats.h:169-215): header
    "1 N", then every value followed by a space, a newline, and a final empty line."""
    with open(path, "w") as f:
        f.write(f"1 {len(ll)}\n")
        f.write("".join("%g " % v for v in ll))
        f.write("\n\n")


def read_mat(path: str, txt: bool) -> np.ndarray:
    """``loadMat`` of a ``saveMat`` file: text "x y" then x*y values, or binary int32 x, int32 y
    and x*y float32 values. Returns an (x, y) float32 array."""
    if txt:
        with open(path) as f:
            tok = f.read().split()
        x, y = int(tok[0]), int(tok[1])
        return np.array(tok[2:2 + x * y], np.float32).reshape(x, y)
    with open(path, "rb") as f:
        buf = f.read()
    x, y = struct.unpack_from("<ii", buf, 0)
    return np.frombuffer(buf, "<f4", x * y, 8).reshape(x, y).copy()


def read_trn(path: str) -> np.ndarray:
    """An MLLR transform file of ``CModelAdapt::SaveTRNMatrices`` (OL_ModelAdapt.cpp:1900-1928):
    " MLLR", " 1<TAB>x y", then x rows of y values."""
    with open(path) as f:
        lines = f.read().split("\n")
    if lines[0].strip() not in ("MLLR", "fMLLR"):
        raise ValueError(f"{path}: not a transform file")
    _, x, y = (int(v) for v in lines[1].split())
    vals = " ".join(lines[2:]).split()
    return np.array(vals[:x * y], np.float64).reshape(x, y)
