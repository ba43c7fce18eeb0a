"""Seeded synthetic workloads for the GMM hot path.

No public dataset is involved: the reference ships only a toy example, and the benchmark
configurations are defined by their shapes and value distributions. Every generator takes an
explicit seed and uses numpy's PCG64 generator, so the same call gives the same arrays on any
host.

Configurations (frames x components x dims):
  C1  plain EM: 64-component generator (w ~ Dirichlet(1), mu ~ N(0, 2^2),
      var ~ LogNormal(0, 0.5)), N = 100k, D = 39; fit M = 64 from a random-frame init.
  C2  UBM EM at scale: 512-component generator, N = 10M, D = 39; fit M = 2048.
  C3  batched MAP: UBM M = 1024, D = 60; speakers draw from the UBM with 16 of its means
      shifted; frame counts lognormal clipped to [200, 30000].
  C4  batched MLLR: UBM M = 2048, D = 39; speakers' frames are A x + b of UBM samples,
      A = I + 0.1 N(0,1), b ~ N(0, 0.5); frame counts U[1000, 20000].
  C5  serving: 200 resident GMMs (M = 1024, D = 60); scoring lengths lognormal in
      [100, 10000], adaptation lengths in [500, 30000].
"""
from __future__ import annotations

import numpy as np


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def generator_gmm(seed: int, M: int, D: int, mean_sd: float = 2.0, var_sigma: float = 0.5):
    """Random diagonal GMM: w ~ Dirichlet(1), mu ~ N(0, mean_sd^2), var ~ LogNormal(0, s)."""
    r = rng(seed)
    w = r.dirichlet(np.ones(M)).astype(np.float32)
    mu = (r.standard_normal((M, D)) * mean_sd).astype(np.float32)
    var = np.exp(r.standard_normal((M, D)) * var_sigma).astype(np.float32)
    return w, mu, var


def sample_gmm(seed: int, w, mu, var, N: int, chunk: int = 1 << 20) -> np.ndarray:
    """N frames from the diagonal GMM, float32 [N, D], frames in random component order."""
    r = rng(seed)
    M, D = mu.shape
    p = np.asarray(w, np.float64)
    p = p / p.sum()
    X = np.empty((N, D), np.float32)
    sd = np.sqrt(np.asarray(var, np.float32))
    for s in range(0, N, chunk):
        e = min(N, s + chunk)
        comp = r.choice(M, size=e - s, p=p)
        z = r.standard_normal((e - s, D), dtype=np.float32)
        z *= sd[comp]
        z += mu[comp]
        X[s:e] = z
    return X


def generator_gmm_full(seed: int, M: int, D: int, mean_sd: float = 2.0, corr: float = 0.6):
    """Random full-covariance GMM: w ~ Dirichlet(1), mu ~ N(0, mean_sd^2), cov = S C S with a
    random correlation structure C = (B B^T + D I) normalised to unit diagonal (B ~ N(0, corr^2))
    and scales S ~ LogNormal(0, 0.4). Returns float32 w [M], mu [M, D], cov [M, D, D]."""
    r = rng(seed)
    w = r.dirichlet(np.ones(M)).astype(np.float32)
    mu = (r.standard_normal((M, D)) * mean_sd).astype(np.float32)
    cov = np.empty((M, D, D), np.float32)
    for m in range(M):
        B = r.standard_normal((D, D)) * corr
        A = B @ B.T + D * np.eye(D)
        d = 1.0 / np.sqrt(np.diag(A))
        C = A * d[:, None] * d[None, :]
        s = np.exp(r.standard_normal(D) * 0.4)
        Cm = (C * s[:, None] * s[None, :]).astype(np.float32)
        cov[m] = 0.5 * (Cm + Cm.T)
    return w, mu, cov


def sample_gmm_full(seed: int, w, mu, cov, N: int) -> np.ndarray:
    """N frames from the full-covariance GMM, float32 [N, D]."""
    r = rng(seed)
    M, D = mu.shape
    p = np.asarray(w, np.float64)
    p = p / p.sum()
    comp = r.choice(M, size=N, p=p)
    L = np.linalg.cholesky(np.asarray(cov, np.float64))
    z = r.standard_normal((N, D))
    X = np.empty((N, D), np.float32)
    for m in range(M):  # per component: x = L_m z + mu_m
        idx = np.nonzero(comp == m)[0]
        X[idx] = (z[idx] @ L[m].T + mu[m]).astype(np.float32)
    return X


def random_frame_init(seed: int, X: np.ndarray, M: int):
    """Random-init model: M random frames as means, global variance, uniform weights
    (the initialisation the reference README recommends)."""
    r = rng(seed)
    N, D = X.shape
    idx = r.choice(N, size=M, replace=N < M)
    mu = X[idx].astype(np.float32).copy()
    # global variance in float64, over at most 1M frames
    sub = X if N <= (1 << 20) else X[r.choice(N, size=1 << 20, replace=False)]
    gv = sub.astype(np.float64).var(axis=0)
    var = np.tile(gv.astype(np.float32), (M, 1))
    w = np.full(M, 1.0 / M, np.float32)
    return w, mu, var


def config_em(seed: int, N: int, D: int, M_gen: int, M_fit: int):
    """C1/C2-style workload: (X, init_w, init_mu, init_var)."""
    gw, gmu, gvar = generator_gmm(seed, M_gen, D)
    X = sample_gmm(seed + 1, gw, gmu, gvar, N)
    w, mu, var = random_frame_init(seed + 2, X, M_fit)
    return X, w, mu, var


def c1(seed: int = 1, N: int = 100_000):
    return config_em(seed, N, 39, 64, 64)


def c2(seed: int = 2, N: int = 10_000_000):
    return config_em(seed, N, 39, 512, 2048)


def speaker_lengths(seed: int, S: int, lo: int, hi: int, dist: str = "lognormal",
                    median: float = 3000.0, sigma: float = 1.0) -> np.ndarray:
    r = rng(seed)
    if dist == "uniform":
        return r.integers(lo, hi + 1, size=S).astype(np.int64)
    n = np.exp(np.log(median) + sigma * r.standard_normal(S))
    return np.clip(np.round(n), lo, hi).astype(np.int64)


def c3(seed: int = 3, S: int = 1000, M: int = 1024, D: int = 60, lo: int = 200,
       hi: int = 30000, shift_comps: int = 16):
    """Batched MAP workload: UBM, concatenated speaker frames, per-speaker offsets."""
    uw, umu, uvar = generator_gmm(seed, M, D)
    lens = speaker_lengths(seed + 1, S, lo, hi)
    offs = np.zeros(S + 1, np.int64)
    offs[1:] = np.cumsum(lens)
    X = np.empty((int(offs[-1]), D), np.float32)
    r = rng(seed + 2)
    for s in range(S):
        mu_s = umu.copy()
        comps = r.choice(M, size=shift_comps, replace=False)
        mu_s[comps] += r.standard_normal((shift_comps, D)).astype(np.float32)
        X[offs[s]:offs[s + 1]] = sample_gmm(seed * 100003 + s, uw, mu_s, uvar, int(lens[s]))
    return X, offs, (uw, umu, uvar)


def c4(seed: int = 4, S: int = 500, M: int = 2048, D: int = 39, lo: int = 1000, hi: int = 20000):
    """Batched MLLR workload: UBM, concatenated affine-transformed speaker frames, offsets,
    and the true per-speaker transforms (A, b)."""
    uw, umu, uvar = generator_gmm(seed, M, D)
    lens = speaker_lengths(seed + 1, S, lo, hi, dist="uniform")
    offs = np.zeros(S + 1, np.int64)
    offs[1:] = np.cumsum(lens)
    X = np.empty((int(offs[-1]), D), np.float32)
    r = rng(seed + 2)
    A = np.empty((S, D, D), np.float32)
    b = np.empty((S, D), np.float32)
    for s in range(S):
        A[s] = np.eye(D, dtype=np.float32) + 0.1 * r.standard_normal((D, D)).astype(np.float32)
        b[s] = (r.standard_normal(D) * np.sqrt(0.5)).astype(np.float32)
        Z = sample_gmm(seed * 100003 + s, uw, umu, uvar, int(lens[s]))
        X[offs[s]:offs[s + 1]] = Z @ A[s].T + b[s]
    return X, offs, (uw, umu, uvar), (A, b)
