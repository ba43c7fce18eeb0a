"""Generates the golden fixtures in this directory from the reference itself.

Run where the reference sources are present (they are read in place, never copied):

    python tests/golden/make_golden.py [--ref-root <reference GMM project root>]

It builds ``oracle/_ref/libgmmref.so`` (the reference CPU estimator and CModelAdapt compiled
from their own sources, see oracle/Makefile) and records its outputs on small inputs:

* ``example.npz``  -- the first 1000 frames of the reference's example/data.bin, the
  example/myModel.gmm model, the matching 6-digit values of example/data.logL, and the
  reference's full-precision per-frame log-likelihoods and E-step statistics (1 and 4 threads).
* ``em_small.npz`` -- seeded C1-style data (N=2048, D=39, 16 components): three EM iterations
  of CModelAdapt::IterEM (per-iteration total log-likelihood and final model), and the first
  E-step's statistics at 4 threads.
* ``edge.npz``     -- zero-weight components (reordering), a single-component model, N < 100
  (single-thread path), an outlier frame (numerical-stability branch), D = 1, and an EM update
  that kills an under-occupied component.
* ``map_mllr.npz`` -- mean-only MAP (tau = 16) and one global MLLR transform, with and without
  the UBM-based initialisation.
* ``train.npz``    -- TrainFromScratch with four option sets.
* ``train_full.npz`` -- TrainFromScratch with full covariances (one split per round, and several).
* ``full.npz``     -- full covariances: per-frame log-likelihoods of the first 1000 frames of
  example/data.bin under example/myModelFC.gmm (4 threads) and their E-step statistics; three EM
  iterations (weights, means, covariances) and one MAP iteration (tau = 16, all parameters) of
  a seeded full-covariance model. The reference's single-precision LAPACK calls go through the
  restatement in oracle/ref/shim/acml.h.
* ``mllr_map.npz`` -- MLLR+MAP (adaptation type 4): one global MLLR transform, then one MAP
  iteration (tau = 16, means and variances) of the transformed UBM against the original UBM.
* ``robust.npz``   -- --robust: the auxiliary statistics (one thread) of a diagonal and a
  full-covariance model, two robust EM iterations of each, and one robust MAP iteration
  (tau = 16, means and variances) of a diagonal UBM.
* ``full_mllr.npz`` -- global MLLR of a seeded full-covariance UBM (M = 16, D = 8), with and
  without the UBM-based initialisation: W and the transformed means; and its fMLLR transform.
* ``fmllr.npz``    -- fMLLR (ComputeW_fMLLR, 20 passes) of a diagonal UBM (M = 32, D = 12) from
  one speaker of seeded affinely transformed UBM samples: the transform and the E-step
  statistics (packed full second order) it was computed from.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from gmm_gb300 import formats, synth  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=O.REF_ROOT)
    a = ap.parse_args()
    O.REF_SRC = os.path.join(a.ref_root, "lib_bmssr")
    O.build(ref=True)

    # ---- example/ ---------------------------------------------------------------
    ex = os.path.join(a.ref_root, "example")
    X = formats.read_raw(os.path.join(ex, "data.bin"))[:1000]
    g = formats.read_gmm_txt(os.path.join(ex, "myModel.gmm"))
    with open(os.path.join(ex, "data.logL")) as f:
        f.readline()
        ll_file = np.array(f.read().split()[:1000], np.float64)
    ll_ref = O.ref_loglikes(X, g.w, g.mu, g.var, threads=4)
    s1 = O.ref_accumulate(X, g.w, g.mu, g.var, threads=1)
    s4 = O.ref_accumulate(X, g.w, g.mu, g.var, threads=4)
    np.savez_compressed(os.path.join(HERE, "example.npz"), X=X, w=g.w, mu=g.mu, var=g.var,
                        ll_file=ll_file, ll_ref=ll_ref,
                        n1=s1["n"], F1=s1["F"], S1=s1["S"], totLL1=s1["totLL"],
                        n4=s4["n"], F4=s4["F"], S4=s4["S"], totLL4=s4["totLL"])

    # ---- EM on seeded C1-style data --------------------------------------------
    X, w, mu, var = synth.config_em(11, 2048, 39, 16, 16)
    st = O.ref_accumulate(X, w, mu, var, threads=4)
    ew, emu, evar, ell = O.ref_em(X, w, mu, var, 3, threads=4)
    np.savez_compressed(os.path.join(HERE, "em_small.npz"), X=X, w=w, mu=mu, var=var,
                        n=st["n"], F=st["F"], S=st["S"], totLL=st["totLL"],
                        em_ll=ell, em_w=ew, em_mu=emu, em_var=evar)

    # ---- edge cases -------------------------------------------------------------
    out = {}
    gw, gmu, gvar = synth.generator_gmm(21, 8, 6)
    Xe = synth.sample_gmm(22, gw, gmu, gvar, 600)
    wz = gw.copy(); wz[[1, 5]] = 0.0
    wz /= wz.sum()
    s = O.ref_accumulate(Xe, wz, gmu, gvar, threads=3)
    out.update(zw_X=Xe, zw_w=wz, zw_mu=gmu, zw_var=gvar, zw_order=s["order"], zw_n=s["n"],
               zw_F=s["F"], zw_S=s["S"], zw_totLL=s["totLL"])
    s = O.ref_accumulate(Xe, gw[:1] * 0 + 1, gmu[:1], gvar[:1], threads=2)
    out.update(m1_n=s["n"], m1_F=s["F"], m1_S=s["S"], m1_totLL=s["totLL"])
    s = O.ref_accumulate(Xe[:50], gw, gmu, gvar, threads=4)
    out.update(n50_n=s["n"], n50_F=s["F"], n50_S=s["S"], n50_totLL=s["totLL"])
    Xo = Xe[:200].copy(); Xo[17] = 1e19
    s = O.ref_accumulate(Xo, gw, gmu, gvar, threads=2)
    out.update(out_X=Xo, out_n=s["n"], out_F=s["F"], out_S=s["S"], out_totLL=s["totLL"])
    out.update(out_ll=O.ref_loglikes(Xo, gw, gmu, gvar, threads=2))
    X1 = Xe[:, :1].copy()
    s = O.ref_accumulate(X1, gw, gmu[:, :1], gvar[:, :1], threads=2)
    out.update(d1_n=s["n"], d1_F=s["F"], d1_S=s["S"], d1_totLL=s["totLL"])
    # an init whose last component sits far from the data: EM kills it (occupancy < 2)
    Xk, wk, muk, vark = synth.config_em(23, 800, 6, 4, 5)
    muk[4] = 50.0
    kw, kmu, kvar, kll = O.ref_em(Xk, wk, muk, vark, 2, threads=2)
    out.update(kill_X=Xk, kill_w0=wk, kill_mu0=muk, kill_var0=vark, kill_w=kw, kill_mu=kmu,
               kill_var=kvar, kill_ll=kll)
    np.savez_compressed(os.path.join(HERE, "edge.npz"), **out)

    # ---- MAP and MLLR -----------------------------------------------------------
    uw, umu, uvar = synth.generator_gmm(31, 32, 12)
    Xs = synth.sample_gmm(32, uw, umu + 0.3, uvar, 4000)
    mw, mmu, mvar, mll = O.ref_map(Xs, uw, umu, uvar, 16, iters=1, upM=True, threads=2)
    W0, amu0 = O.ref_mllr(Xs, uw, umu, uvar, ubm_init=False, threads=2)
    W1, amu1 = O.ref_mllr(Xs, uw, umu, uvar, ubm_init=True, threads=2)
    np.savez_compressed(os.path.join(HERE, "map_mllr.npz"), X=Xs, w=uw, mu=umu, var=uvar,
                        map_w=mw, map_mu=mmu, map_var=mvar, map_ll=mll,
                        mllr_W0=W0, mllr_mu0=amu0, mllr_W1=W1, mllr_mu1=amu1)
    for fn in sorted(os.listdir(HERE)):
        if fn.endswith(".npz"):
            print(fn, os.path.getsize(os.path.join(HERE, fn)))

    train_fixture()
    train_full_fixture()
    full_fixture(a.ref_root)
    fmllr_fixture()
    mllr_map_fixture()
    robust_fixture()
    full_mllr_fixture()


def full_fixture(ref_root):
    """Full-covariance outputs of the reference build (see the module docstring)."""
    ex = os.path.join(ref_root, "example")
    X = formats.read_raw(os.path.join(ex, "data.bin"))[:1000]
    g = formats.read_gmm_txt(os.path.join(ex, "myModelFC.gmm"))
    out = {"ex_X": X, "ex_w": g.w, "ex_mu": g.mu, "ex_cov": g.var}
    out["ex_ll"] = O.ref_full_loglikes(X, g.w, g.mu, g.var, threads=4)
    st = O.ref_full_accumulate(X, g.w, g.mu, g.var, threads=1)
    out.update(ex_n=st["n"], ex_F=st["F"], ex_Sp=st["Sp"], ex_totLL=st["totLL"])
    w, mu, cov = synth.generator_gmm_full(41, 6, 10)
    Xs = synth.sample_gmm_full(42, w, mu + 0.3, cov, 3000)
    out.update(X=Xs, w=w, mu=mu, cov=cov)
    ew, emu, ecov, ell = O.ref_full_adapt(Xs, w, mu, cov, 0, 3, threads=2)
    out.update(em_w=ew, em_mu=emu, em_cov=ecov, em_ll=ell)
    mw, mmu, mcov, mll = O.ref_full_adapt(Xs, w, mu, cov, 16, 1, threads=2)
    out.update(map_w=mw, map_mu=mmu, map_cov=mcov, map_ll=mll)
    np.savez_compressed(os.path.join(HERE, "full.npz"), **out)


def full_mllr_fixture():
    w, mu, cov = synth.generator_gmm_full(51, 16, 8)
    X = synth.sample_gmm_full(52, w, mu + 0.4, cov, 3000)
    W0, mu0 = O.ref_full_mllr(X, w, mu, cov)
    W1, mu1 = O.ref_full_mllr(X, w, mu, cov, ubm_init=True)
    fW = O.ref_fmllr_full(X, w, mu, cov)
    np.savez_compressed(os.path.join(HERE, "full_mllr.npz"), X=X, w=w, mu=mu, cov=cov, W0=W0, mu0=mu0, W1=W1,
                        mu1=mu1, fW=fW)


def robust_fixture():
    e = dict(np.load(os.path.join(HERE, "em_small.npz")))
    f = dict(np.load(os.path.join(HERE, "full.npz")))
    mm = dict(np.load(os.path.join(HERE, "map_mllr.npz")))
    out = {}
    a = O.ref_aux_accumulate(e["X"], e["w"], e["mu"], e["var"])
    out.update(diag_aux=a["aux"], diag_aux2=a["aux2"], diag_aux3=a["aux3"])
    a = O.ref_aux_accumulate(f["X"], f["w"], f["mu"], f["cov"], full=True)
    out.update(full_aux=a["aux"], full_aux2=a["aux2"], full_aux3=a["aux3"])
    w, mu, var, ll = O.ref_robust_adapt(e["X"], e["w"], e["mu"], e["var"], 0, 2)
    out.update(diag_em_w=w, diag_em_mu=mu, diag_em_var=var, diag_em_ll=ll)
    w, mu, cov, ll = O.ref_robust_adapt(f["X"], f["w"], f["mu"], f["cov"], 0, 2, full=True)
    out.update(full_em_w=w, full_em_mu=mu, full_em_cov=cov, full_em_ll=ll)
    w, mu, var, ll = O.ref_robust_adapt(mm["X"], mm["w"], mm["mu"], mm["var"], 16, 1, upW=False)
    out.update(map_w=w, map_mu=mu, map_var=var)
    np.savez_compressed(os.path.join(HERE, "robust.npz"), **out)


def mllr_map_fixture():
    g = dict(np.load(os.path.join(HERE, "map_mllr.npz")))
    w, mu, var = O.ref_adapt_model(g["X"], g["w"], g["mu"], g["var"], 4, tau=16, it_map=1, upM=True, upV=True,
                                   threads=2)
    np.savez_compressed(os.path.join(HERE, "mllr_map.npz"), w=w, mu=mu, var=var)


def fmllr_fixture():
    X, offs, (uw, umu, uvar), _ = synth.c4(5, 2, 32, 12, 3000, 4000)
    X = X[offs[0]:offs[1]]
    W, st = O.ref_fmllr(X, uw, umu, uvar, threads=1)
    np.savez_compressed(os.path.join(HERE, "fmllr.npz"), X=X, w=uw, mu=umu, var=uvar, W=W, n=st["n"], F=st["F"],
                        Sp=st["Sp"], totLL=st["totLL"])


def train_full_fixture():
    """TrainFromScratch with full covariances (the split along the leading eigenvector; the
    reference build's ssyevr is the restated stand-in of oracle/ref/shim/acml.h)."""
    w, mu, cov = synth.generator_gmm_full(61, 4, 6)
    X = synth.sample_gmm_full(62, w, mu, cov, 3000)
    out = {"X": X}
    for name, kw in {"one": dict(nummix=4, iters_em=3),
                     "multi": dict(nummix=6, iters_em=3, split_x=0.5, split_th=0.2)}.items():
        rw, rmu, rcov = O.ref_train_full(X, **kw)
        out.update({f"{name}_w": rw, f"{name}_mu": rmu, f"{name}_cov": rcov})
    np.savez_compressed(os.path.join(HERE, "train_full.npz"), **out)


def train_fixture():
    """TrainFromScratch (OL_ModelAdapt.cpp:667-821) by the reference build on seeded data."""
    gw, gmu, gvar = synth.generator_gmm(31, 6, 5)
    X = synth.sample_gmm(32, gw, gmu, gvar, 3000)
    out = {"X": X}
    cases = {"one": dict(nummix=6, iters_em=3),
             "multi": dict(nummix=8, iters_em=3, split_x=0.5, split_th=0.2),
             "llth_quiet": dict(nummix=8, iters_em=2, ll_th=0.01, verbosity=0),
             "llth_verbose": dict(nummix=8, iters_em=2, ll_th=0.01, verbosity=1)}
    for name, kw in cases.items():
        w, mu, var = O.ref_train(X, **kw)
        out.update({f"{name}_w": w, f"{name}_mu": mu, f"{name}_var": var})
    np.savez_compressed(os.path.join(HERE, "train.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--full-only":
        O.build(ref=True)
        full_fixture(O.REF_ROOT)
    elif len(sys.argv) > 1 and sys.argv[1] == "--train-full-only":
        O.build(ref=True)
        train_full_fixture()
    elif len(sys.argv) > 1 and sys.argv[1] == "--robust-only":
        O.build(ref=True)
        robust_fixture()
    elif len(sys.argv) > 1 and sys.argv[1] == "--mllr-map-only":
        O.build(ref=True)
        mllr_map_fixture()
    elif len(sys.argv) > 1 and sys.argv[1] == "--fmllr-only":
        O.build(ref=True)
        fmllr_fixture()
    else:
        main()
