"""Host-side mirror of the reference's re-estimation driver ``CModelAdapt``
(GMM/lib_bmssr/trainer/OL_ModelAdapt.{h,cpp}) for the diagonal EM / MAP / MLLR routes of
``trainGMM --type 2`` (MAP, with ``--tau 0`` for plain EM) and ``--type 1`` (MLLR).

The loops run on the device: statistics, updates and the model stay resident between
iterations, and only the final model (or transform) comes back. Option names and defaults are
the command-line defaults of ``CModelAdapt::GetOptions`` (OL_ModelAdapt.cpp:2032-2132).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _lib
from .formats import GMModel

FROM_SCRATCH, MLLR, MAP, FMLLR, MLLR_MAP = 0, 1, 2, 3, 4


@dataclass
class Options:
    """Subset of ``CModelAdapt::OPTIONS`` on the diagonal hot path."""
    adaptType: int = MAP
    tau: int = 0
    iterCountEM: int = 0
    iterCountMAP: int = 0
    AdaptMeanBool: bool = False
    AdaptVarBool: bool = False
    AdaptWeightBool: bool = False
    iterMLLR: int = 1
    iterfMLLR: int = 20             # _iter_fMLLR (fixed to 20 in the reference)
    mllrUBMInit: bool = False
    applyTransforms: bool = False
    min_var: float = 1e-6
    splitXpercAtOnce: float = 0.0   # --split-X
    splitTh: float = 0.0            # --split-th
    llTh: float = 0.0               # --ll-Th
    verbosity: int = 0
    robustCov: bool = False         # --robust
    precision: int = _lib.PREC_FP32


_RESET_VAR = np.frombuffer(np.array([0x01010101], np.uint32).tobytes(), np.float32)[0]


def _empty_model(M: int, D: int, full: bool = False) -> GMModel:
    """``GMModel(dim, nummix, full)``: zero weights, components in GMMMixture::Reset state (mean
    0; diagonal variances of bytes 0x01 from memset, full covariances the identity;
    OL_GMModel.cpp:45-83, 120-165)."""
    var = (np.tile(np.eye(D, dtype=np.float32), (M, 1, 1)) if full
           else np.full((M, D), _RESET_VAR, np.float32))
    return GMModel(np.zeros(M, np.float32), np.zeros((M, D), np.float32), var)


def leading_eigenpair(cov: np.ndarray):
    """Largest eigenvalue (float32) and its unit eigenvector (float32) of a symmetric matrix, in
    FP64; the sign makes the largest-magnitude component positive (the eigenvector's sign is not
    fixed by the problem; getEigValVecs, OL_ModelAdapt.cpp:73-160, takes LAPACK's)."""
    lam, vec = np.linalg.eigh(np.asarray(cov, np.float64))
    v = vec[:, -1]
    big = int(np.argmax(np.abs(v)))
    if v[big] < 0:
        v = -v
    return np.float32(lam[-1]), v.astype(np.float32)


def _gauss_stats(model: GMModel, get_list: bool):
    """``CModelAdapt::GetGaussStats`` (OL_ModelAdapt.cpp:951-990): index of the largest weight
    (the highest index among equal maxima), zero-weight indices from the top down, and the
    non-zero indices sorted by decreasing weight in the reference's insertion order."""
    i_max, wm = 0, np.float32(0.0)
    zero, srt = [], []
    for m in range(model.M - 1, -1, -1):
        w = model.w[m]
        if wm < w:
            wm, i_max = w, m
        if w == 0:
            zero.append(m)
            continue
        if get_list:
            k = 0
            while k < len(srt) and model.w[srt[k]] > w:
                k += 1
            srt.insert(k, m)
    return i_max, zero, srt


def _split_gaussian(model: GMModel, m2: int, mnew: int) -> None:
    """``CModelAdapt::splitGaussian`` (OL_ModelAdapt.cpp:612-665): the new component takes the
    covariance, both take half the weight; the means move by +-sqrt(var)/2 (diagonal) or by
    +-sqrt(lambda) v along the leading eigenvector of the covariance (full)."""
    model.var[mnew] = model.var[m2]
    w = np.float32(model.w[m2] / np.float32(2.0))
    model.w[mnew] = w
    model.w[m2] = w
    if model.full:
        lam, v = leading_eigenpair(model.var[m2])
        if lam < 0:
            raise RuntimeError("splitGaussian(): covariance matrix not positive definite!")
        shift = (np.sqrt(lam) * v).astype(np.float32)
    else:
        shift = (np.sqrt(model.var[m2].astype(np.float64)) * 0.5).astype(np.float32)
    model.mu[mnew] = model.mu[m2] + shift
    model.mu[m2] = model.mu[m2] - shift


def _compose(W_sum: np.ndarray, W_new: np.ndarray) -> np.ndarray:
    """``CModelAdapt::UpdateMLLRMatrix`` (OL_ModelAdapt.cpp:1319-1340): [A|b] <- [A_new A |
    A_new b + b_new], accumulated in the reference's loop order."""
    D = W_sum.shape[0]
    out = np.zeros_like(W_sum)
    for k in range(D):
        for x in range(D):
            s = 0.0
            for y in range(D):
                s += W_new[k, y] * W_sum[y, x]
            out[k, x] += s
            out[k, D] += W_new[k, x] * W_sum[x, D]
        out[k, D] += W_new[k, D]
    return out


class ModelAdapt:
    """EM / MAP / MLLR driver on one GB300 handle."""

    def __init__(self, options: Options | None = None, device: int = 0):
        self.opt = options or Options()
        self.dev = _lib.Handle(device)
        self.dev.set_precision(self.opt.precision)
        self.dev.set_robust(self.opt.robustCov)
        self._X = None
        self._model: GMModel | None = None
        self._W = None
        self.ll_history: list[float] = []

    def SetOptions(self, opt: Options):
        self.opt = opt
        self.dev.set_precision(opt.precision)
        self.dev.set_robust(opt.robustCov)

    def InsertData(self, X: np.ndarray):
        self._X = np.ascontiguousarray(X, np.float32)
        self._uploaded = False

    def _ensure_features(self):
        if self._X is None:
            raise RuntimeError("AdaptModel(): Insert adaptation data first!")
        if not getattr(self, "_uploaded", False):
            self.dev.upload_features(self._X)
            self._uploaded = True

    def _acc_flags(self):
        o = self.opt
        f = (_lib.ACC_MEAN if o.AdaptMeanBool else 0) | (_lib.ACC_VAR if o.AdaptVarBool else 0)
        if o.AdaptWeightBool and not o.AdaptMeanBool and not o.AdaptVarBool:
            f |= _lib.ACC_PROBS_ONLY
        return f

    def _upload(self, model: GMModel):
        self.dev.set_options(-1e20, 1e-4, self.opt.min_var)
        model.rearrange()
        if model.full:
            self.dev.upload_model_full(model.w, model.mu, model.var)
        else:
            self.dev.upload_model(model.w, model.mu, model.var)

    def _read(self, model: GMModel):
        model.w, model.mu, model.var = self.dev.read_model_full() if model.full else self.dev.read_model()

    def _iter_full(self, model: GMModel, ubm: GMModel | None, iters: int) -> GMModel:
        """IterEM (ubm None) / IterMAP on a full-covariance model: insertModel (rearrange +
        upload), the E-step with full second-order statistics, UpdateModelEM / UpdateModelMAP."""
        o = self.opt
        self._ensure_features()
        for _ in range(iters):
            self._upload(model)
            if ubm is not None:
                self.dev.set_prior_full(ubm.w, ubm.mu, ubm.var)
            self.dev.accumulate_full_device(self._acc_flags())
            self.ll_history.append(self.dev.read_stats_full()["totLL"])
            if ubm is None or o.tau == 0:
                before = model.copy()
                alive = self.dev.em_update_full(o.AdaptWeightBool, o.AdaptMeanBool, o.AdaptVarBool)
                if alive == 0:  # all Gaussians discarded: keep the initial model
                    model = (ubm if ubm is not None else before).copy()
                    continue
            else:
                self.dev.map_update_full(o.tau, o.AdaptWeightBool, o.AdaptMeanBool, o.AdaptVarBool)
            self._read(model)
        return model

    def IterEM(self, model: GMModel, iters: int) -> GMModel:
        """``CModelAdapt::IterEM`` (OL_ModelAdapt.cpp:1276-1296) on the device."""
        o = self.opt
        if model.full:
            return self._iter_full(model, None, iters)
        self._ensure_features()
        self.dev.set_options(-1e20, 1e-4, o.min_var)
        self.dev.upload_model(model.w, model.mu, model.var)
        ll, _ = self.dev.em_iterate(iters, o.AdaptWeightBool, o.AdaptMeanBool, o.AdaptVarBool)
        self.ll_history.extend(float(v) for v in ll)
        model.w, model.mu, model.var = self.dev.read_model()
        return model

    def IterMAP(self, model: GMModel, ubm: GMModel, iters: int) -> GMModel:
        """``CModelAdapt::IterMAP`` (OL_ModelAdapt.cpp:1298-1317) on the device."""
        o = self.opt
        if model.full:
            return self._iter_full(model, ubm, iters)
        self._ensure_features()
        for _ in range(iters):
            self._upload(model)
            self.dev.set_prior(ubm.w, ubm.mu, ubm.var)
            self.dev.accumulate_device(self._acc_flags())
            self.ll_history.append(self.dev.read_stats()["totLL"])
            if o.tau == 0:
                alive = self.dev.em_update(o.AdaptWeightBool, o.AdaptMeanBool, o.AdaptVarBool)
                if alive == 0:
                    model = ubm.copy()
                    continue
            else:
                self.dev.map_update(o.tau, o.AdaptWeightBool, o.AdaptMeanBool, o.AdaptVarBool)
            model.w, model.mu, model.var = self.dev.read_model()
        return model

    def ComputeW_MLLR(self, model: GMModel, ubm: GMModel) -> np.ndarray:
        """``CModelAdapt::ComputeW_MLLR`` (OL_ModelAdapt.cpp:1417-1482); a full-covariance model
        uses its covariance diagonals (GetMixtureVarDiag)."""
        self._ensure_features()
        self._upload(model)
        if model.full:
            self.dev.set_prior_full(ubm.w, ubm.mu, ubm.var)
            self.dev.accumulate_full_device(_lib.ACC_MEAN)
            return self.dev.mllr_estimate_full(self.opt.mllrUBMInit)
        self.dev.set_prior(ubm.w, ubm.mu, ubm.var)
        self.dev.accumulate_device(_lib.ACC_MEAN)
        return self.dev.mllr_estimate(self.opt.mllrUBMInit)

    def IterW_MLLR(self, ubm: GMModel, iters: int) -> np.ndarray:
        """``CModelAdapt::IterW_MLLR`` (OL_ModelAdapt.cpp:1365-1415)."""
        W = self.ComputeW_MLLR(ubm, ubm)
        if iters > 1:
            sp = self.AdaptModelMLLR(ubm, W)
            for _ in range(1, iters - 1):
                Wt = self.ComputeW_MLLR(sp, ubm)
                sp = self.AdaptModelMLLR(sp, Wt)
                W = _compose(W, Wt)
            Wt = self.ComputeW_MLLR(sp, ubm)
            W = _compose(W, Wt)
        return W

    def _em_step(self, model: GMModel, update: bool):
        """One AccumulateStats + UpdateModelEM of TrainFromScratch: insertModel rearranges the
        model in place, then the device accumulates and (if asked) updates it."""
        self._upload(model)
        if model.full:
            self.dev.accumulate_full_device(_lib.ACC_MEAN | _lib.ACC_VAR)
            st = self.dev.read_stats_full()
        else:
            self.dev.accumulate_device(_lib.ACC_MEAN | _lib.ACC_VAR)
            st = self.dev.read_stats()
        alive = None
        if update:
            alive = self.dev.em_update_full(True, True, True) if model.full else self.dev.em_update(True, True, True)
            self._read(model)
        return st, alive

    def splitMultipleGaussians(self, model: GMModel) -> None:
        """``CModelAdapt::splitMultipleGaussians`` (OL_ModelAdapt.cpp:590-610)."""
        o = self.opt
        i_max, zero, srt = _gauss_stats(model, o.splitXpercAtOnce > 0.0)
        n_split = int(np.ceil(np.float32(o.splitXpercAtOnce) * np.float32(model.M - len(zero))))
        if n_split < 2:
            _split_gaussian(model, i_max, zero[0])
            return
        th = np.float32(o.splitTh) * model.w[i_max]
        for n, (m, z) in enumerate(zip(srt, zero + [None] * max(0, len(srt) - len(zero)))):
            if model.w[m] < th or z is None or n >= n_split:
                break
            _split_gaussian(model, m, z)

    def TrainFromScratch(self, nummix: int, init: GMModel | None = None, fullcov: bool = False) -> GMModel:
        """``CModelAdapt::TrainFromScratch`` (OL_ModelAdapt.cpp:667-821): a global Gaussian, then
        EM iterations on the device alternating with splits of the heaviest Gaussians into free
        slots until nummix components (or a stop rule). fullcov: full covariance matrices (an
        init model, if given, decides: a diagonal one switches the training to diagonal, as the
        reference warns)."""
        o = self.opt
        self._ensure_features()
        if self._X.shape[0] <= 3:
            raise RuntimeError("TrainFromScratch(): Not enough data to model training.")
        D = self._X.shape[1]
        if init is not None:
            fullcov = init.full
        if init is None:
            # global statistics: one component, every posterior 1
            g = GMModel(np.ones(1, np.float32), np.zeros((1, D), np.float32),
                        np.eye(D, dtype=np.float32)[None] if fullcov else np.ones((1, D), np.float32))
            _, alive = self._em_step(g, True)
            if alive == 0:
                raise RuntimeError("trainFromScratch(): amount of data too low to estimate a model, or data are "
                                   "constant!")
            init = g
            max_iter = nummix
        else:
            if nummix <= init.M:
                raise RuntimeError("trainFromScratch(): init model already contains specified number of Gaussians!")
            max_iter = nummix - init.M
        model = _empty_model(nummix, D, fullcov)
        model.w[:init.M], model.mu[:init.M], model.var[:init.M] = init.w, init.mu, init.var
        if nummix < 2:
            max_iter = 0
        iters_em = 2 if (o.iterCountEM < 2 and o.llTh > 0.0) else o.iterCountEM
        lowest = -np.finfo(np.float32).max
        ll = [lowest, lowest, lowest]
        m2 = m3 = None
        non_zero = init.M
        for it in range(max_iter):
            for _ in range(iters_em):
                st, _ = self._em_step(model, False)
                if o.verbosity:  # the reference only computes the average LL when verbose
                    ll[0] = np.float32(st["totLL"] / st["totN"])
                if non_zero > 1:
                    non_zero = (self.dev.em_update_full(True, True, True) if model.full
                                else self.dev.em_update(True, True, True))
                    self._read(model)
                if non_zero < 2:
                    if non_zero < 1:
                        model = init.copy()
                    break
            if non_zero == 0 or non_zero == nummix:
                break
            if o.llTh > 0.0:
                mx = max(ll[1], ll[2])
                if it > 2 and ll[0] - mx < o.llTh:
                    if mx > ll[0]:
                        model = (m2 if mx == ll[1] else m3).copy()
                    break
                m3 = m2.copy() if m2 is not None else _empty_model(0, D, fullcov)
                m2 = model.copy()
                ll[2], ll[1] = ll[1], ll[0]
            if it < max_iter - 1:
                self.splitMultipleGaussians(model)
                non_zero += 1
        model.rearrange()
        self._model = model
        return model

    def AdaptModelMLLR(self, model: GMModel, W: np.ndarray) -> GMModel:
        """``CModelAdapt::AdaptModelMLLR`` (OL_ModelAdapt.cpp:1583-1612)."""
        out = model.copy()
        self.dev.set_options(-1e20, 1e-4, self.opt.min_var)
        if out.full:
            self.dev.upload_model_full(out.w, out.mu, out.var)
            self.dev.mllr_apply_full(W)
            out.w, out.mu, out.var = self.dev.read_model_full()
            return out
        self.dev.upload_model(out.w, out.mu, out.var)
        self.dev.mllr_apply(W)
        out.w, out.mu, out.var = self.dev.read_model()
        return out

    def AdaptModel(self, ubm: GMModel):
        """``CModelAdapt::AdaptModel`` (OL_ModelAdapt.cpp:1163-1226): MAP, MLLR, fMLLR, MLLR+MAP."""
        o = self.opt
        if o.adaptType == MAP:
            model = ubm.copy()
            if o.iterCountEM:
                model = self.IterEM(model, o.iterCountEM)
            if o.iterCountMAP:
                model = self.IterMAP(model, ubm, o.iterCountMAP)
            self._model = model
        elif o.adaptType == FMLLR:
            self._ensure_features()
            self._upload(ubm.copy())
            self._W = (self.dev.fmllr_estimate_full(o.iterfMLLR) if ubm.full
                       else self.dev.fmllr_estimate(o.iterfMLLR))
        elif o.adaptType == MLLR:
            self._W = self.IterW_MLLR(ubm, o.iterMLLR)
            if o.applyTransforms:
                self._model = self.AdaptModelMLLR(ubm, self._W)
        elif o.adaptType == MLLR_MAP:
            # MLLR of the UBM, then AdaptModelMAP of the transformed model with the original
            # UBM as the MAP prior (OL_ModelAdapt.cpp:1190-1205)
            try:
                W = self.IterW_MLLR(ubm, o.iterMLLR)
                model = self.AdaptModelMLLR(ubm, W)
            except _lib.GMMError as e:
                if e.code != _lib.ERR_MLLR:
                    raise
                model = ubm.copy()  # not enough data for MLLR: MAP only, as the reference warns
            if o.iterCountEM:
                model = self.IterEM(model, o.iterCountEM)
            if o.iterCountMAP:
                model = self.IterMAP(model, ubm, o.iterCountMAP)
            self._model = model
        else:
            raise NotImplementedError("adaptation type not built")

    def PickUpClientModel(self) -> GMModel | None:
        m, self._model = self._model, None
        return m

    def PickUpTRNMatrix(self):
        W, self._W = self._W, None
        return W
