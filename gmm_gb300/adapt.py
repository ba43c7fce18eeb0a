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
    mllrUBMInit: bool = False
    applyTransforms: bool = False
    min_var: float = 1e-6
    verbosity: int = 0
    precision: int = _lib.PREC_FP32


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
        self._X = None
        self._model: GMModel | None = None
        self._W = None
        self.ll_history: list[float] = []

    def SetOptions(self, opt: Options):
        self.opt = opt
        self.dev.set_precision(opt.precision)

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
        self.dev.upload_model(model.w, model.mu, model.var)

    def IterEM(self, model: GMModel, iters: int) -> GMModel:
        """``CModelAdapt::IterEM`` (OL_ModelAdapt.cpp:1276-1296) on the device."""
        o = self.opt
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
        """``CModelAdapt::ComputeW_MLLR`` (OL_ModelAdapt.cpp:1417-1482)."""
        self._ensure_features()
        self._upload(model)
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

    def AdaptModelMLLR(self, model: GMModel, W: np.ndarray) -> GMModel:
        """``CModelAdapt::AdaptModelMLLR`` (OL_ModelAdapt.cpp:1583-1612)."""
        out = model.copy()
        self.dev.set_options(-1e20, 1e-4, self.opt.min_var)
        self.dev.upload_model(out.w, out.mu, out.var)
        self.dev.mllr_apply(W)
        out.w, out.mu, out.var = self.dev.read_model()
        return out

    def AdaptModel(self, ubm: GMModel):
        """``CModelAdapt::AdaptModel`` (OL_ModelAdapt.cpp:1163-1226) for MAP and MLLR."""
        o = self.opt
        if o.adaptType == MAP:
            model = ubm.copy()
            if o.iterCountEM:
                model = self.IterEM(model, o.iterCountEM)
            if o.iterCountMAP:
                model = self.IterMAP(model, ubm, o.iterCountMAP)
            self._model = model
        elif o.adaptType == MLLR:
            self._W = self.IterW_MLLR(ubm, o.iterMLLR)
            if o.applyTransforms:
                self._model = self.AdaptModelMLLR(ubm, self._W)
        else:
            raise NotImplementedError("only MAP (incl. EM with tau = 0) and MLLR are on the "
                                      "diagonal hot path")

    def PickUpClientModel(self) -> GMModel | None:
        m, self._model = self._model, None
        return m

    def PickUpTRNMatrix(self):
        W, self._W = self._W, None
        return W
