"""Host-side mirror of the reference estimator interface, backed by the sm_103a engine.

``GMMStatsEstimatorGB300`` offers the members of the reference's
``GMMStatsEstimator<TS, TV, TL>`` (GMM/lib_bmssr/trainer/OL_GMMStatsEstimator.h:57-182) that
the trainer and the scorer use: the public knobs ``_minLogLike``, ``_minGamma``, ``_min_var``,
``_numThreads``, ``_verbosity``, ``_fNumStabilityTroubles``; ``insertModel``,
``setModelToBeUsed``, ``setAccFlags`` / ``resetAccFlags``, ``setSameDataFlag``,
``accumulateStatsMT``, ``compVecsLogLikeMT`` and ``getEstimationType``. Argument meaning and
error behaviour follow the reference: ``insertModel`` moves zero-weight components of the
caller's model behind the others (the reference mutates the model the same way) and raises on a
variance below ``_min_var``; ``accumulateStatsMT`` adds into the caller's ``GMMStats`` (the
reference only ever ``+=``-s into it) and allocates it when unallocated.

There is no CPU fallback: every call goes to the CUDA library, and constructing the estimator
without a GPU raises.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .formats import GMModel


class GMMStats:
    """Mirror of ``GMMStats<double>`` (lib_bmssr/model/OL_GMMStats.h:44-148) for diagonal
    models: per-component ``mixProb`` (n), first-order ``mean`` (F) and second-order ``var`` (S)
    sums, the accumulated total log-likelihood and frame count."""

    def __init__(self, dim: int = 0, nummix: int = 0, allocMeans: bool = True,
                 allocVars: bool = False, allocFullVars: bool = False):
        self._allocated = False
        self._allM = self._allV = self._allFV = False
        if nummix:
            self.alloc(dim, nummix, allocMeans, allocVars, allocFullVars)

    def alloc(self, dim, nummix, allocMeans=True, allocVars=False, allocFullVars=False):
        """allocFullVars: second-order statistics of a full-covariance model, the packed upper
        triangle [nummix, dim(dim+1)/2] (GMMStats' _varsize, OL_GMMStats.cpp:233-239)."""
        self._dim, self._M = dim, nummix
        self._allM, self._allV = bool(allocMeans), bool(allocVars or allocFullVars)
        self._allFV = bool(allocFullVars)
        self.n = np.zeros(nummix)
        self.F = np.zeros((nummix, dim))
        self.S = np.zeros((nummix, dim * (dim + 1) // 2 if self._allFV else dim))
        self._totLogLike = 0.0
        self._totalAccSamples = 0
        self._allocated = True

    def reset(self):
        self.n[:] = 0
        self.F[:] = 0
        self.S[:] = 0
        self._totLogLike = 0.0
        self._totalAccSamples = 0

    def isAllocated(self):
        return self._allocated

    def getMixNum(self):
        return self._M

    def getDim(self):
        return self._dim

    def getTotLogLike(self):
        return self._totLogLike

    def getTotAccSamples(self):
        return self._totalAccSamples

    def getProb(self, m):
        return self.n[m]

    def getMean(self, m):
        return self.F[m]

    def getVar(self, m):
        return self.S[m]

    def save(self, filename: str, saveTxt: bool) -> None:
        """``GMMStats<double>::save`` file layout (formats.write_gmm_stats)."""
        from . import formats
        formats.write_gmm_stats(filename, saveTxt, self.n, self.F if self._allM else None,
                                self.S if self._allV else None)

    def load(self, filename: str, loadTxt: bool) -> None:
        """``GMMStats<double>::load``: (re)allocates to the file's sizes and fills it."""
        from . import formats
        n, F, S = formats.read_gmm_stats(filename, loadTxt)
        D = F.shape[1] if F is not None else (S.shape[1] if S is not None else 0)
        full = S is not None and F is not None and S.shape[1] != D
        self.alloc(D, len(n), F is not None, S is not None and not full, full)
        self.n[:] = n
        if F is not None:
            self.F[:] = F
        if S is not None:
            self.S[:] = S

    def hasFullCov(self):
        return getattr(self, "_allFV", False)

    def __iadd__(self, o: "GMMStats"):
        if self._M != o._M:
            raise ValueError("operator+= : Inconsistent statistics differing in number of mixtures!")
        self.n += o.n
        if self._allM and o._allM:
            self.F += o.F
        if self._allV and o._allV:
            self.S += o.S
        self._totalAccSamples += o._totalAccSamples
        self._totLogLike += o._totLogLike
        return self


class GMMStatsEstimatorGB300:
    """Drop-in for the reference estimator on one GB300 (see module docstring)."""

    def __init__(self, GPU_id: int = 0, precision: int = _lib.PREC_FP32):
        self._minLogLike = -1e20
        self._minGamma = 1e-4
        self._min_var = 1e-6
        self._numThreads = 1          # accepted for interface parity; the GPU ignores it
        self._NAccBlocks_CUDA = 8     # idem (partials are per CTA on this engine)
        self._memoryBuffDataGB = 0.0
        self._memoryBuffDataGB_GPU = 0.0
        self._verbosity = 1
        self._fNumStabilityTroubles = False
        self._fSameDataProvided = False
        self._flagsSet = False
        self._fMixProbOnly = self._fMean = self._fVar = False
        self._models: list[GMModel] = []
        self._model: GMModel | None = None
        self._dev = _lib.Handle(GPU_id)
        self._dev.set_precision(precision)
        self._features_key = None
        self._estimType = "GB300 " + ("TC" if precision == _lib.PREC_TC else "FP32")

    # -- reference API -------------------------------------------------------------
    def getEstimationType(self) -> str:
        return self._estimType

    def insertModel(self, model: GMModel, first: bool = True):
        if first:
            self._models = []
            self._dev.clear_model_slots()
        elif self._models and model.D != self._models[0].D:
            raise RuntimeError("Models (GMMs) have to have same dimensions")
        model.rearrange()
        bad = np.zeros(1, bool) if model.full else (model.var[model.w > 0] < self._min_var)
        if bad.any():
            raise RuntimeError("insertModel(): model contains very low variances "
                               f"[{float(model.var[model.w > 0][bad].min())}]!")
        self._models.append(model)
        n = len(self._models) - 1
        if not model.full:  # the group's diagonal models stay resident on the device
            self._dev.upload_model_slot(n, model.w, model.mu, model.var)
        self.setModelToBeUsed(n)

    def setModelToBeUsed(self, n: int):
        """OL_GMMStatsEstimator.cpp:318-325: switch to model n of the group (a device-to-device
        copy of its resident slot; a full-covariance model is uploaded again)."""
        self._model = self._models[n]
        self._dev.set_options(self._minLogLike, self._minGamma, self._min_var)
        if self._model.full:  # GMM_ERR_MODEL (RuntimeError) if a covariance is not positive definite
            self._dev.upload_model_full(self._model.w, self._model.mu, self._model.var)
        else:
            self._dev.select_model(n)

    def setAccFlags(self, mixProbsOnly, meanStats, varStats, varFull=False, auxStats=False):
        if auxStats:
            raise NotImplementedError("robust auxiliary statistics are not built")
        self._flagsSet = True
        # full second-order statistics imply variance statistics (OL_GMMStatsEstimator.cpp:410-412)
        self._fMixProbOnly, self._fMean = bool(mixProbsOnly), bool(meanStats)
        self._fVar = bool(varStats) or bool(varFull)

    def resetAccFlags(self):
        self._flagsSet = False

    def setSameDataFlag(self):
        self._fSameDataProvided = True

    def _flags(self, gmms: GMMStats) -> int:
        if not self._flagsSet:
            self._fMixProbOnly = not gmms._allM and not gmms._allV
            self._fMean, self._fVar = gmms._allM, gmms._allV
        f = 0
        if self._fMixProbOnly:
            f |= _lib.ACC_PROBS_ONLY
        if self._fMean:
            f |= _lib.ACC_MEAN
        if self._fVar:
            f |= _lib.ACC_VAR
        return f

    def _features(self, vectors, NSamples, dim):
        X = np.asarray(vectors)
        if X.ndim != 2 or X.shape[1] != dim or X.shape[0] < NSamples:
            raise ValueError("vectors must be an [N, dim] array")
        X = X[:NSamples]
        key = (X.__array_interface__["data"][0], X.shape)
        if not (self._fSameDataProvided and key == self._features_key):
            self._dev.upload_features(X)
            self._features_key = key
        self._fSameDataProvided = False

    def accumulateStatsMT(self, vectors, NSamples: int, dim: int, gmms: GMMStats):
        if self._model is None:
            raise RuntimeError("accumulateStats(): None model inserted!")
        if dim != self._model.D:
            raise RuntimeError("accumulateStats(): Inconsistent model & feature dimensions!")
        flags = self._flags(gmms)
        full = self._model.full
        if not gmms.isAllocated():
            gmms.alloc(dim, self._model.M, self._fMean or self._fVar, self._fVar and not full,
                       self._fVar and full)
        self._features(vectors, NSamples, dim)
        st = self._dev.accumulate_full(flags) if full else self._dev.accumulate(flags)
        part = GMMStats(dim, self._model.M, gmms._allM, gmms._allV and not full, gmms._allV and full)
        part.n[:] = st["n"]
        part.F[:] = st["F"]
        part.S[:] = st["Sp"] if full else st["S"]
        part._totLogLike = st["totLL"]
        part._totalAccSamples = st["totN"]
        gmms += part

    def compVecsLogLikeMT(self, vecs, NSamples: int, dim: int, outLogLikes=None):
        if self._model is None:
            raise RuntimeError("compVecsLogLikeMT(): None model inserted!")
        if dim != self._model.D:
            raise RuntimeError("compVecsLogLike(): Inconsistent model & feature dimensions!")
        self._features(vecs, NSamples, dim)
        ll = self._dev.loglikes_full() if self._model.full else self._dev.loglikes()
        self._fNumStabilityTroubles = bool((ll == np.float32(self._minLogLike)).any())
        if outLogLikes is not None:
            outLogLikes[:NSamples] = ll
            return outLogLikes
        return ll

    def getNewInstance(self):
        return GMMStatsEstimatorGB300(precision=_lib.PREC_TC if "TC" in self._estimType else _lib.PREC_FP32)
