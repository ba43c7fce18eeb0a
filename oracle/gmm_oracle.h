/*
 * CPU oracle for the GMM E-step / M-step hot path. TEST INFRASTRUCTURE ONLY: the tests, the
 * smoke check and the CPU-baseline leg of bench.py call it as the checker; the product
 * (gmm_gb300) never links or loads it.
 *
 * Two restatements of the reference algorithm (GMMTeam/GMM, lib_bmssr):
 *   orc32_*  "port": the reference CPU estimator's float semantics, operation by operation
 *            (float log-likelihood with no fused multiply-add, sequential log-add with the
 *            15-nat cutoff, float posteriors, float products accumulated in double, the same
 *            frame split over threads and the same ordered merge). It is pinned against the
 *            reference itself compiled from its sources (oracle/_ref) and against the
 *            reference's golden file example/data.logL.
 *   orc64_*  FP64 oracle: the same discrete rules (zero-weight skip, minGamma prune, min_var
 *            floor, minimum-occupancy kill, weight denominator = all frames) in double with an
 *            exact max-shifted log-sum-exp (no cutoff).
 * Model arrays are flat: w[M], mu[M*D], var[M*D] (diagonal covariances), in the order the
 * caller gives; components with w <= 0 are skipped exactly as the reference skips the
 * zero-weight components that GMModel::RearrangeMixtures moved behind the others.
 */
#ifndef GMM_ORACLE_H
#define GMM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* accumulation flags (match the C-ABI of the product) */
#define ORC_ACC_MEAN 1
#define ORC_ACC_VAR 2
#define ORC_ACC_PROBS_ONLY 4

typedef struct {
  float minLogLike; /* -1e20 */
  float minGamma;   /* 1e-4 */
  float min_var;    /* 1e-6 */
  int threads;      /* reference _numThreads */
} orc_opts;

/* GMModel::RearrangeMixtures (OL_GMModel.cpp:857-885): order[k] = original index at slot k. */
int orc_rearrange_order(int M, const float* w, int* order);

/* GMMStatsEstimator::compVecsLogLikeMT (OL_GMMStatsEstimator.cpp:811-879). Returns 0, or
 * 1 if a variance is below min_var (insertModel throws there), 2 on bad arguments. */
int orc32_loglikes(const float* X, long long N, int D, int M, const float* w, const float* mu,
                   const float* var, const orc_opts* o, float* out, int* stability_trouble);

/* GMMStatsEstimator::accumulateStatsMT (OL_GMMStatsEstimator.cpp:884-971) into zeroed
 * n[M], F[M*D], S[M*D]; *totLL and *totN receive the accumulated totals. */
int orc32_accumulate(const float* X, long long N, int D, int M, const float* w, const float* mu,
                     const float* var, const orc_opts* o, int flags, double* n, double* F,
                     double* S, double* totLL, long long* totN);

/* FP64 oracle: exact LSE, same pruning rules. */
int orc64_loglikes(const float* X, long long N, int D, int M, const float* w, const float* mu,
                   const float* var, const orc_opts* o, double* out);
int orc64_accumulate(const float* X, long long N, int D, int M, const float* w, const float* mu,
                     const float* var, const orc_opts* o, int flags, double* n, double* F,
                     double* S, double* totLL, long long* totN);

/* CModelAdapt::UpdateModelEM (OL_ModelAdapt.cpp:823-949), in place on float arrays.
 * Returns the number of components left with non-zero weight. */
int orc_em_update(int M, int D, float* w, float* mu, float* var, const double* n,
                  const double* F, const double* S, long long totN, int upW, int upM, int upV,
                  float min_var);

/* FP64 EM update (no float rounding of intermediate means): outputs in double. */
int orc64_em_update(int M, int D, const float* w, const double* n, const double* F,
                    const double* S, long long totN, int upW, int upM, int upV, double min_var,
                    double* ow, double* omu, double* ovar);

/* CModelAdapt::UpdateModelMAP with tau > 0 (OL_ModelAdapt.cpp:1024-1106), in place on the
 * adapted model (w, mu, var) against the prior (ubm_*). */
void orc_map_update(int M, int D, float* w, float* mu, float* var, const float* ubm_w,
                    const float* ubm_mu, const float* ubm_var, const double* n, const double* F,
                    const double* S, long long totN, int tau, int upW, int upM, int upV,
                    float min_var);

/* Global MLLR mean transform, one iteration (CModelAdapt::ComputeW_MLLR + ComputeKiGi_MLLR +
 * prepareKiGiInitMatrices + MATRIX::_Invert_Gen, OL_ModelAdapt.cpp:1417-1581,
 * Matrix4_LMa.cpp:2232-2300). W is D x (D+1) row-major. Returns 0, or 3 if the
 * CheckInvertibility conditions fail (OL_ModelAdapt.cpp:1851-1878). */
int orc_mllr_w(int M, int D, const float* mu, const float* var, const float* ubm_mu,
               const float* ubm_var, const double* n, const double* F, int ubm_init,
               float min_var, double* W);

/* CModelAdapt::AdaptModelMLLR (OL_ModelAdapt.cpp:1583-1612): omu = A*mu + b. */
void orc_mllr_apply(int M, int D, const float* mu, const double* W, float* omu);

/* Pivot-free Gauss-Jordan inverse in place (MATRIX::_Invert_Gen semantics). */
void orc_gj_invert(int n, double* a);

/* Full covariances (cov: M*D*D row-major, symmetric). FP64: Cholesky, |L^-1 (x-mu)|^2, exact
 * LSE; Sp = packed upper triangle [M][D(D+1)/2]. Return 4 if a covariance is not positive
 * definite (the reference's getCovInverse throws). */
int orc64_full_prepare(int M, int D, const float* w, const float* cov, double* chol, double* logdet);
int orc64_full_loglikes(const float* X, long long N, int D, int M, const float* w, const float* mu,
                        const float* cov, double* out);
int orc64_full_accumulate(const float* X, long long N, int D, int M, const float* w, const float* mu,
                          const float* cov, const orc_opts* o, int flags, double* n, double* F,
                          double* Sp, double* totLL, long long* totN);
/* The reference's full-covariance EM and MAP updates (float model, double arithmetic). */
int orc_full_em_update(int M, int D, float* w, float* mu, float* cov, const double* n,
                       const double* F, const double* Sp, long long totN, int upW, int upM, int upV);
void orc_full_map_update(int M, int D, float* w, float* mu, float* cov, const float* ubm_w,
                         const float* ubm_mu, const float* ubm_cov, const double* n, const double* F,
                         const double* Sp, long long totN, int tau, int upW, int upM, int upV);

/* fMLLR: the E-step of a diagonal model with packed full second-order statistics (FP64), and
 * ComputeW_fMLLR from such statistics (W: D x (D+1) row-major). Return 0, 3 (CheckInvertibility)
 * or 5 (EstimateAb_fmllr: negative discriminant or zero root). */
int orc64_accumulate_fullstats(const float* X, long long N, int D, int M, const float* w,
                               const float* mu, const float* var, const orc_opts* o, double* n,
                               double* F, double* Sp, double* totLL, long long* totN);
int orc_fmllr_w(int M, int D, const float* mu, const float* var, const double* n, const double* F,
                const double* Sp, long long totN, int iters, double* W);

/* --robust: auxiliary statistics (FP64 posteriors; full = 1 for a full-covariance model, var
 * then [M][D][D]), GetNIndFrames + MakeRobustStats (S modified in place, nind out; returns 6
 * for a zero global variance) and the EM updates with the kill rule on nind. */
int orc64_aux_stats(const float* X, long long N, int D, int M, const float* w, const float* mu,
                    const float* var, int full, const orc_opts* o, double* aux, double* aux2, double* aux3);
int orc_make_robust(int M, int D, int full, const double* n, const double* F, double* S,
                    const double* aux, const double* aux2, const double* aux3, double* nind);
int orc_em_update_nind(int M, int D, float* w, float* mu, float* var, const double* n,
                       const double* F, const double* S, long long totN, int upW, int upM, int upV,
                       float min_var, const double* nind);
int orc_full_em_update_nind(int M, int D, float* w, float* mu, float* cov, const double* n,
                            const double* F, const double* Sp, long long totN, int upW, int upM, int upV,
                            const double* nind);

#ifdef __cplusplus
}
#endif
#endif
