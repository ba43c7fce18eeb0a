/*
 * gmm_gb300 -- C ABI of the GB300 (sm_103a) GMM statistics engine.
 *
 * One handle = one CUDA stream on one device with a device-resident model, feature block,
 * statistics and scratch. Every entry point returns a status (GMM_OK = 0); on failure
 * gmm_last_error(h) gives the message. Calls on one handle must not run concurrently from
 * several host threads; different handles are independent. All calls are synchronous from the
 * caller's point of view (they return after the device work finished) unless stated otherwise.
 *
 * The entry points replace the reference's thin GPU layer GMMStatsEstimator_GPU
 * (GMM/lib_bmssr/trainer/CU_GMMStatsEstimator_CUDA.h:125-183) and the host estimator above it
 * (GMMStatsEstimator_CUDA, OL_GMMStatsEstimator_CUDA.h:39-105); the re-estimation entry points
 * replace CModelAdapt's UpdateModelEM / UpdateModelMAP / MLLR routines
 * (GMM/lib_bmssr/trainer/OL_ModelAdapt.cpp). Citations below give the exact member each one
 * stands in for.
 *
 * Layouts: features X are row-major float32 [N][D]; a model is w[M], mu[M][D], var[M][D]
 * (diagonal covariances) in the caller's component order. Components with w <= 0 are skipped,
 * which is what the reference does after GMModel::RearrangeMixtures moved them behind the
 * others; statistics come back in the caller's order (zero for skipped components).
 */
#ifndef GMM_GB300_H
#define GMM_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gmm_ctx* gmm_handle;

/* status codes */
#define GMM_OK 0
#define GMM_ERR_ARG 1         /* bad argument (null pointer, size out of range) */
#define GMM_ERR_CUDA 2        /* CUDA runtime error; the message names the call */
#define GMM_ERR_STATE 3       /* call out of order (e.g. no model or features uploaded) */
#define GMM_ERR_MODEL 4       /* a variance below min_var (insertModel throws, OL_GMMStatsEstimator.cpp:287-296) */
#define GMM_ERR_NOMEM 5       /* device allocation refused, or over the handle's memory budget */
#define GMM_ERR_UNSUPPORTED 6 /* configuration outside the implemented range (e.g. D too large) */
#define GMM_ERR_MLLR 7        /* MLLR invertibility conditions fail (OL_ModelAdapt.cpp:1851-1878) */
#define GMM_ERR_TIMEOUT 8     /* a bounded device-side wait expired */

/* precision modes */
#define GMM_PREC_FP32 0 /* plain FP32 replica of the reference CPU arithmetic */
#define GMM_PREC_TC 1   /* tcgen05 tensor-core fused path, split-bf16 operands, FP32 accumulate */

/* accumulation flags (GMMStatsEstimator::setAccFlags, OL_GMMStatsEstimator.h:107-113) */
#define GMM_ACC_MEAN 1
#define GMM_ACC_VAR 2
#define GMM_ACC_PROBS_ONLY 4

/* Create a handle on `device` (GMMStatsEstimator_GPU::GMMStatsEstimator_GPU(int GPU_id),
 * CU_GMMStatsEstimator_CUDA.cu; context creation :977-1016). */
int gmm_create(int device, gmm_handle* out);
int gmm_destroy(gmm_handle h);
/* Message of the last failed call on h (or of the last failed gmm_create when h is NULL). */
const char* gmm_last_error(gmm_handle h);

/* Estimator knobs: GMMStatsEstimator::_minLogLike, _minGamma, _min_var
 * (OL_GMMStatsEstimator.h:59-61; defaults -1e20, 1e-4, 1e-6). */
int gmm_set_options(gmm_handle h, float min_loglike, float min_gamma, float min_var);
int gmm_set_precision(gmm_handle h, int mode);
/* Device-memory budget for this handle in bytes (0 = unlimited); allocations past it fail with
 * GMM_ERR_NOMEM (the reference pre-checks memory in getNSamples2GPU,
 * CU_GMMStatsEstimator_CUDA.cu:1136-1225). */
int gmm_set_memory_budget(gmm_handle h, size_t bytes);
/* The handle's cudaStream_t, for callers that time or order work around it. */
int gmm_get_stream(gmm_handle h, void** stream);

/* Model upload and precompute: insertModel (OL_GMMStatsEstimator.cpp:234-313) +
 * GMMStatsEstimator_GPU::uploadModel (CU_GMMStatsEstimator_CUDA.cu:284-318). */
int gmm_upload_model(gmm_handle h, int M, int D, const float* w, const float* mu, const float* var);

/* Model group (GMMStatsEstimator::insertModel with first = false and setModelToBeUsed,
 * OL_GMMStatsEstimator.cpp:234-325): models kept resident on the device in numbered slots, so a
 * switch between them copies nothing from the host. gmm_upload_model_slot stores a model (host
 * arrays as for gmm_upload_model) in `slot` (0 <= slot < 4096; every model of the group must
 * have the same D, as the reference requires) without changing the model in use;
 * gmm_select_model makes slot n the resident model (a device-to-device copy and the same
 * precompute and variance check as gmm_upload_model; the statistics of the previous model are
 * dropped); gmm_clear_model_slots frees the group (insertModel with first = true). */
int gmm_upload_model_slot(gmm_handle h, int slot, int M, int D, const float* w, const float* mu,
                          const float* var);
int gmm_select_model(gmm_handle h, int slot);
int gmm_clear_model_slots(gmm_handle h);
/* Prior model for MAP (the UBM argument of CModelAdapt::UpdateModelMAP, OL_ModelAdapt.cpp:993). */
int gmm_set_prior(gmm_handle h, const float* w, const float* mu, const float* var);
/* Copy the device-resident model back (w[M], mu[M*D], var[M*D]). */
int gmm_read_model(gmm_handle h, float* w, float* mu, float* var);

/* Feature upload: alignVectors + uploadParam (OL_GMMStatsEstimator_CUDA.cpp:291-328,
 * CU_GMMStatsEstimator_CUDA.cu:431-470). The host variant copies from host memory; the device
 * variant keeps a reference to caller-owned device memory (it must outlive its use). */
int gmm_upload_features(gmm_handle h, const float* X, long long N, int D);
int gmm_upload_features_device(gmm_handle h, const float* dX, long long N, int D);

/* E-step over the resident features: accumulateStatsMT (OL_GMMStatsEstimator.cpp:884-971) /
 * GMMStatsEstimator_CUDA::accumulateStatsMT (OL_GMMStatsEstimator_CUDA.cpp:395-511).
 * Statistics are zeroed first and returned in FP64: n[M], F[M*D], S[M*D] (any of them may be
 * NULL), the total log-likelihood and the number of frames. */
int gmm_accumulate(gmm_handle h, int flags, double* n, double* F, double* S, double* tot_loglike,
                   long long* tot_frames);
/* Same E-step, statistics left on the device for the M-step entry points below. */
int gmm_accumulate_device(gmm_handle h, int flags);
int gmm_read_stats(gmm_handle h, double* n, double* F, double* S, double* tot_loglike,
                   long long* tot_frames);

/* E-step over host features (gmm_upload_features + gmm_accumulate_device in one call): on the
 * tensor-core path the frames go up in chunks on a copy stream while the logits kernels already
 * run on the chunks that landed, so the transfer hides behind compute (X should be page-locked
 * for that); afterwards the features are resident as after gmm_upload_features. Statistics stay
 * on the device (gmm_read_stats, the M-step entry points). */
int gmm_accumulate_host(gmm_handle h, int flags, const float* X, long long N, int D);

/* Per-frame log-likelihoods: compVecsLogLikeMT (OL_GMMStatsEstimator.cpp:811-879) /
 * compLogLikes + getLogLikes (CU_GMMStatsEstimator_CUDA.cu:606-643). out: N floats (host). */
int gmm_loglikes(gmm_handle h, float* out);

/* ------------------------------------------------------------------ full covariances
 * The full-covariance model family (GMModel with Var[D*D], the reference's --full-cov models):
 * insertModel's full branch (OL_GMMStatsEstimator.cpp:298-305, getCovInverse / getLogDet
 * :155-229), computeMixLogLikeFullCov (:593-620), accumulateStats with full second-order
 * statistics (:1334-1378) and the full branches of UpdateModelEM / UpdateModelMAP
 * (OL_ModelAdapt.cpp:905-917, 1074-1083). The full model lives beside the diagonal one on the
 * handle and shares its resident features. cov: [M][D][D] row-major, symmetric; 1 <= D <= 64.
 * A covariance that is not positive definite fails with GMM_ERR_MODEL (the reference throws
 * "cholesky factorization failed"). Second-order statistics are the packed upper triangle per
 * component in row order: Sp[m][k*D + kk - k(k+1)/2] = sum g x_k x_kk for kk >= k
 * (GMMStats' full layout). Arithmetic: FP64 Cholesky factor, |L^-1 (x - mu)|^2 in FP32 with
 * fused multiply-adds, float products of the statistics summed in double-float; the precision
 * mode of the handle does not apply. */
int gmm_upload_model_full(gmm_handle h, int M, int D, const float* w, const float* mu, const float* cov);
int gmm_set_prior_full(gmm_handle h, const float* w, const float* mu, const float* cov);
int gmm_read_model_full(gmm_handle h, float* w, float* mu, float* cov);
int gmm_accumulate_full(gmm_handle h, int flags, double* n, double* F, double* Sp, double* tot_loglike,
                        long long* tot_frames);
int gmm_accumulate_full_device(gmm_handle h, int flags);
int gmm_read_stats_full(gmm_handle h, double* n, double* F, double* Sp, double* tot_loglike,
                        long long* tot_frames);
int gmm_loglikes_full(gmm_handle h, float* out);
/* MLLR of the full model (ComputeW_MLLR reads the covariance diagonals, GetMixtureVarDiag):
 * W from the occupancies and first-order statistics of the last gmm_accumulate_full*, and
 * AdaptModelMLLR on the full model's means. */
int gmm_mllr_estimate_full(gmm_handle h, int ubm_init, double* W);
int gmm_mllr_apply_full(gmm_handle h, const double* W);
/* UpdateModelEM / UpdateModelMAP (tau > 0, against gmm_set_prior_full) on the full model. */
int gmm_em_update_full(gmm_handle h, int up_weight, int up_mean, int up_var, int* alive);
int gmm_map_update_full(gmm_handle h, int tau, int up_weight, int up_mean, int up_var);

/* fMLLR (feature-space MLLR, one regression class) against the resident diagonal model:
 * CModelAdapt::ComputeW_fMLLR (OL_ModelAdapt.cpp:1614-1719) with ComputeKiGi_fMLLR (:1794-1848)
 * and EstimateAb_fmllr (:1721-1792). Runs the E-step over the resident features with full
 * second-order statistics (the plain FP32 log-likelihood kernel whatever the precision mode),
 * then the row passes (`iters`; the reference uses 20) on the device in FP64. W: D x (D+1)
 * row-major [A | b]; features are adapted as x' = A x + b. GMM_ERR_MLLR when CheckInvertibility
 * fails or a row's quadratic has no usable root. D <= 64. */
int gmm_fmllr_estimate(gmm_handle h, int iters, double* W);
/* fMLLR of the full-covariance model: its E-step with full statistics, and the covariance
 * diagonals in G and k (ComputeKiGi_fMLLR reads GetMixtureVarDiag). */
int gmm_fmllr_estimate_full(gmm_handle h, int iters, double* W);
/* Applies W to the features uploaded with gmm_upload_features, in place on the device. */
int gmm_fmllr_apply(gmm_handle h, const double* W);

/* --robust (CModelAdapt::OPTIONS::_robustCov): E-steps also gather the auxiliary statistics of
 * consecutive frames (GMMStatsEstimator::accumulateAuxStats, OL_GMMStatsEstimator.cpp:1253-1286;
 * pairs inside the resident block, the reference's one-thread behaviour), and the EM / MAP
 * updates first apply GetNIndFrames + MakeRobustStats (OL_ModelAdapt.cpp:468-588) to the device
 * statistics (the second-order part is modified in place; UpdateModelEM kills components with
 * fewer than 2 independent frames). Diagonal and full-covariance models. Robust E-steps run on
 * the plain kernels whatever the precision mode (they need every frame's posteriors). */
int gmm_set_robust(gmm_handle h, int on);
/* The auxiliary statistics of the last robust E-step of the diagonal (full = 0) or
 * full-covariance (full = 1) model: aux [M][D] (sum g |x_t - x_t-1|), aux2 [M] (sum sqrt(post)),
 * aux3 [M] (sum g); any pointer may be NULL. */
int gmm_read_aux(gmm_handle h, int full, double* aux, double* aux2, double* aux3);

/* Autotuner of the tensor-core statistics kernel (no counterpart in the reference): on the first
 * E-step of a shape (K, component chunks, frame-tile bucket) it times 1, 2 and 3 waves of CTAs
 * and keeps the fastest for the handle's later E-steps. On by default; off = one wave, the fixed
 * decomposition. The decomposition only groups the partial sums (which frame tiles share an FP32
 * period, which periods share an FP64 partial), so results with different choices differ only in
 * the rounding of those sums. gmm_autotune_choice lists the choices made so far (*n entries; keys
 * and waves up to cap). */
int gmm_set_autotune(gmm_handle h, int on);
int gmm_autotune_choice(gmm_handle h, int* n, long long* keys, int* waves, int cap);

/* Sparse tile schedule of the tensor-core statistics (no counterpart in the reference). A frame
 * keeps posteriors above minGamma for a handful of components, so the E-step of the resident
 * features (D <= 39, at most 32 chunks of 128 active components) can group the components into
 * chunks that lie together in feature space, have the logits kernel record per frame the chunks
 * holding a posterior that can survive the pruning, sort the frames by that record, and run the
 * statistics only on the (128-frame tile, chunk) pairs that have one: 1.85 of 16 chunks per
 * tile in UBM EM at M = 2048, D = 39, where it takes an EM iteration over 10M frames from 29.8
 * to 13.6 ms. The skipped pairs' posteriors are all pruned, so nothing is dropped; but a sorted
 * tile gathers a component's posterior mass, and the tensor core's round-toward-zero
 * accumulation of a tile's sums then loses more low bits: variances within 2.4e-5 relative of
 * FP64 after one UBM EM iteration (1e-5 with the dense schedule; 1.1e-5 for the reference's own
 * FP32 arithmetic). mode 0: off (the default, every pair); 1: on for E-steps of at least 2048
 * frame tiles; 2: on for every E-step. */
int gmm_set_tile_schedule(gmm_handle h, int mode);

/* Test hook (no counterpart in the reference): the number of clock cycles (default 4e9, about
 * 2 s) a tensor-core pipeline role waits on a barrier before it gives up; the kernel then lets
 * its copies and MMAs in flight finish (always with the default limit), frees its tensor memory
 * and the call returns GMM_ERR_TIMEOUT with the handle still usable. A limit of a few hundred
 * cycles makes the waits of any tensor-core E-step expire, so tests can check that path without
 * a fault. cycles <= 0 restores the default. Not meant for production use. */
int gmm_set_wait_limit(gmm_handle h, long long cycles);

/* M-step on the device statistics (FP64 math, float model), in place on the resident model:
 * CModelAdapt::UpdateModelEM (OL_ModelAdapt.cpp:823-949). *alive = components left with
 * non-zero weight. */
int gmm_em_update(gmm_handle h, int up_weight, int up_mean, int up_var, int* alive);
/* CModelAdapt::UpdateModelMAP with tau > 0 (OL_ModelAdapt.cpp:1024-1106) against the prior. */
int gmm_map_update(gmm_handle h, int tau, int up_weight, int up_mean, int up_var);
/* One MAP iteration for S speakers in one call: the per-speaker loop of Model_ADAPT
 * (projects/Model_ADAPT/Model_ADAPT.cpp:170-240) around CModelAdapt::AdaptModel with
 * adaptType MAP and one MAP iteration (OL_ModelAdapt.cpp:1163-1174, AdaptModelMAP :1250-1274,
 * IterMAP :1298-1316, UpdateModelMAP :1024-1106). The resident model is the UBM; the resident
 * features hold every speaker's frames back to back, speaker s owning rows
 * [offs[s], offs[s+1]) (offs: S + 1 non-decreasing entries, offs[S] <= N). With GMM_PREC_TC one
 * fused E-step covers all speakers; with GMM_PREC_FP32 the speakers run one after the other.
 * Outputs (host, any may be NULL): w [S][M], mu [S][M][D], var [S][M][D], ll [S] (each speaker's
 * total log-likelihood under the UBM). tau >= 1. The resident model is not changed. The batched
 * calls (gmm_map_batch[_device], gmm_mllr_batch) keep their device working buffers on the handle
 * between calls, grown to the largest batch seen and released by gmm_destroy; they count against
 * the handle's memory budget. With GMM_PREC_TC over the resident frames, a batch layout (speaker
 * count, padded tiles, work items, buffers) that comes on two calls in a row is captured into a
 * CUDA graph after the second call ran, and later calls with that layout replay it; the speaker
 * offsets and the per-call tables are uploaded every call, so the results equal an eager call's
 * bit for bit. Per-kernel profiling (gmm_profile_enable) runs calls eagerly. */
int gmm_map_batch(gmm_handle h, int S, const long long* offs, int tau, int up_weight, int up_mean,
                  int up_var, float* w, float* mu, float* var, double* ll);
/* Global MLLR mean transforms for S speakers in one call (one regression class, one iteration):
 * the per-speaker loop of Model_ADAPT around CModelAdapt::AdaptModel with adaptType MLLR
 * (OL_ModelAdapt.cpp:1175-1184: IterW_MLLR -> ComputeW_MLLR :1417-1482, ComputeKiGi_MLLR
 * :1525-1581, prepareKiGiInitMatrices :1484-1523 when ubm_init, CheckInvertibility :1851-1878,
 * AdaptModelMLLR :1583-1612). Speakers own resident frame ranges as in gmm_map_batch; the
 * resident model is the UBM. The G and k sums over components run as GEMMs with FP32 products
 * (G on the tensor cores under GMM_PREC_TC, split-bf16 operands) and sums in FP32 per 128
 * components, added in FP64 (GMM_PREC_FP32) or in FP32 with round-to-nearest (GMM_PREC_TC); the
 * single-speaker gmm_mllr_estimate keeps the reference's FP64 sequence. Each row is solved in
 * FP64 by the elimination order of the reference's pivot-free Gauss-Jordan inverse. Outputs (host, any
 * may be NULL): W [S][D][D+1] row-major, status [S] (GMM_OK or GMM_ERR_MLLR when the speaker has
 * too few components or frames; its W is zero and its means stay the UBM's), mu_out [S][M][D]
 * adapted means, ll [S]. */
int gmm_mllr_batch(gmm_handle h, int S, const long long* offs, int ubm_init, double* W, int* status,
                   float* mu_out, double* ll);
/* gmm_map_batch / gmm_mllr_batch over frames in host memory: X [N][D] becomes the handle's
 * features (as gmm_upload_features would make it). On the tensor-core path the frames are copied
 * in chunks of whole speakers on a second stream and each chunk's log-likelihood kernels start
 * as soon as its frames have landed, so the transfer overlaps the E-step (page-locked X lets the
 * copies run asynchronously); otherwise the frames are uploaded first. Results are those of
 * gmm_upload_features + gmm_map_batch / gmm_mllr_batch. */
int gmm_map_batch_host(gmm_handle h, const float* X, long long N, int D, int S, const long long* offs, int tau,
                       int up_weight, int up_mean, int up_var, float* w, float* mu, float* var, double* ll);
int gmm_mllr_batch_host(gmm_handle h, const float* X, long long N, int D, int S, const long long* offs,
                        int ubm_init, double* W, int* status, float* mu_out, double* ll);
/* The same with device outputs (d_w, d_mu, d_var, d_ll on the handle's device; any may be NULL). */
int gmm_map_batch_device(gmm_handle h, int S, const long long* offs, int tau, int up_weight,
                         int up_mean, int up_var, float* d_w, float* d_mu, float* d_var,
                         double* d_ll);
/* `iters` EM iterations entirely on the device (CModelAdapt::IterEM with tau = 0,
 * OL_ModelAdapt.cpp:1276-1296): each iteration moves zero-weight components behind the others
 * as insertModel does, accumulates and updates. ll[i] = total log-likelihood of iteration i.
 * The resident model is left in the reference's final component order. */
int gmm_em_iterate(gmm_handle h, int iters, int up_weight, int up_mean, int up_var, double* ll,
                   int* alive);

/* Global MLLR mean transform from the device statistics (mean statistics required):
 * CModelAdapt::ComputeW_MLLR + ComputeKiGi_MLLR + MATRIX::Invert (OL_ModelAdapt.cpp:1417-1581,
 * Matrix4_LMa.cpp:2232-2300), with the UBM-based initialisation of prepareKiGiInitMatrices
 * (:1484-1523) from the prior when ubm_init != 0. W: D x (D+1) row-major FP64 (host). */
int gmm_mllr_estimate(gmm_handle h, int ubm_init, double* W);
/* CModelAdapt::AdaptModelMLLR (OL_ModelAdapt.cpp:1583-1612): resident means <- A mu + b. */
int gmm_mllr_apply(gmm_handle h, const double* W);

/* Allocation-free E-step. No counterpart in the reference: it exists for callers that cannot let
 * this library allocate device memory -- an application whose framework owns the whole device
 * memory pool, or a latency-critical loop in which a cudaMalloc/cudaFree (and the device
 * synchronisation a cudaFree implies) is not allowed once it runs. It computes what
 * gmm_accumulate computes with the plain FP32 path, from caller-owned device arrays
 * (dX [N][D], dw [M], dmu [M][D], dvar [M][D]) into the caller-owned device array
 * d_stats = n[M] | F[M*D] | S[M*D] | total log-likelihood (FP64, zeroed first), on `stream`
 * (a cudaStream_t; NULL = legacy default stream). The call is synchronous: it synchronises
 * `stream` before it returns, so the statistics are ready on return.
 * Working memory is one fixed 32 MiB array compiled into the library; every GPU that loads the
 * library keeps it until the process exits. Limits: M <= 4096, D <= 128, and one slice of
 * statistics (8 * M_active * (1 + 2D) bytes) plus 256 frames of posteriors must fit beside the
 * model tables (GMM_ERR_UNSUPPORTED beyond; every M <= 4096, D <= 128 fits). Each call looks up
 * the array's address in the current context (no allocation, so a cudaDeviceReset between calls
 * is harmless); the first call on a device may load the library's device code, so make that
 * first call before any stream capture. All calls share the array, so calls that overlap on the
 * GPU (different streams or threads at the same time) race; serialise them. Errors are reported
 * through gmm_last_error(NULL). */
int gmm_accumulate_noalloc(const float* dX, long long N, int D, int M, const float* dw,
                           const float* dmu, const float* dvar, float min_loglike, float min_gamma,
                           float min_var, int flags, double* d_stats, void* stream);

/* Per-kernel device time accounting (CUDA events on the handle's stream; the reference's
 * GPU_CUDA_TIMER, CU_GMMStatsEstimator_CUDA.cu:50-55). gmm_profile_read fills up to `cap`
 * entries of names/milliseconds/launch counts and returns the number of kernels seen. */
int gmm_profile_enable(gmm_handle h, int on);
int gmm_profile_reset(gmm_handle h);
int gmm_profile_read(gmm_handle h, int cap, const char** names, double* ms, long long* launches);
/* Number of kernel launches this handle issued since creation (all kernels); 0 for a null handle. */
long long gmm_launch_count(gmm_handle h);

/* ------------------------------------------------------------------ feature files
 * The reference's parameter-file formats (Param::Load / LoadHTK / LoadRaw, param/OL_Param.cpp:224-580):
 * GMM_PRM_SVES "SV-ES-PARAM" files, GMM_PRM_HTK big-endian HTK files, GMM_PRM_RAW
 * (int32 frames, int32 dim, floats). dwnsmp > 1 keeps every dwnsmp-th frame. */
#define GMM_PRM_SVES 0
#define GMM_PRM_HTK 1
#define GMM_PRM_RAW 2
/* Reads one file: with out = NULL only *N (frames after down-sampling) and *D are returned;
 * otherwise up to cap_frames frames [N][D] go to out. GMM_ERR_ARG for a missing or bad file. */
int gmm_read_param(const char* path, int prm_type, unsigned int dwnsmp, float* out, long long cap_frames,
                   long long* N, int* D);
/* File-by-file accumulation: accumulateStatsMT(CFileList&, ...) (OL_GMMStatsEstimator.cpp:641-698).
 * Files are read on a loader thread into page-locked buffers and appended until the buffered
 * frames reach buffer_gb GiB (the reference's _memoryBuffDataGB), then each batch is copied to the
 * device and accumulated while the loader reads the next one. Statistics are zeroed first and
 * summed over all batches on the device (read them with gmm_read_stats; the M-step entry points
 * use them). Missing or empty files are skipped, as the reference does; *files_used counts the
 * files that contributed frames. The batches are transient: afterwards no features are resident. */
int gmm_accumulate_files(gmm_handle h, int flags, int n_files, const char* const* paths, int prm_type,
                         unsigned int dwnsmp, double buffer_gb, int* files_used);

/* ------------------------------------------------------------------ request server
 * Continuous-batching server for scoring and MAP-adaptation requests against resident GMMs. It
 * replaces the reference's one-request-at-a-time tools: getLogLike's per-file scoring
 * (projects/GetLogLikeGMM/main.cpp:119-180 -> compVecsLogLikeMT, OL_GMMStatsEstimator.cpp:811-879)
 * and Model_ADAPT's per-speaker MAP loop (projects/Model_ADAPT/Model_ADAPT.cpp:170-240 ->
 * CModelAdapt::AdaptModel / AdaptModelMAP, OL_ModelAdapt.cpp:1163-1274). All models of a server
 * have the same M and D (1 <= D <= 63, tensor-core path). A worker thread admits queued requests
 * in arrival order while their device footprint fits one of two request arenas of
 * request_bytes / 2 each, runs each batch as one fused E-step, and overlaps the next batch's
 * preparation and upload with the running one. A request's result does not depend on what else
 * is in its batch (bit-identical). */
typedef struct gmm_server_s* gmm_server;
#define GMM_REQ_SCORE 0  /* total (and optionally per-frame) log-likelihood under the model */
#define GMM_REQ_MAP 1    /* one MAP iteration against the model (the model is the UBM) */
#define GMM_REQ_QUEUED 0
#define GMM_REQ_RUNNING 1
#define GMM_REQ_DONE 2
#define GMM_REQ_FAILED 3
int gmm_server_create(int device, int D, int M, int max_models, size_t request_bytes, gmm_server* out);
int gmm_server_destroy(gmm_server s);
const char* gmm_server_last_error(gmm_server s); /* NULL server: the last create error */
/* minLogLike, minGamma, min_var as in gmm_set_options; max_batch = most requests per batch. */
int gmm_server_set_options(gmm_server s, float min_loglike, float min_gamma, float min_var, int max_batch);
/* Makes a model resident (w [M], mu [M][D], var [M][D]); *model_id receives its id. */
int gmm_server_add_model(gmm_server s, const float* w, const float* mu, const float* var, int* model_id);
/* Queues a request on frames [N][D] (host). By default the frames are copied at submit, so the
 * caller may reuse them; with GMM_SUBMIT_NO_COPY they must stay valid until gmm_server_result
 * (page-locked memory is then copied to the device directly). GMM_SUBMIT_FRAME_LL keeps the
 * per-frame log-likelihoods. For GMM_REQ_MAP, tau >= 1 and up_* select the adapted parameters
 * (as gmm_map_batch). */
#define GMM_SUBMIT_FRAME_LL 1
#define GMM_SUBMIT_NO_COPY 2
int gmm_server_submit(gmm_server s, int kind, int model_id, const float* frames, long long N, int tau,
                      int up_weight, int up_mean, int up_var, int options, long long* ticket);
int gmm_server_poll(gmm_server s, long long ticket, int* state); /* GMM_REQ_* state */
/* Blocks until the request finished (timeout_ms < 0: no limit; GMM_ERR_TIMEOUT on expiry). */
int gmm_server_wait(gmm_server s, long long ticket, int timeout_ms);
/* Copies a finished request's results (any pointer may be NULL: total_ll; frame_ll [N];
 * w [M], mu [M][D], var [M][D] for MAP; latency from submit to completion in ms) and releases
 * the ticket. Returns the request's own status. */
int gmm_server_result(gmm_server s, long long ticket, double* total_ll, float* frame_ll, float* w, float* mu,
                      float* var, double* latency_ms);
int gmm_server_stats(gmm_server s, long long* batches, long long* completed, long long* failed,
                     size_t* peak_batch_bytes);

#ifdef __cplusplus
}
#endif
#endif
