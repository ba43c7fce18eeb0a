// Internal declarations shared by the gmm_gb300 translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <map>
#include <vector>

#include "gmm_gb300.h"

namespace gmm {

constexpr double kMinusLog2Pi = -1.837877066409345;  // OL_GMMStatsEstimator.h:280
constexpr int kMaxMix = 32767;                        // GMModel::NumMixes is __int16
constexpr int kMaxDim = 1024;
constexpr int kMaxModelSlots = 4096;  // models in one handle's group
// How long (clock cycles, ~2 s) a tensor-core pipeline role may wait on an mbarrier before it
// gives up, raises the CTA's abort flag and the kernel reports GMM_ERR_TIMEOUT.
constexpr long long kDefaultWaitLimit = 4000000000LL;

// ------------------------------------------------------------------ error plumbing
struct Error {
  int code;
  std::string msg;
};

// ------------------------------------------------------------------ per-kernel timing
struct KernelTimer {
  std::string name;
  double ms = 0.0;
  long long launches = 0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
};

struct FullModel;  // full-covariance model and statistics (full_kernels.cu)

// ------------------------------------------------------------------ tensor-core model planes
struct TcModel {
  int K = 0;            // padded contraction length (multiple of 16) of [x, x^2, 1, ...]
  int Mpad = 0;         // active components padded to the component tile
  uint16_t* planes = nullptr;  // 3 bf16 planes of W~ in the UMMA K-major tile layout
  int* comp_of_row = nullptr;  // row r of the padded active list -> caller component index
  float* ll2 = nullptr;        // per-frame log2-domain LSE of the current E-step
  // [Mpad][D] centres of the statistics kernel's sums (the row's mean; 0 for padding rows)
  float* cent = nullptr;
  int D = 0;
};

struct TcFeatures {
  int K = 0;
  long long Npad = 0;
  uint16_t* planes = nullptr;  // 3 bf16 planes of Z = [x, x^2, 1, ...] per frame tile
};

// Sparse tile schedule of the tensor-core statistics kernel (tc_schedule.cu): device buffers.
constexpr int kSchedGridMax = 1024;  // work items (CTAs of the statistics launch) at most
constexpr int kSchedChunksMax = 32;  // component chunks the frame masks cover
constexpr long long kSchedMinTiles = 2048;  // mode 1: E-steps of at least this many frame tiles
// A chunk is active for a frame when one of its logits lies within log2(minGamma) - margin of
// the frame's log2-LSE; the margin (log2 units) covers the rounding difference between the
// logits kernel's and the statistics kernel's logits of the same pair (~1e-5).
constexpr double kSchedMargin2 = 0.25;
struct TileSched {
  int mode = 0;                   // gmm_set_tile_schedule: 0 off, 1 large E-steps, 2 always
  long long Npad = 0;             // frame rows the frame buffers hold
  int K = 0;
  int chunks = 0;                 // component chunks the lists cover
  long long lists_nT = 0;         // tiles per chunk list
  uint32_t* fmask = nullptr;      // [Npad] chunks with a kept posterior, per frame row
  uint32_t* kbuf = nullptr;       // [2][Npad] sort keys (ping-pong)
  int* vbuf = nullptr;            // [2][Npad] sort values
  int* perm = nullptr;            // sorted row -> original row (inside vbuf)
  long long* srow = nullptr;      // [Npad] sorted row -> frame (-1: padding)
  int* hist = nullptr;            // [256][sort blocks], then [256] digit offsets
  uint16_t* planes = nullptr;     // 3 bf16 planes of the sorted frames (tile images)
  float* ll2 = nullptr;           // [Npad] log2-LSE of the sorted frames
  uint32_t* tmask = nullptr;      // [Npad / 128] union of the masks of a sorted tile
  int* lists = nullptr;           // [chunks][tiles] active tiles of each chunk
  int* counts = nullptr;          // [chunks] list lengths
  int4* work = nullptr;           // [kSchedGridMax] {W chunk, 0, list offset, tiles}
  int* item_off = nullptr;        // [chunks + 1] first work item of each chunk, then the count
  int* gact = nullptr;            // [M] active list grouped into spatially coherent chunks
  int gact_cap = 0;
  CUtensorMap zmap;               // over `planes`
};

// One device-resident model of a handle's model group (caller order, as uploaded).
struct ModelSlot {
  int M = 0, D = 0;
  float *w = nullptr, *mu = nullptr, *var = nullptr;
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;

  float minLL = -1e20f, minGamma = 1e-4f, min_var = 1e-6f;
  int precision = GMM_PREC_FP32;
  size_t budget = 0, allocated = 0;

  // model (caller order), device
  int M = 0, D = 0, Mact = 0;
  float *w = nullptr, *mu = nullptr, *var = nullptr;
  float *icov = nullptr, *logG = nullptr, *logW = nullptr;
  int* act = nullptr;      // active component indices in order (w > 0)
  int* flag = nullptr;     // device flags: [0] bad variance, [1] stability trouble, [2] alive,
                           // [3] timeout, [4] active count
  int* hflag = nullptr;    // pinned mirror of flag
  float *pw = nullptr, *pmu = nullptr, *pvar = nullptr;  // MAP prior
  bool have_prior = false;
  bool model_dirty = true;  // precompute needed
  std::vector<ModelSlot> slots;  // model group: gmm_upload_model_slot / gmm_select_model
  TileSched sched;               // sparse tile schedule of the tensor-core statistics
  bool sched_active = false;     // the current model planes are grouped for the schedule

  // features
  long long N = 0;
  int Dx = 0;  // feature dimension (checked against the model's at each E-step)
  const float* X = nullptr;
  float* Xown = nullptr;

  // statistics (FP64, caller order): n[M], F[M*D], S[M*D], then totLL, and frames as double
  double* stats = nullptr;
  double* llpart = nullptr;  // per-block log-likelihood partial sums
  size_t llpart_cap = 0;
  long long tot_frames = 0;
  int acc_flags = 0;
  bool stats_valid = false;

  // scratch
  float* logits = nullptr;  // plain path: [Mact][chunk] raw log posteriors
  size_t logits_cap = 0;
  float* ll = nullptr;      // per-frame log-likelihood, N floats
  size_t ll_cap = 0;
  double* part = nullptr;   // plain path: per (slice, component) partial statistics
  size_t part_cap = 0;
  double* hstage = nullptr; size_t hstage_cap = 0;  // pinned staging for results

  // model backup for the all-components-killed fallback of IterEM
  float *bw = nullptr, *bmu = nullptr, *bvar = nullptr;

  // tensor-core path
  TcModel tcm;
  TcFeatures tcx;
  bool tcx_valid = false;
  double* tcpart = nullptr;  // per-CTA FP64 partial statistics
  size_t tcpart_cap = 0;
  CUtensorMap tm_zfull, tm_wfull;  // TMA maps over the operand images (box = one 128-row tile)
  int* tc_err = nullptr;                          // bounded-wait expiry flag
  long long wait_limit = kDefaultWaitLimit;       // clock cycles a pipeline wait may take
  double* tc_llpart = nullptr;                    // per-thread log-likelihood partials
  size_t tc_llpart_cap = 0;
  int sms = 0;
  // EM iterations replayed from a CUDA graph: shapes fixed at all M components (padded rows for
  // the dead ones), the active count read on the device, no host readbacks inside an iteration
  bool static_shapes = false;
  // autotuner: statistics-kernel decomposition (CTA waves) measured once per shape
  bool autotune = true;
  std::map<long long, int> tuned_waves;  // key: K, component chunks, frame tiles (bucket)
  cudaGraphExec_t em_graph = nullptr;
  long long em_graph_key[31] = {};
  // batched MAP over the resident frames replayed from a CUDA graph while the batch layout (and
  // every buffer the kernels read or write) stays the same: the kernels of one call, captured
  cudaGraphExec_t map_graph = nullptr;
  long long map_graph_key[48] = {};
  long long map_last_key[48] = {};  // the previous call's key: a layout is captured when it repeats
  int map_graph_launches = 0;  // kernel launches inside the graph (the launch count adds them)
  double* ll_hist = nullptr;  // [ll_hist_cap + 1]: per-iteration total LL, then a counter
  int ll_hist_cap = 0;

  // full-covariance model (own parameters and statistics; shares the features and scratch)
  FullModel* full = nullptr;

  // host-to-device copies that overlap the E-step (gmm_accumulate_host)
  cudaStream_t copy_stream = nullptr;
  std::vector<cudaEvent_t> copy_events;

  // --robust: auxiliary statistics of the diagonal model [aux (M x D) | aux2 (M) | aux3 (M)],
  // per-frame gs of a chunk, the previous chunk's last posteriors, independent-frame counts
  bool robust = false;
  double* aux = nullptr;
  size_t aux_cap = 0;
  bool aux_valid = false;
  float* gs = nullptr;
  size_t gs_cap = 0;
  float* gprev = nullptr;
  size_t gprev_cap = 0;
  double* nind = nullptr;
  size_t nind_cap = 0;

  // grow-only device scratch of the batched speaker calls (gmm_map_batch, gmm_mllr_batch):
  // kept between calls so that a call allocates nothing once the largest batch has been seen;
  // released by gmm_destroy
  struct Scratch {
    void* p = nullptr;
    size_t cap = 0;
  };
  Scratch scratch[32];

  // timing
  bool profile = false;
  std::vector<KernelTimer> timers;
  long long launches = 0;
};

// device allocation through the handle's budget
int dalloc(Ctx* c, void** p, size_t bytes, const char* what);
void dfree(Ctx* c, void* p, size_t bytes);
int fail(Ctx* c, int code, const std::string& msg);
int cuda_fail(Ctx* c, cudaError_t e, const char* what);

// kernel timing around a launch
struct LaunchScope {
  Ctx* c;
  KernelTimer* t = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  LaunchScope(Ctx* c, const char* name);
  ~LaunchScope();
};
#define GMM_LAUNCH(ctx, name) ::gmm::LaunchScope _ls_##__LINE__((ctx), (name))

// ------------------------------------------------------------------ plain FP32 path
int plain_precompute(Ctx* c);
int plain_precompute_async(Ctx* c);  // the same launches without the host readback
int plain_estep(Ctx* c, int flags, bool want_stats, float* ll_out_dev);
int plain_ll_chunk(Ctx* c, long long f0, long long nf, float* G, long long ldg, float* llout);
// E-step of the resident diagonal model with packed full second-order statistics (fMLLR):
// stats [n (M) | F (M x D) | S (M x D(D+1)/2) | totLL | pad] on the device, zeroed by the callee.
int diag_fullstats_estep(Ctx* c, double* stats);

// ------------------------------------------------------------------ M-step
int mstep_em(Ctx* c, int upW, int upM, int upV, int* alive);
int mstep_map(Ctx* c, int tau, int upW, int upM, int upV);
// device-side steps of a captured EM iteration
int mstep_em_restore(Ctx* c);           // restore the backup model if no component survived
int record_iteration_ll(Ctx* c);        // append the statistics' total LL to c->ll_hist
int mstep_rearrange(Ctx* c);
int mstep_mllr(Ctx* c, int ubm_init, double* W_host);
int mstep_mllr_apply(Ctx* c, const double* W_host);

// ------------------------------------------------------------------ tensor-core path
int tc_supported(int D);
int tc_prepare_features(Ctx* c);
int tc_prepare_model(Ctx* c, bool sched_ok);
int tc_estep(Ctx* c, int flags, bool want_stats, float* ll_out_dev);
int tc_estep_streamed(Ctx* c, const float* Xh, int flags, int nchunks);

// One MAP iteration for S speakers against the resident model (the UBM); speaker s owns the
// resident frames [offs[s], offs[s+1]).
struct MapBatch {
  int S = 0, tau = 0, upW = 0, upM = 0, upV = 0, flags = 0;
  const long long* offs = nullptr;    // host, S + 1 entries
  const long long* d_offs = nullptr;  // the same on the device
  float* w = nullptr;                 // device outputs: [S][M] weights, [S][M][D] means, variances
  float* mu = nullptr;
  float* var = nullptr;
  float* aw = nullptr;                // device scratch [S][M]
  double* ll = nullptr;               // device output [S]: per-speaker total log-likelihood
  const float* Xh = nullptr;          // frames in host memory (null: the resident features)
};
// Columns of the tensor-core operand layout (features Z, model W, statistics partials) of width
// K = 2D + 1 rounded up to 16 (so K >= 2D + 2): x_d at d, the constant at D, x_d^2 at K/2 + d,
// zeros elsewhere. The first-order statistics and the count lead, so an E-step without
// second-order statistics multiplies only the first tc_mean_cols(D) columns; the squares start at
// a column fixed by K, so code specialised on K addresses them with constant offsets.
__host__ __device__ inline int tc_col_one(int D) { return D; }
__host__ __device__ inline int tc_col_sq(int K, int d) { return K / 2 + d; }
__host__ __device__ inline int tc_mean_cols(int D) { return (D + 1 + 15) / 16 * 16; }
// Physical column of statistic e in the order n / F / S used by the plain layout's readers
// (e < D: F_e, D <= e < 2D: S_(e-D), e = 2D: n).
__host__ __device__ inline int tc_stat_col(int D, int K, int e) { return e < D ? e : e == 2 * D ? D : K / 2 + (e - D); }
// The tensor-core statistics kernel accumulates around a centre c per component row (the
// component's mean at the E-step): F' = sum g (x - c), S' = sum g (x - c)^2. Readers of its
// partials sum the pieces and add the centre back in FP64.
__host__ __device__ inline double tc_uncentre_F(double Fc, double n, double c) { return Fc + c * n; }
__host__ __device__ inline double tc_uncentre_S(double Sc, double Fc, double n, double c) {
  return Sc + c * (2.0 * Fc + c * n);
}

// x / d correctly rounded, given r = RN(1 / d) (__drcp_rn): q = RN(x r), the remainder x - d q
// exactly by FMA, then RN(q + remainder r) is RN(x / d) for normal operands (Markstein's theorem).
// Two FMAs and a product instead of a division, where many quotients share one divisor: GB300
// runs FP64 at 1/64 of its FP32 rate and a division is an order of magnitude more FP64 work.
__device__ __forceinline__ double div_by_rcp(double x, double d, double r) {
  const double q = __dmul_rn(x, r);
  const double e = __fma_rn(-d, q, x);
  return __fma_rn(e, r, q);
}

// Slots of Ctx::scratch
enum ScratchSlot {
  SC_OFFS, SC_AW, SC_W, SC_MU, SC_VAR, SC_LL, SC_ROWMAP, SC_TILESLOT, SC_WORK, SC_PAD, SC_PART,
  SC_PIECE0, SC_NPIECES, SC_ROWCOMP, SC_MLLR_W, SC_MLLR_ST, SC_MLLR_N, SC_MLLR_F, SC_MLLR_G,
  SC_MLLR_K, SC_MLLR_B, SC_MLLR_XI, SC_MLLR_GP, SC_MLLR_KP, SC_MLLR_AIMG, SC_MLLR_BIMG, SC_MLLR_RVAR,
  SC_COUNT
};
static_assert(SC_COUNT <= 32, "Ctx::scratch slots");
// Tensor-core G data term of batched MLLR: d_G [S][D][T] (FP64) from the dense counts d_n [S][M].
int tc_mllr_g(Ctx* c, int S, const double* d_n, double* d_G);
// Pointer to at least `bytes` of the slot's buffer (grown, contents not kept, when smaller).
int scratch(Ctx* c, int slot, size_t bytes, const char* what, void** out);

// Per-speaker statistics from the tensor-core path: FP64 partials of pieces of at most 8192
// frames, [piece][chunk][K cols][128 rows] (operand-layout columns, tc_stat_col; rows = padded
// active list; first- and second-order sums centred on cent, see tc_uncentre); speaker s owns pieces [piece0[s], piece0[s] + npieces[s]), summed in piece order.
struct SpeakerStats {
  int S = 0, n_chunks = 0, K = 0, pieces = 0;
  double* part = nullptr;
  int* piece0 = nullptr;       // [S]
  int* npieces = nullptr;      // [S]
  int* row_of_comp = nullptr;  // [M], -1 for inactive components
  const float* cent = nullptr; // [rows][D] centres of the partials (tc_uncentre)
  size_t part_bytes = 0;
};
// Xh: the frames in host memory (copied into the handle's feature buffer chunk by chunk, the
// copies overlapping the logits kernels), or null for the resident features.
int tc_speaker_stats(Ctx* c, int S, const long long* offs, const long long* d_offs, double* d_ll,
                     bool second_order, const float* Xh, SpeakerStats* ss);
int ensure_copy_stream(Ctx* c, int n_events);
void tc_free_speaker_stats(Ctx* c, SpeakerStats* ss);
// Per-speaker statistics from the plain path: [speaker][n (M) | F (M x D) | S (M x D) | totLL | pad]
// MAP update for all speakers from either form (exactly one of plain / ss is non-null).
int mstep_map_batch(Ctx* c, const MapBatch& b, const double* plain, const SpeakerStats* ss);
int tc_map_batch(Ctx* c, const MapBatch& b);
int plain_map_batch(Ctx* c, const MapBatch& b);
// Plain FP32 per-speaker statistics in the plain layout (one E-step per speaker); *out is a
// device array the caller frees with dfree(c, *out, *bytes).
int plain_speaker_stats(Ctx* c, int S, const long long* offs, int flags, double** out, size_t* bytes);
int mstep_mllr_batch(Ctx* c, int S, const double* plain, const SpeakerStats* ss, int ubm_init, double* dW,
                     int* dstatus, float* dmu_out, double* dll);

// Feature files (SVES / HTK / RAW): header (frames after down-sampling, dimension) and frames.
// Both return -1 for a file that cannot be opened, GMM_ERR_ARG with *err for a bad file.
int param_header(const char* path, int type, unsigned dwnsmp, long long* N, int* D, std::string* err);
int param_read(const char* path, int type, unsigned dwnsmp, float* out, std::string* err);

// One tensor-core E-step over a batch of requests that may use different resident models (all
// with the same D and chunk count): feature planes for the batch's padded row layout, the
// logits / log-sum-exp kernel over every row (W chunks from the tile's model), and the
// statistics kernel over explicit work items. Device pointers; launched on c->stream.
struct TcBatch {
  int D = 0, K = 0;
  int n_chunks = 0;                   // W chunks per model
  int w_chunks_total = 0;             // W chunks in the shared planes
  const uint16_t* wplanes = nullptr;  // shared W planes (tile images)
  const float* cent = nullptr;        // [W plane rows][D] centres of the statistics sums
  const CUtensorMap* wmap = nullptr;  // 2-D map over wplanes, box = K rows
  const float* X = nullptr;           // batch frames [N][D]
  long long N = 0, Rpad = 0;          // frames, padded rows (multiple of 128)
  const long long* row_frame = nullptr;  // [Rpad]
  const int* tile_wbase = nullptr;       // [Rpad / 128] first W chunk of the row tile's model
  uint16_t* zplanes = nullptr;        // [3][Rpad][K]
  float* ll2 = nullptr;               // [Rpad]
  float* ll = nullptr;                // [N] per-frame log-likelihood
  double* llpart = nullptr;           // [>= sms * 128]
  int n_work = 0;                     // statistics CTAs (0: log-likelihoods only)
  const int4* work = nullptr;         // {W chunk, chunk in model, first FT tile, FT tiles}
  const int* tile_slot = nullptr;     // [Rpad / FT] statistics slot of each FT tile
  double* part = nullptr;             // [slots][n_chunks][K][128], centred (tc_uncentre)
  size_t part_bytes = 0;              // zeroed before the statistics kernel adds into it
  int single_comp = 0;
  bool second_order = true;           // S statistics wanted (else only the [x | 1] columns)
};
int tc_stats_ft(int K);  // frames per statistics tile for K
int tc_flush_tiles(int K);  // statistics tiles per speaker piece (one FP64 slot)
// The statistics kernel's partials are centred (tc_uncentre) for second-order statistics with
// K > 80 (the sparse kernel); otherwise they are plain sums.
bool tc_stats_centred(int K, bool second_order);
// sparse tile schedule (tc_schedule.cu)
bool sched_supported(int chunks, int Mact);
int sched_prepare(Ctx* c, long long Npad, int K, int chunks);
void sched_free(Ctx* c);
void sched_group(Ctx* c, const int* act, int Mact, const int* mact_dev, int chunks, int D, const float* mu);
void sched_sort(Ctx* c, long long Npad, int chunks);
void sched_lists(Ctx* c, long long Npad, int chunks, int grid);
void sched_reduce(Ctx* c, int K, int Mrows, int chunks, const int* comp_of_row, const float* cent,
                  const double* part, int flags);
int tc_k(int D);
int tc_run_batch(Ctx* c, const TcBatch& b);
int tc_run_batch_part(Ctx* c, const TcBatch& b, int tile0, int ntl, int stages);
int tc_make_wmap(Ctx* c, CUtensorMap* map, const uint16_t* planes, long long rows, int K);
int tc_build_model(Ctx* c, int D, int K, int Mact, int Mpad, long long plane_rows, long long row0,
                   const int* act, const float* w, const float* mu, const float* var,
                   uint16_t* planes, int* comp_of_row, float* cent);

int sync(Ctx* c, const char* what);

// Full-covariance model state (allocated on the first gmm_upload_model_full).
void full_destroy(Ctx* c);

// --robust: auxiliary statistics of frames [f0, f0 + nf) from the chunk's log joints (c->logits,
// ldg) and LLs into aux (caller order, M components); GetNIndFrames + MakeRobustStats on the
// device statistics (second-order part modified in place), *nind -> the device counts.
int robust_chunk(Ctx* c, int M, int D, int Mact, const int* act, long long f0, long long nf, long long ldg,
                 double* aux);
int robust_make(Ctx* c, int M, int D, int full, double* stats, const double* aux, double** nind);
int ensure_aux(Ctx* c, double** aux, size_t* cap, int M, int D);
bool full_aux(Ctx* c, const double** aux, int* M, int* D);  // the full model's valid auxiliary statistics
// fMLLR of the full model: its device statistics, means, and a new device array of covariance
// diagonals (the caller frees it with dfree(c, *diag, M * D * sizeof(float))).
int full_fmllr_inputs(Ctx* c, const double** stats, const float** mu, float** diag, int* M, int* D,
                      long long* frames);

}  // namespace gmm

// The opaque handle type of the C ABI is the context itself.
struct gmm_ctx : public gmm::Ctx {};
