// Request server: resident GMMs, scoring and MAP-adaptation requests, continuous batching.
//
// The reference serves one utterance or one speaker at a time: getLogLike scores a file list
// against a model (projects/GetLogLikeGMM/main.cpp:119-180, compVecsLogLikeMT) and Model_ADAPT
// adapts one speaker after another (projects/Model_ADAPT/Model_ADAPT.cpp:170-240,
// CModelAdapt::AdaptModel -> AdaptModelMAP, OL_ModelAdapt.cpp:1163-1274). The server runs the same
// per-request arithmetic -- per-frame log-likelihoods, or one MAP iteration against the request's
// model -- for many requests at once:
//
// * Models stay resident: their tensor-core operand planes share one array (each model on its
//   own 128-row tiles), parameters in [model][M][D] arrays.
// * A worker thread forms batches from the queue in arrival order, admitting requests while their
//   device footprint fits one of two request arenas; a request that arrives while a batch runs
//   joins the next batch, whose host preparation and host-to-device copy (on a second stream)
//   overlap the running batch.
// * Each batch is one tensor-core E-step over all its rows: every request starts on a 128-row
//   tile; the logits kernel takes the W chunks of the tile's model; MAP requests are cut into
//   pieces of one FP64 flush period (8192 frames), each piece owning a statistics slot, so a
//   request's FP64 sums are the same whatever else is in the batch: results are bit-identical
//   alone and in a mix.
// * Latency is measured from submit to the moment the worker sees the batch finished.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gmm_internal.cuh"

namespace gmm {
namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// arena bytes kept back from admission for the batch's own small arrays (work items, offsets)
constexpr size_t kArenaSlack = (size_t)4 << 20;

struct Req {
  long long ticket = 0;
  int kind = 0;  // GMM_REQ_SCORE / GMM_REQ_MAP
  int model = 0;
  long long N = 0;
  std::vector<float> frames;     // own copy (default)
  const float* src = nullptr;    // caller's frames (GMM_SUBMIT_NO_COPY)
  int tau = 16, upW = 0, upM = 1, upV = 0, want_frame_ll = 0;
  int state = GMM_REQ_QUEUED;
  int status = GMM_OK;
  std::string err;
  double ll = 0.0;
  std::vector<float> frame_ll, w, mu, var;
  double t_submit = 0.0, t_admit = 0.0, t_done = 0.0;
  size_t foot = 0, hin_foot = 0, hout_foot = 0;  // device, pinned input, pinned output bytes
  // batch layout
  long long row0 = 0, rows = 0, x0 = 0;
  int piece0 = 0, pieces = 0;
};

// MAP update over the statistics pieces of each MAP request (the expression order of
// map_comp_kernel for weights and means; the variance in FP64 throughout, as the tensor-core
// path's M-steps compute it). One warp per (request, component).
__global__ void srv_map_kernel(int R, int M, int D, int K, int n_chunks, const int* __restrict__ req_model,
                               const int* __restrict__ req_piece0, const int* __restrict__ req_pieces,
                               const long long* __restrict__ req_frames, const int* __restrict__ req_par,
                               const int* __restrict__ row_of_comp, const float* __restrict__ cent,
                               const double* __restrict__ part,
                               const float* __restrict__ mw, const float* __restrict__ mmu,
                               const float* __restrict__ mvar, float min_var, float* __restrict__ ow,
                               float* __restrict__ omu, float* __restrict__ ovar,
                               float* __restrict__ adapted_w) {
  const long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= (long long)R * M) return;
  const int r = (int)(t / M), m = (int)(t - (long long)r * M);
  const int mod = req_model[r];
  const int tau = req_par[4 * r], upW = req_par[4 * r + 1], upM = req_par[4 * r + 2], upV = req_par[4 * r + 3];
  const float uwm = mw[(size_t)mod * M + m];
  const float* um = mmu + ((size_t)mod * M + m) * D;
  const float* uv = mvar + ((size_t)mod * M + m) * D;
  const int row = row_of_comp[(size_t)mod * M + m];
  const size_t cs = 128;
  // FP64 sums over the request's pieces, in piece order
  auto col = [&](int e) -> double {
    double v = 0.0;
    for (int p = 0; p < req_pieces[r]; ++p) {
      const double* st = part + ((size_t)(req_piece0[r] + p) * n_chunks + row / 128) * K * 128 + (row % 128);
      v = p == 0 ? st[(size_t)e * cs] : __dadd_rn(v, st[(size_t)e * cs]);
    }
    return v;
  };
  const double mp = row >= 0 ? col(tc_col_one(D)) : 0.0;
  const bool adapt = uwm != 0.0f && mp > 0.0;
  const unsigned int tot = (unsigned int)req_frames[r];
  const double alfa = adapt ? __ddiv_rn(mp, __dadd_rn(mp, (double)tau)) : 0.0;
  const double one_m = __dsub_rn(1.0, alfa);
  if (lane == 0) {
    float aw = 0.0f;
    const bool wset = adapt && upW && tot > 0;
    if (wset) {
      const double t1 = __dmul_rn(alfa, __ddiv_rn(mp, (double)tot));
      aw = (float)__dadd_rn(t1, __dmul_rn(one_m, (double)uwm));
    }
    ow[t] = wset ? aw : uwm;
    adapted_w[t] = aw;
  }
  const double rmp = adapt ? __drcp_rn(mp) : 0.0;  // the D quotients below share the divisor mp
  // centred statistics (the sparse kernel) or plain sums (cent null)
  const float* cr = cent ? cent + ((size_t)mod * n_chunks * 128 + (row >= 0 ? row : 0)) * D : nullptr;
  for (int k = lane; k < D; k += 32) {
    float am = um[k], av = uv[k];
    if (adapt && (upM || upV)) {
      // the statistics kernel's sums are centred on the component's mean (cr)
      const double c = cr ? (double)cr[k] : 0.0, Fc = col(k);
      const double a1 = gmm::div_by_rcp(__dmul_rn(alfa, gmm::tc_uncentre_F(Fc, mp, c)), mp, rmp);
      const double amd = __dadd_rn(a1, __dmul_rn(one_m, (double)um[k]));
      am = (float)amd;
      if (upV) {
        // FP64 variance update: the second moment of the adapted model less the square of the
        // adapted mean, both in FP64
        const double second = __dadd_rn((double)uv[k], __dmul_rn((double)um[k], (double)um[k]));
        const double b1 =
            gmm::div_by_rcp(__dmul_rn(alfa, gmm::tc_uncentre_S(col(tc_col_sq(K, k)), Fc, mp, c)), mp, rmp);
        const double b2 = __dadd_rn(b1, __dmul_rn(one_m, second));
        av = (float)__dsub_rn(b2, __dmul_rn(amd, amd));
        if (av < min_var) av = min_var;
      }
    }
    omu[(size_t)t * D + k] = am;
    ovar[(size_t)t * D + k] = av;
  }
}

// Weight renormalisation per MAP request (sequential FP64 sum in component order).
__global__ void srv_norm_kernel(int R, int M, const int* __restrict__ req_par,
                                const float* __restrict__ adapted_w, float* __restrict__ ow) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= R || !req_par[4 * r + 1]) return;
  double corr = 0.0;
  if (lane == 0)
    for (int m = 0; m < M; ++m) corr = __dadd_rn(corr, (double)adapted_w[(size_t)r * M + m]);
  corr = __shfl_sync(0xffffffffu, corr, 0);
  if (corr != 0.0) {
    const float fc = (float)corr;
    for (int m = lane; m < M; m += 32) ow[(size_t)r * M + m] = __fdiv_rn(ow[(size_t)r * M + m], fc);
  }
}

// Per-request total log-likelihood over its frames (fixed order).
__global__ void srv_ll_kernel(const long long* __restrict__ x0, const long long* __restrict__ n,
                              const float* __restrict__ ll, double* __restrict__ out) {
  __shared__ double red[32];
  const int r = blockIdx.x;
  double v = 0.0;
  for (long long f = threadIdx.x; f < n[r]; f += blockDim.x) v += (double)ll[x0[r] + f];
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    out[r] = s;
  }
}

__global__ void srv_row_of_comp_kernel(int M, int Mpad, const int* __restrict__ comp_of_row,
                                       int* __restrict__ row_of_comp) {
  for (int m = threadIdx.x; m < M; m += blockDim.x) row_of_comp[m] = -1;
  __syncthreads();
  for (int r = threadIdx.x; r < Mpad; r += blockDim.x)
    if (comp_of_row[r] >= 0) row_of_comp[comp_of_row[r]] = r;
}

}  // namespace

struct Server {
  Ctx c;  // device, compute stream, error flag, allocation accounting, profiling
  cudaStream_t copy_stream = nullptr;
  int D = 0, K = 0, M = 0, n_chunks = 0, max_models = 0, n_models = 0, FT = 128, FLUSH = 64;
  int max_batch = 4096;
  // resident models
  uint16_t* wplanes = nullptr;
  CUtensorMap wmap;
  float *mw = nullptr, *mmu = nullptr, *mvar = nullptr;
  int *mact = nullptr, *comp_of_row = nullptr, *row_of_comp = nullptr;
  float* cent = nullptr;  // [W plane rows][D] centres of the statistics sums
  std::vector<int> mact_host;
  // request arenas (device) and pinned staging, two of each
  size_t arena_bytes = 0;
  char* arena[2] = {nullptr, nullptr};
  char* hin[2] = {nullptr, nullptr};
  char* hout[2] = {nullptr, nullptr};
  size_t hin_bytes = 0, hout_bytes = 0;
  cudaEvent_t copied[2], finished[2];
  double* llpart = nullptr;
  // queue
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Req*> pending;
  std::unordered_map<long long, Req*> reqs;
  long long next_ticket = 1;
  bool stop = false;
  std::thread worker;
  std::string last_error;
  // counters
  long long n_batches = 0, n_done = 0, n_failed = 0;
  size_t peak_batch = 0;
  int err_code = GMM_OK;
};

namespace {

// Device bytes a request needs in an arena.
size_t footprint(const Server* s, long long N, int kind) {
  const long long rows = (N + 127) / 128 * 128;
  size_t b = align256((size_t)N * s->D * 4) + align256((size_t)rows * s->K * 2 * 3) + align256((size_t)rows * 4) +
             align256((size_t)rows * 8) + align256((size_t)(rows / 128) * 4) + align256((size_t)(rows / s->FT) * 4) +
             align256((size_t)N * 4) + 256;
  if (kind == GMM_REQ_MAP) {
    const long long tiles = rows / s->FT;
    const long long pieces = std::max<long long>(1, (tiles + s->FLUSH - 1) / s->FLUSH);
    b += (size_t)pieces * s->n_chunks * s->K * 128 * 8 + align256((size_t)s->M * 4 * 2) +
         2 * align256((size_t)s->M * s->D * 4) + 1024;
  }
  return b;
}

struct Batch {
  std::vector<Req*> reqs;  // layout order
  int slot = 0;            // arena / staging index
  size_t dev_bytes = 0;
  // device pointers inside the arena
  float* X = nullptr;
  size_t meta_bytes = 0;
  long long N = 0, Rpad = 0;
  long long* row_frame = nullptr;
  int* tile_wbase = nullptr;
  int* tile_slot = nullptr;
  uint16_t* zplanes = nullptr;
  float* ll2 = nullptr;
  float* ll = nullptr;
  double* part = nullptr;
  int4* work = nullptr;
  int n_work = 0;
  bool second_order = false;  // a MAP request of the batch updates variances
  long long* rx0 = nullptr;
  long long* rn = nullptr;
  double* rll = nullptr;
  int R_map = 0;
  int *m_model = nullptr, *m_piece0 = nullptr, *m_pieces = nullptr, *m_par = nullptr;
  long long* m_frames = nullptr;
  float *ow = nullptr, *omu = nullptr, *ovar = nullptr, *oaw = nullptr;
  // host staging offsets of the outputs
  size_t h_rll = 0, h_fll = 0, h_w = 0, h_mu = 0, h_var = 0;
};

struct Bump {
  char* base;
  size_t off = 0, cap;
  Bump(char* b, size_t c) : base(b), cap(c) {}
  template <typename T>
  T* take(size_t count) {
    T* p = reinterpret_cast<T*>(base + off);
    off = align256(off + count * sizeof(T));
    return p;
  }
};

// Lays out the admitted requests (MAP requests first, grouped by model; then scoring requests
// by model), fills the pinned input staging, and returns false if anything does not fit.
bool plan(Server* s, Batch& b) {
  std::stable_sort(b.reqs.begin(), b.reqs.end(), [](const Req* x, const Req* y) {
    if ((x->kind == GMM_REQ_MAP) != (y->kind == GMM_REQ_MAP)) return x->kind == GMM_REQ_MAP;
    return x->model < y->model;
  });
  long long rows = 0, frames = 0;
  int pieces = 0, R_map = 0;
  for (Req* r : b.reqs) {
    r->row0 = rows;
    r->rows = (r->N + 127) / 128 * 128;
    r->x0 = frames;
    rows += r->rows;
    frames += r->N;
    if (r->kind == GMM_REQ_MAP) {
      const long long tiles = r->rows / s->FT;
      r->piece0 = pieces;
      r->pieces = (int)std::max<long long>(1, (tiles + s->FLUSH - 1) / s->FLUSH);
      pieces += r->pieces;
      ++R_map;
    }
  }
  const int R = (int)b.reqs.size();
  b.N = frames;
  b.Rpad = rows;
  b.R_map = R_map;
  // statistics work items: per model, its MAP tiles split into ranges of whole pieces of about
  // equal size, one CTA per (range, W chunk of the model)
  std::vector<int4> work;
  const long long map_tiles = [&] {
    long long t = 0;
    for (Req* r : b.reqs)
      if (r->kind == GMM_REQ_MAP) t += r->rows / s->FT;
    return t;
  }();
  if (map_tiles > 0) {
    const int sms = s->c.sms > 0 ? s->c.sms : 148;
    const long long target = std::max<long long>(s->FLUSH / 4, map_tiles * s->n_chunks / std::max(1, sms));
    size_t i = 0;
    while (i < b.reqs.size() && b.reqs[i]->kind == GMM_REQ_MAP) {
      const int model = b.reqs[i]->model;
      long long t0 = b.reqs[i]->row0 / s->FT, acc = 0;
      long long cur = t0;
      for (; i < b.reqs.size() && b.reqs[i]->kind == GMM_REQ_MAP && b.reqs[i]->model == model; ++i) {
        const Req* r = b.reqs[i];
        const long long rt = r->rows / s->FT;
        for (int p = 0; p < r->pieces; ++p) {
          const long long pt = std::min<long long>(s->FLUSH, rt - (long long)p * s->FLUSH);
          acc += pt;
          cur += pt;
          if (acc >= target) {
            for (int ch = 0; ch < s->n_chunks; ++ch)
              work.push_back(make_int4(model * s->n_chunks + ch, ch, (int)t0, (int)(cur - t0)));
            t0 = cur;
            acc = 0;
          }
        }
      }
      if (cur > t0)
        for (int ch = 0; ch < s->n_chunks; ++ch)
          work.push_back(make_int4(model * s->n_chunks + ch, ch, (int)t0, (int)(cur - t0)));
    }
  }
  b.n_work = (int)work.size();
  // device arena layout
  Bump d(s->arena[b.slot], s->arena_bytes);
  b.row_frame = d.take<long long>((size_t)rows);
  b.tile_wbase = d.take<int>((size_t)rows / 128);
  b.tile_slot = d.take<int>((size_t)rows / s->FT);
  b.work = d.take<int4>(work.size());
  b.rx0 = d.take<long long>(R);
  b.rn = d.take<long long>(R);
  b.m_model = d.take<int>(R_map);
  b.m_piece0 = d.take<int>(R_map);
  b.m_pieces = d.take<int>(R_map);
  b.m_par = d.take<int>(4 * (size_t)R_map);
  b.m_frames = d.take<long long>(R_map);
  b.meta_bytes = d.off;  // everything above comes from the host in one copy
  b.X = d.take<float>((size_t)frames * s->D);
  const size_t in_bytes = d.off;
  b.zplanes = d.take<uint16_t>((size_t)3 * rows * s->K);
  b.ll2 = d.take<float>((size_t)rows);
  b.ll = d.take<float>((size_t)frames);
  b.part = d.take<double>((size_t)pieces * s->n_chunks * s->K * 128);
  const size_t out0 = d.off;  // outputs, copied back in one piece
  b.rll = d.take<double>(R);
  b.ow = d.take<float>((size_t)R_map * s->M);
  b.omu = d.take<float>((size_t)R_map * s->M * s->D);
  b.ovar = d.take<float>((size_t)R_map * s->M * s->D);
  const size_t out1 = d.off;
  b.oaw = d.take<float>((size_t)R_map * s->M);
  // staging holds the layout arrays and the frames of the requests that were copied at submit
  size_t staged_end = b.meta_bytes;
  for (const Req* r : b.reqs)
    if (!r->src) staged_end = std::max(staged_end, (size_t)((const char*)(b.X + (size_t)(r->x0 + r->N) * s->D) - s->arena[b.slot]));
  (void)in_bytes;
  if (d.off > d.cap || staged_end > s->hin_bytes) return false;
  b.dev_bytes = d.off;
  // host staging: same offsets as the device block for the inputs
  char* h = s->hin[b.slot];
  auto H = [&](const void* dp) { return h + ((const char*)dp - s->arena[b.slot]); };
  float* hx = reinterpret_cast<float*>(H(b.X));
  long long* hrf = reinterpret_cast<long long*>(H(b.row_frame));
  int* hwb = reinterpret_cast<int*>(H(b.tile_wbase));
  int* hts = reinterpret_cast<int*>(H(b.tile_slot));
  std::memcpy(H(b.work), work.data(), work.size() * sizeof(int4));
  long long* hx0 = reinterpret_cast<long long*>(H(b.rx0));
  long long* hn = reinterpret_cast<long long*>(H(b.rn));
  int* hmm = reinterpret_cast<int*>(H(b.m_model));
  int* hp0 = reinterpret_cast<int*>(H(b.m_piece0));
  int* hpn = reinterpret_cast<int*>(H(b.m_pieces));
  int* hpar = reinterpret_cast<int*>(H(b.m_par));
  long long* hmf = reinterpret_cast<long long*>(H(b.m_frames));
  int im = 0;
  for (int i = 0; i < R; ++i) {
    Req* r = b.reqs[i];
    if (!r->src) std::memcpy(hx + (size_t)r->x0 * s->D, r->frames.data(), (size_t)r->N * s->D * sizeof(float));
    for (long long k = 0; k < r->rows; ++k) hrf[r->row0 + k] = k < r->N ? r->x0 + k : -1;
    for (long long t = r->row0 / 128; t < (r->row0 + r->rows) / 128; ++t) hwb[t] = r->model * s->n_chunks;
    for (long long t = r->row0 / s->FT; t < (r->row0 + r->rows) / s->FT; ++t)
      hts[t] = r->kind == GMM_REQ_MAP ? r->piece0 + (int)((t - r->row0 / s->FT) / s->FLUSH) : 0;
    hx0[i] = r->x0;
    hn[i] = r->N;
    if (r->kind == GMM_REQ_MAP) {
      hmm[im] = r->model;
      hp0[im] = r->piece0;
      hpn[im] = r->pieces;
      hpar[4 * im] = r->tau;
      hpar[4 * im + 1] = r->upW;
      hpar[4 * im + 2] = r->upM;
      hpar[4 * im + 3] = r->upV;
      hmf[im] = r->N;
      if (r->upV) b.second_order = true;
      ++im;
    }
  }
  // output staging offsets (relative to out0)
  b.h_rll = (char*)b.rll - (s->arena[b.slot] + out0);
  b.h_w = (char*)b.ow - (s->arena[b.slot] + out0);
  b.h_mu = (char*)b.omu - (s->arena[b.slot] + out0);
  b.h_var = (char*)b.ovar - (s->arena[b.slot] + out0);
  b.h_fll = out1 - out0;  // per-frame LLs follow the outputs in the host staging
  if (out1 - out0 + (size_t)frames * 4 > s->hout_bytes) return false;
  return true;
}

// Enqueues one batch: H2D on the copy stream, kernels and D2H on the compute stream.
int launch(Server* s, Batch& b) {
  Ctx* c = &s->c;
  cudaError_t e = cudaMemcpyAsync(s->arena[b.slot], s->hin[b.slot], b.meta_bytes, cudaMemcpyHostToDevice, s->copy_stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "server: cudaMemcpyAsync(batch layout)");
  // frames: runs of consecutive staged requests in one copy each; no-copy requests straight
  // from the caller's memory
  const char* hx = s->hin[b.slot] + ((const char*)b.X - s->arena[b.slot]);
  const size_t fb = (size_t)s->D * sizeof(float);
  for (size_t i = 0; i < b.reqs.size() && e == cudaSuccess;) {
    const Req* r = b.reqs[i];
    if (r->src) {
      if (r->N > 0) e = cudaMemcpyAsync(b.X + (size_t)r->x0 * s->D, r->src, (size_t)r->N * fb, cudaMemcpyHostToDevice, s->copy_stream);
      ++i;
      continue;
    }
    size_t j = i;
    long long n = 0;
    while (j < b.reqs.size() && !b.reqs[j]->src) n += b.reqs[j++]->N;
    if (n > 0) e = cudaMemcpyAsync(b.X + (size_t)r->x0 * s->D, hx + (size_t)r->x0 * fb, (size_t)n * fb, cudaMemcpyHostToDevice, s->copy_stream);
    i = j;
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "server: cudaMemcpyAsync(batch frames)");
  cudaEventRecord(s->copied[b.slot], s->copy_stream);
  cudaStreamWaitEvent(c->stream, s->copied[b.slot], 0);
  // the statistics pieces (zeroed by the statistics launch, which adds into them)
  const long long pieces_bytes = (long long)((const char*)b.rll - (const char*)b.part);
  TcBatch t;
  t.D = s->D;
  t.K = s->K;
  t.n_chunks = s->n_chunks;
  t.w_chunks_total = s->max_models * s->n_chunks;
  t.wplanes = s->wplanes;
  t.cent = s->cent;
  t.wmap = &s->wmap;
  t.X = b.X;
  t.N = b.N;
  t.Rpad = b.Rpad;
  t.row_frame = b.row_frame;
  t.tile_wbase = b.tile_wbase;
  t.zplanes = b.zplanes;
  t.ll2 = b.ll2;
  t.ll = b.ll;
  t.llpart = s->llpart;
  t.n_work = b.n_work;
  t.work = b.work;
  t.tile_slot = b.tile_slot;
  t.part = b.part;
  t.part_bytes = (size_t)pieces_bytes;
  t.single_comp = s->M == 1;
  t.second_order = b.second_order;
  int rc = tc_run_batch(c, t);
  if (rc) return rc;
  const int R = (int)b.reqs.size();
  {
    GMM_LAUNCH(c, "srv_ll_kernel");
    srv_ll_kernel<<<R, 256, 0, c->stream>>>(b.rx0, b.rn, b.ll, b.rll);
  }
  if (b.R_map > 0) {
    {
      GMM_LAUNCH(c, "srv_map_kernel");
      const long long tot = (long long)b.R_map * s->M;
      srv_map_kernel<<<(unsigned)((tot + 7) / 8), 256, 0, c->stream>>>(
          b.R_map, s->M, s->D, s->K, s->n_chunks, b.m_model, b.m_piece0, b.m_pieces, b.m_frames, b.m_par,
          s->row_of_comp, gmm::tc_stats_centred(s->K, b.second_order) ? s->cent : nullptr, b.part, s->mw, s->mmu,
          s->mvar, c->min_var, b.ow, b.omu, b.ovar, b.oaw);
    }
    {
      GMM_LAUNCH(c, "srv_norm_kernel");
      srv_norm_kernel<<<(b.R_map + 7) / 8, 256, 0, c->stream>>>(b.R_map, s->M, b.m_par, b.oaw, b.ow);
    }
  }
  const size_t out_bytes = (size_t)((const char*)b.oaw - (const char*)b.rll);
  cudaMemcpyAsync(s->hout[b.slot], b.rll, out_bytes, cudaMemcpyDeviceToHost, c->stream);
  bool any_fll = false;
  for (Req* r : b.reqs) any_fll |= r->want_frame_ll != 0;
  if (any_fll && b.N > 0)
    cudaMemcpyAsync(s->hout[b.slot] + b.h_fll, b.ll, (size_t)b.N * 4, cudaMemcpyDeviceToHost, c->stream);
  cudaEventRecord(s->finished[b.slot], c->stream);
  return GMM_OK;
}

// Waits for a launched batch and hands its results to the requests.
void finish(Server* s, Batch& b) {
  cudaError_t e = cudaEventSynchronize(s->finished[b.slot]);
  int herr = 0;
  if (e == cudaSuccess) {
    cudaMemcpy(&herr, s->c.tc_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (herr) cudaMemset(s->c.tc_err, 0, sizeof(int));
  }
  const double t = now_ms();
  const char* h = s->hout[b.slot];
  const double* rll = reinterpret_cast<const double*>(h + b.h_rll);
  const float* fll = reinterpret_cast<const float*>(h + b.h_fll);
  std::lock_guard<std::mutex> lk(s->mu);
  int im = 0;
  for (size_t i = 0; i < b.reqs.size(); ++i) {
    Req* r = b.reqs[i];
    if (e != cudaSuccess || herr) {
      r->state = GMM_REQ_FAILED;
      r->status = e != cudaSuccess ? GMM_ERR_CUDA : GMM_ERR_TIMEOUT;
      r->err = e != cudaSuccess ? std::string("server batch: ") + cudaGetErrorString(e)
                                : "server batch: a bounded device wait expired";
      ++s->n_failed;
    } else {
      r->ll = rll[i];
      if (r->want_frame_ll) r->frame_ll.assign(fll + r->x0, fll + r->x0 + r->N);
      if (r->kind == GMM_REQ_MAP) {
        const size_t M = s->M, D = s->D;
        const float* w = reinterpret_cast<const float*>(h + b.h_w) + (size_t)im * M;
        const float* mu = reinterpret_cast<const float*>(h + b.h_mu) + (size_t)im * M * D;
        const float* var = reinterpret_cast<const float*>(h + b.h_var) + (size_t)im * M * D;
        r->w.assign(w, w + M);
        if (r->upM || r->upV) r->mu.assign(mu, mu + M * D);
        if (r->upV) r->var.assign(var, var + M * D);
      }
      r->state = GMM_REQ_DONE;
    }
    if (r->kind == GMM_REQ_MAP) ++im;
    r->frames.clear();
    r->frames.shrink_to_fit();
    r->t_done = t;
    ++s->n_done;
  }
  s->cv_done.notify_all();
}

void worker_loop(Server* s) {
  cudaSetDevice(s->c.device);
  Batch running;
  bool have_running = false;
  int slot = 0;
  for (;;) {
    Batch next;
    next.slot = slot;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (!have_running) s->cv_work.wait(lk, [&] { return s->stop || !s->pending.empty(); });
      if (s->stop && s->pending.empty() && !have_running) return;
      // admission: arrival order, while the footprint fits the free arena
      size_t used = 0, hin = 0, hout = 0;
      const double t = now_ms();
      while (!s->pending.empty() && (int)next.reqs.size() < s->max_batch) {
        Req* r = s->pending.front();
        if (r->foot > s->arena_bytes - kArenaSlack || r->hin_foot > s->hin_bytes - kArenaSlack ||
            r->hout_foot > s->hout_bytes - kArenaSlack) {  // can never fit
          s->pending.pop_front();
          r->state = GMM_REQ_FAILED;
          r->status = GMM_ERR_NOMEM;
          r->err = "request needs more device memory than the server's request arena";
          r->t_done = t;
          ++s->n_failed;
          s->cv_done.notify_all();
          continue;
        }
        if (used + r->foot > s->arena_bytes - kArenaSlack || hin + r->hin_foot > s->hin_bytes - kArenaSlack ||
            hout + r->hout_foot > s->hout_bytes - kArenaSlack)
          break;
        used += r->foot;
        hin += r->hin_foot;
        hout += r->hout_foot;
        s->pending.pop_front();
        r->state = GMM_REQ_RUNNING;
        r->t_admit = t;
        next.reqs.push_back(r);
      }
    }
    bool launched = false;
    if (!next.reqs.empty()) {
      int rc = plan(s, next) ? launch(s, next) : fail(&s->c, GMM_ERR_NOMEM, "server: batch layout does not fit");
      if (rc) {
        std::lock_guard<std::mutex> lk(s->mu);
        for (Req* r : next.reqs) {
          r->state = GMM_REQ_FAILED;
          r->status = rc;
          r->err = s->c.err;
          r->t_done = now_ms();
          ++s->n_failed;
        }
        s->cv_done.notify_all();
      } else {
        launched = true;
        std::lock_guard<std::mutex> lk(s->mu);
        ++s->n_batches;
        s->peak_batch = std::max(s->peak_batch, next.dev_bytes);
      }
    }
    if (have_running) {
      finish(s, running);
      have_running = false;
    }
    if (launched) {
      running = std::move(next);
      have_running = true;
      slot ^= 1;
    }
  }
}

}  // namespace
}  // namespace gmm

using gmm::Server;

extern "C" {

struct gmm_server_s : public Server {};

static thread_local std::string g_srv_create_err;

static int srv_fail(Server* s, int code, const std::string& m) {
  if (s) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->last_error = m;
  } else {
    g_srv_create_err = m;
  }
  return code;
}

const char* gmm_server_last_error(gmm_server s) {
  if (!s) return g_srv_create_err.c_str();
  return s->last_error.c_str();
}

int gmm_server_create(int device, int D, int M, int max_models, size_t request_bytes, gmm_server* out) {
  if (!out) return srv_fail(nullptr, GMM_ERR_ARG, "gmm_server_create: null output");
  *out = nullptr;
  if (D < 1 || D > 63) return srv_fail(nullptr, GMM_ERR_UNSUPPORTED, "gmm_server_create: the server runs the tensor-core path (1 <= D <= 63)");
  if (M < 1 || M > 32767 || max_models < 1) return srv_fail(nullptr, GMM_ERR_ARG, "gmm_server_create: bad M or model count");
  if (request_bytes < ((size_t)64 << 20)) return srv_fail(nullptr, GMM_ERR_ARG, "gmm_server_create: request memory below 64 MiB");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
    return srv_fail(nullptr, GMM_ERR_CUDA, "gmm_server_create: no CUDA device is available");
  if (device < 0 || device >= n) return srv_fail(nullptr, GMM_ERR_ARG, "gmm_server_create: device id out of range");
  cudaSetDevice(device);
  gmm_server_s* s = new (std::nothrow) gmm_server_s();
  if (!s) return srv_fail(nullptr, GMM_ERR_NOMEM, "gmm_server_create: out of host memory");
  gmm::Ctx* c = &s->c;
  c->device = device;
  cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking);
  cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
  s->D = D;
  s->M = M;
  s->K = gmm::tc_k(D);
  s->FT = gmm::tc_stats_ft(s->K);
  s->FLUSH = gmm::tc_flush_tiles(s->K);
  s->n_chunks = (M + 127) / 128;
  s->max_models = max_models;
  s->arena_bytes = request_bytes / 2;
  const long long wrows = (long long)max_models * s->n_chunks * 128;
  int rc = gmm::dalloc(c, (void**)&s->wplanes, (size_t)3 * wrows * s->K * 2, "server model planes");
  if (!rc) rc = gmm::dalloc(c, (void**)&s->mw, sizeof(float) * max_models * M, "server weights");
  if (!rc) rc = gmm::dalloc(c, (void**)&s->mmu, sizeof(float) * max_models * (size_t)M * D, "server means");
  if (!rc) rc = gmm::dalloc(c, (void**)&s->mvar, sizeof(float) * max_models * (size_t)M * D, "server variances");
  if (!rc) rc = gmm::dalloc(c, (void**)&s->mact, sizeof(int) * max_models * M, "server active lists");
  if (!rc) rc = gmm::dalloc(c, (void**)&s->comp_of_row, sizeof(int) * wrows, "server row maps");
  if (!rc) rc = gmm::dalloc(c, (void**)&s->row_of_comp, sizeof(int) * max_models * M, "server component rows");
  if (!rc) rc = gmm::dalloc(c, (void**)&s->cent, sizeof(float) * wrows * D, "server statistics centres");
  if (!rc) rc = gmm::dalloc(c, (void**)&s->llpart, sizeof(double) * 256 * 128, "server LL partials");
  if (!rc) rc = gmm::dalloc(c, (void**)&c->tc_err, sizeof(int), "server error flag");
  for (int i = 0; i < 2 && !rc; ++i) rc = gmm::dalloc(c, (void**)&s->arena[i], s->arena_bytes, "server request arena");
  if (!rc) {
    cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream);
    cudaMemsetAsync(s->wplanes, 0, (size_t)3 * wrows * s->K * 2, c->stream);
    rc = gmm::tc_make_wmap(c, &s->wmap, s->wplanes, wrows, s->K);
  }
  // pinned staging: the inputs are at most about a third of a request's device footprint
  // (frames and row maps, not the operand planes), the outputs a quarter of it
  s->hin_bytes = s->arena_bytes / 2;
  s->hout_bytes = s->arena_bytes / 4;
  for (int i = 0; i < 2 && !rc; ++i) {
    if (cudaMallocHost((void**)&s->hin[i], s->hin_bytes) != cudaSuccess ||
        cudaMallocHost((void**)&s->hout[i], s->hout_bytes) != cudaSuccess)
      rc = gmm::fail(c, GMM_ERR_NOMEM, "server: pinned staging");
    cudaEventCreateWithFlags(&s->copied[i], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&s->finished[i], cudaEventDisableTiming);
  }
  if (!rc && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = gmm::fail(c, GMM_ERR_CUDA, "server: set-up");
  if (rc) {
    g_srv_create_err = c->err;
    gmm_server_destroy(s);
    return rc;
  }
  s->worker = std::thread(gmm::worker_loop, s);
  *out = s;
  return GMM_OK;
}

int gmm_server_destroy(gmm_server s) {
  if (!s) return GMM_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  cudaSetDevice(s->c.device);
  cudaDeviceSynchronize();
  for (auto& kv : s->reqs) delete kv.second;
  for (int i = 0; i < 2; ++i) {
    if (s->arena[i]) cudaFree(s->arena[i]);
    if (s->hin[i]) cudaFreeHost(s->hin[i]);
    if (s->hout[i]) cudaFreeHost(s->hout[i]);
    if (s->copied[i]) cudaEventDestroy(s->copied[i]);
    if (s->finished[i]) cudaEventDestroy(s->finished[i]);
  }
  void* bufs[] = {s->wplanes,     s->mw,          s->mmu,  s->mvar,   s->mact,
                  s->comp_of_row, s->row_of_comp, s->cent, s->llpart, s->c.tc_err};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
  if (s->c.stream) cudaStreamDestroy(s->c.stream);
  delete s;
  return GMM_OK;
}

int gmm_server_set_options(gmm_server s, float min_loglike, float min_gamma, float min_var, int max_batch) {
  if (!s) return GMM_ERR_ARG;
  if (max_batch < 1) return srv_fail(s, GMM_ERR_ARG, "gmm_server_set_options: max_batch must be >= 1");
  std::lock_guard<std::mutex> lk(s->mu);
  s->c.minLL = min_loglike;
  s->c.minGamma = min_gamma;
  s->c.min_var = min_var;
  s->max_batch = max_batch;
  return GMM_OK;
}

int gmm_server_add_model(gmm_server s, const float* w, const float* mu, const float* var, int* model_id) {
  if (!s || !w || !mu || !var || !model_id) return GMM_ERR_ARG;
  const int M = s->M, D = s->D;
  std::vector<int> act;
  for (int m = 0; m < M; ++m) {
    if (w[m] > 0.0f) act.push_back(m);
    for (int d = 0; d < D; ++d)
      if (var[(size_t)m * D + d] < s->c.min_var)
        return srv_fail(s, GMM_ERR_MODEL, "insertModel(): model contains very low variances (< min_var)");
  }
  if (act.empty()) return srv_fail(s, GMM_ERR_MODEL, "model has no component with non-zero weight");
  int id;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->n_models >= s->max_models) return GMM_ERR_NOMEM;
    id = s->n_models;
  }
  gmm::Ctx* c = &s->c;
  cudaSetDevice(c->device);
  // a private stream: the worker may be running batches on the compute stream meanwhile
  cudaStream_t st;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  gmm::Ctx tmp;
  tmp.device = c->device;
  tmp.stream = st;
  const size_t md = (size_t)M * D;
  cudaMemcpyAsync(s->mw + (size_t)id * M, w, sizeof(float) * M, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(s->mmu + (size_t)id * md, mu, sizeof(float) * md, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(s->mvar + (size_t)id * md, var, sizeof(float) * md, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(s->mact + (size_t)id * M, act.data(), sizeof(int) * act.size(), cudaMemcpyHostToDevice, st);
  const int Mpad = s->n_chunks * 128;
  gmm::tc_build_model(&tmp, D, s->K, (int)act.size(), Mpad, (long long)s->max_models * Mpad,
                      (long long)id * Mpad, s->mact + (size_t)id * M, s->mw + (size_t)id * M,
                      s->mmu + (size_t)id * md, s->mvar + (size_t)id * md, s->wplanes,
                      s->comp_of_row + (size_t)id * Mpad, s->cent);
  gmm::srv_row_of_comp_kernel<<<1, 1024, 0, st>>>(M, Mpad, s->comp_of_row + (size_t)id * Mpad,
                                                  s->row_of_comp + (size_t)id * M);
  cudaError_t e = cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  if (e != cudaSuccess) return srv_fail(s, GMM_ERR_CUDA, std::string("gmm_server_add_model: ") + cudaGetErrorString(e));
  std::lock_guard<std::mutex> lk(s->mu);
  s->mact_host.push_back((int)act.size());
  s->n_models = id + 1;
  *model_id = id;
  return GMM_OK;
}

int gmm_server_submit(gmm_server s, int kind, int model_id, const float* frames, long long N, int tau,
                      int up_w, int up_m, int up_v, int options, long long* ticket) {
  if (!s || !ticket || (N > 0 && !frames)) return GMM_ERR_ARG;
  if (kind != GMM_REQ_SCORE && kind != GMM_REQ_MAP) return srv_fail(s, GMM_ERR_ARG, "gmm_server_submit: unknown request kind");
  if (N < 0 || (kind == GMM_REQ_MAP && tau < 1)) return srv_fail(s, GMM_ERR_ARG, "gmm_server_submit: bad frame count or tau");
  gmm::Req* r = new (std::nothrow) gmm::Req();
  if (!r) return GMM_ERR_NOMEM;
  r->kind = kind;
  r->model = model_id;
  r->N = N;
  if (options & GMM_SUBMIT_NO_COPY) r->src = frames;
  else r->frames.assign(frames, frames + (size_t)N * s->D);
  r->tau = tau;
  r->upW = up_w;
  r->upM = up_m;
  r->upV = up_v;
  r->want_frame_ll = (options & GMM_SUBMIT_FRAME_LL) != 0;
  r->foot = gmm::footprint(s, N, kind);
  {
    const size_t rows = (size_t)((N + 127) / 128 * 128);
    r->hin_foot = gmm::align256((r->src ? 0 : (size_t)N * s->D * 4) + rows * 8 + rows / 128 * 4 + rows / s->FT * 4) + 1024;
    r->hout_foot = gmm::align256(8 + (size_t)N * 4 +
                                 (kind == GMM_REQ_MAP ? (size_t)s->M * 4 * (2 + 2 * s->D) : 0)) + 1024;
  }
  r->t_submit = gmm::now_ms();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (model_id < 0 || model_id >= s->n_models) {
      delete r;
      s->last_error = "gmm_server_submit: unknown model id";
      return GMM_ERR_ARG;
    }
    r->ticket = s->next_ticket++;
    s->reqs[r->ticket] = r;
    s->pending.push_back(r);
    *ticket = r->ticket;
  }
  s->cv_work.notify_one();
  return GMM_OK;
}

int gmm_server_poll(gmm_server s, long long ticket, int* state) {
  if (!s || !state) return GMM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) {
    s->last_error = "gmm_server_poll: unknown ticket";
    return GMM_ERR_ARG;
  }
  *state = it->second->state;
  return GMM_OK;
}

int gmm_server_wait(gmm_server s, long long ticket, int timeout_ms) {
  if (!s) return GMM_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) {
    s->last_error = "gmm_server_wait: unknown ticket";
    return GMM_ERR_ARG;
  }
  gmm::Req* r = it->second;
  auto done = [&] { return r->state == GMM_REQ_DONE || r->state == GMM_REQ_FAILED; };
  if (timeout_ms < 0) s->cv_done.wait(lk, done);
  else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) return GMM_ERR_TIMEOUT;
  return GMM_OK;
}

int gmm_server_result(gmm_server s, long long ticket, double* total_ll, float* frame_ll, float* w, float* mu,
                      float* var, double* latency_ms) {
  if (!s) return GMM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) {
    s->last_error = "gmm_server_result: unknown ticket";
    return GMM_ERR_ARG;
  }
  gmm::Req* r = it->second;
  if (r->state != GMM_REQ_DONE && r->state != GMM_REQ_FAILED) {
    s->last_error = "gmm_server_result: request not finished";
    return GMM_ERR_STATE;
  }
  const int status = r->status;
  if (status != GMM_OK) s->last_error = r->err;
  if (status == GMM_OK) {
    if (total_ll) *total_ll = r->ll;
    if (frame_ll && !r->frame_ll.empty()) std::memcpy(frame_ll, r->frame_ll.data(), r->frame_ll.size() * 4);
    if (w && !r->w.empty()) std::memcpy(w, r->w.data(), r->w.size() * 4);
    if (mu && !r->mu.empty()) std::memcpy(mu, r->mu.data(), r->mu.size() * 4);
    if (var && !r->var.empty()) std::memcpy(var, r->var.data(), r->var.size() * 4);
    if (latency_ms) *latency_ms = r->t_done - r->t_submit;
  }
  s->reqs.erase(it);
  delete r;
  return status;
}

int gmm_server_stats(gmm_server s, long long* batches, long long* completed, long long* failed,
                     size_t* peak_batch_bytes) {
  if (!s) return GMM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (batches) *batches = s->n_batches;
  if (completed) *completed = s->n_done;
  if (failed) *failed = s->n_failed;
  if (peak_batch_bytes) *peak_batch_bytes = s->peak_batch;
  return GMM_OK;
}

}  // extern "C"
