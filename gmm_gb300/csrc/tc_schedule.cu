// Sparse tile schedule of the tensor-core statistics kernel.
//
// At minGamma = 1e-4 a frame keeps a posterior for a handful of components (7.6 of 2048 on
// average in UBM EM at N = 200k, M = 2048, D = 39), yet the dense statistics kernel multiplies
// every 128-frame tile by every 128-component chunk. The schedule removes the (tile, chunk)
// pairs whose posteriors are all pruned, which leaves the statistics unchanged:
//
//  1. Components are grouped into chunks that lie together in feature space: the active list is
//     cut by balanced recursive bisection, each cut along the mean coordinate of largest spread
//     (group_level_kernel). A frame's kept components then fall into one or two chunks (1.5 on
//     average at the shape above, against 5.6 chunks for chunks taken in index order).
//  2. The logits kernel, which sees every logit to form the frame's log-sum-exp, records per
//     frame the chunks holding a logit within log2(minGamma) - margin of it (a bit mask).
//  3. The frames are sorted by that mask (stable LSD radix sort, 8 bits a pass), the operand
//     planes and LSE values of the sorted frames are written out, and each sorted tile gets the
//     union of its frames' masks: 1.85 active chunks per tile instead of 16.
//  4. Every chunk gets the list of its active tiles (tile_list_kernel), the lists are cut into
//     work items of about equal length for a fixed grid (work_items_kernel), and the statistics
//     kernel runs over the items; reduce_items_kernel adds each chunk's item partials in item
//     order.
//
// Skipping is exact: a pair is dropped only if its largest logit is at least `margin` below the
// pruning threshold, and the two kernels' logits of a pair differ by far less than the margin
// (the same split-bf16 products, accumulated in a different order). Everything is deterministic
// (the sort is stable, the lists are in tile order), and every launch has a fixed shape, so the
// schedule can be captured in a CUDA graph.
#include <limits.h>

#include "gmm_internal.cuh"

namespace gmm {
namespace {

constexpr int kSortBlock = 4096;  // keys per block of the radix sort (256 threads x 16 rounds)
constexpr int kGroupMax = 4096;   // components the grouping sorts in one block

// One level of the balanced bisection: block s owns the chunk range reached from [0, chunks)
// by the bits of s (most significant first) and, if it spans two chunks or more, sorts its
// components along the mean coordinate of largest spread (ties by component index).
__global__ void __launch_bounds__(1024) group_level_kernel(int level, const int* __restrict__ mact_dev, int Mact,
                                                           int D, const float* __restrict__ mu,
                                                           int* __restrict__ gact) {
  __shared__ float key[kGroupMax];
  __shared__ int idx[kGroupMax];
  __shared__ float vsum[16][64][2];
  __shared__ int axis;
  if (mact_dev) Mact = *mact_dev;
  const int nch = (Mact + 127) / 128;
  int lo = 0, hi = nch;
  for (int l = level - 1; l >= 0; --l) {
    const int mid = lo + (hi - lo) / 2;
    if ((blockIdx.x >> l) & 1) lo = mid;
    else hi = mid;
  }
  if (hi - lo < 2) return;
  const int a = lo * 128, b = min(hi * 128, Mact), n = b - a;
  if (n > kGroupMax) return;  // the host enables the schedule only for Mact <= 4096
  const int tid = threadIdx.x;
  // spread of each mean coordinate over the segment: thread = (dimension, part of the
  // components), sums of the values shifted by the segment's first component (FP32)
  {
    const int d = tid & 63, part = tid >> 6;  // 16 parts of 64 dimensions
    float s1 = 0.0f, s2 = 0.0f;
    if (d < D) {
      const float v0 = mu[(size_t)gact[a] * D + d];
      for (int i = part; i < n; i += 16) {
        const float v = mu[(size_t)gact[a + i] * D + d] - v0;
        s1 += v;
        s2 = fmaf(v, v, s2);
      }
    }
    vsum[part][d][0] = s1;
    vsum[part][d][1] = s2;
  }
  __syncthreads();
  if (tid < 64) {
    float s1 = 0.0f, s2 = 0.0f;
    for (int p = 0; p < 16; ++p) {
      s1 += vsum[p][tid][0];
      s2 += vsum[p][tid][1];
    }
    vsum[0][tid][0] = tid < D ? s2 / n - (s1 / n) * (s1 / n) : -1.0f;
  }
  __syncthreads();
  if (tid == 0) {
    int best_d = 0;
    float best_v = vsum[0][0][0];
    for (int d = 1; d < D; ++d)
      if (vsum[0][d][0] > best_v) {
        best_v = vsum[0][d][0];
        best_d = d;
      }
    axis = best_d;
  }
  __syncthreads();
  const int ax = axis;
  int P = 1;
  while (P < n) P <<= 1;
  for (int i = tid; i < P; i += blockDim.x) {
    if (i < n) {
      idx[i] = gact[a + i];
      key[i] = mu[(size_t)idx[i] * D + ax];
    } else {
      idx[i] = INT_MAX;
      key[i] = INFINITY;
    }
  }
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < P; i += blockDim.x) {
        const int p = i ^ j;
        if (p > i) {
          const bool up = (i & k) == 0;
          const bool gt = key[i] > key[p] || (key[i] == key[p] && idx[i] > idx[p]);
          if (gt == up) {
            const float tk = key[i];
            key[i] = key[p];
            key[p] = tk;
            const int ti = idx[i];
            idx[i] = idx[p];
            idx[p] = ti;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int i = tid; i < n; i += blockDim.x) gact[a + i] = idx[i];
}

// Radix sort, one 8-bit digit per pass: per-block digit counts (digit-major), their exclusive
// scan, then a stable scatter.
__global__ void __launch_bounds__(256) radix_hist_kernel(const uint32_t* __restrict__ keys, long long n, int shift,
                                                         int* __restrict__ hist, int nb) {
  __shared__ int h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kSortBlock;
  for (int i = threadIdx.x; i < kSortBlock; i += 256) {
    const long long k = base + i;
    if (k < n) atomicAdd(&h[(keys[k] >> shift) & 255], 1);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * nb + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of one digit's per-block counts (block d = digit d) and the digit's total.
__global__ void __launch_bounds__(1024) radix_scan_digit_kernel(int* __restrict__ hist, int nb,
                                                                int* __restrict__ dtot) {
  __shared__ int wsum[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int* h = hist + (size_t)blockIdx.x * nb;
  const int per = (nb + 1023) / 1024;
  const int a = min(nb, tid * per), b = min(nb, a + per);
  int s = 0;
  for (int i = a; i < b; ++i) s += h[i];
  int incl = s;
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const int v = wsum[lane];
    int wi = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += u;
    }
    wsum[lane] = wi - v;  // exclusive prefix of the warps
    if (lane == 31) dtot[blockIdx.x] = wi;
  }
  __syncthreads();
  int run = wsum[warp] + incl - s;
  for (int i = a; i < b; ++i) {
    const int v = h[i];
    h[i] = run;
    run += v;
  }
}

// Exclusive scan of the 256 digit totals: the first output position of each digit.
__global__ void __launch_bounds__(256) radix_scan_totals_kernel(int* __restrict__ dtot) {
  __shared__ int t[256];
  const int tid = threadIdx.x;
  t[tid] = dtot[tid];
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {
    const int v = tid >= o ? t[tid - o] : 0;
    __syncthreads();
    t[tid] += v;
    __syncthreads();
  }
  dtot[tid] = tid ? t[tid - 1] : 0;
}

// Each block writes its keys in their original order: 16 rounds of 256 keys, the keys of a
// round ranked by warp, then by lane within the warp (lanes with the same digit found with
// match.any), on top of the block's running offset per digit.
__global__ void __launch_bounds__(256) radix_scatter_kernel(const uint32_t* __restrict__ kin, const int* __restrict__ vin,
                                                            uint32_t* __restrict__ kout, int* __restrict__ vout,
                                                            long long n, int shift, const int* __restrict__ hist,
                                                            int nb, const int* __restrict__ dbase) {
  __shared__ int base[256];
  __shared__ int tot[256];
  __shared__ int wcnt[8][256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  base[tid] = dbase[tid] + hist[(size_t)tid * nb + blockIdx.x];
  for (int round = 0; round < kSortBlock / 256; ++round) {
    const long long k = (long long)blockIdx.x * kSortBlock + round * 256 + tid;
    const bool valid = k < n;
    const uint32_t key = valid ? kin[k] : 0u;
    const int val = valid ? (vin ? vin[k] : (int)k) : 0;
    const int dig = valid ? (int)((key >> shift) & 255) : 256;
#pragma unroll
    for (int w = 0; w < 8; ++w) wcnt[w][tid] = 0;
    __syncthreads();
    const unsigned peers = __match_any_sync(0xffffffffu, dig);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && lane == __ffs(peers) - 1) wcnt[warp][dig] = __popc(peers);
    __syncthreads();
    {
      int run = 0;
#pragma unroll
      for (int w = 0; w < 8; ++w) {
        const int cnt = wcnt[w][tid];
        wcnt[w][tid] = run;
        run += cnt;
      }
      tot[tid] = run;
    }
    __syncthreads();
    if (valid) {
      const int pos = base[dig] + wcnt[warp][dig] + rank;
      kout[pos] = key;
      vout[pos] = val;
    }
    __syncthreads();
    base[tid] += tot[tid];
  }
}

// Block c: the sorted tiles whose mask has bit c, in tile order.
__global__ void __launch_bounds__(1024) tile_list_kernel(const uint32_t* __restrict__ tmask, int nT,
                                                         int* __restrict__ lists, int* __restrict__ counts) {
  __shared__ int wsum[32];
  __shared__ int total;
  const int c = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  int run = 0;
  for (int base = 0; base < nT; base += blockDim.x) {
    const int t = base + tid;
    const bool on = t < nT && ((tmask[t] >> c) & 1u);
    const unsigned bal = __ballot_sync(0xffffffffu, on);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    if (warp == 0) {
      const int v = lane < nw ? wsum[lane] : 0;
      int incl = v;
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
      }
      if (lane < nw) wsum[lane] = incl - v;
      if (lane == 31) total = incl;
    }
    __syncthreads();
    if (on) lists[(size_t)c * nT + run + wsum[warp] + __popc(bal & ((1u << lane) - 1u))] = t;
    run += total;
    __syncthreads();
  }
  if (tid == 0) counts[c] = run;
}

// Work items {W chunk, 0, list offset, tiles} for a grid of `grid` CTAs: every chunk's list cut
// into pieces of L tiles, L chosen so that the pieces fit the grid (at least 4 tiles a piece).
// item_off[c] = first item of chunk c; item_off[chunks] = number of items.
__global__ void work_items_kernel(const int* __restrict__ counts, int chunks, int nT, int grid, int4* __restrict__ work,
                                  int* __restrict__ item_off) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  long long P = 0;
  for (int c = 0; c < chunks; ++c) P += counts[c];
  const long long G = grid - chunks > 1 ? grid - chunks : 1;
  long long L = (P + G - 1) / G;
  if (L < 4) L = 4;
  int b = 0;
  for (int c = 0; c < chunks; ++c) {
    item_off[c] = b;
    for (long long k = 0; k * L < counts[c] && b < grid; ++k) {
      const long long nt = counts[c] - k * L < L ? counts[c] - k * L : L;
      work[b++] = make_int4(c, 0, (int)((long long)c * nT + k * L), (int)nt);
    }
  }
  item_off[chunks] = b;
}

// part [item][K][128] -> stats (caller order): thread = (chunk, d, row) adds n, F_d and S_d of
// the chunk's items in item order; with cent (sums centred on the row's centre, from the sparse
// statistics kernel) it adds the centre back in FP64.
__global__ void reduce_items_kernel(int M, int D, int K, int Mrows, int chunks, const int* __restrict__ item_off,
                                    const int* __restrict__ comp_of_row, const float* __restrict__ cent,
                                    const double* __restrict__ part, int flags, double* __restrict__ stats) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)chunks * D * 128) return;
  const int rr = (int)(t & 127), d = (int)((t >> 7) % D), ch = (int)(t / (128LL * D));
  const int r = ch * 128 + rr;
  if (r >= Mrows) return;
  const int m = comp_of_row[r];
  if (m < 0) return;  // padding row
  const bool sv = (flags & GMM_ACC_VAR) != 0;
  double n = 0.0, F = 0.0, S = 0.0;
  for (int b = item_off[ch]; b < item_off[ch + 1]; ++b) {
    const double* p = part + (size_t)b * K * 128 + rr;
    n += p[(size_t)D * 128];
    F += p[(size_t)d * 128];
    if (sv) S += p[(size_t)(K / 2 + d) * 128];
  }
  const double c = cent ? (double)cent[(size_t)r * D + d] : 0.0;
  if (d == 0) stats[m] += n;
  if (flags & GMM_ACC_MEAN) stats[(size_t)M + (size_t)m * D + d] += tc_uncentre_F(F, n, c);
  if (sv) stats[(size_t)M + (size_t)M * D + (size_t)m * D + d] += tc_uncentre_S(S, F, n, c);
}

}  // namespace

bool sched_supported(int chunks, int Mact) { return chunks >= 1 && chunks <= kSchedChunksMax && Mact <= kGroupMax; }

namespace {
// Frees the buffers that depend on the frame count (their sizes from s.Npad and s.K).
void free_frame_buffers(Ctx* c, TileSched& s) {
  const size_t Np = (size_t)s.Npad, nb = (size_t)((s.Npad + kSortBlock - 1) / kSortBlock);
  dfree(c, s.fmask, sizeof(uint32_t) * Np);
  dfree(c, s.kbuf, 2 * sizeof(uint32_t) * Np);
  dfree(c, s.vbuf, 2 * sizeof(int) * Np);
  dfree(c, s.hist, sizeof(int) * 256 * (nb + 1));
  dfree(c, s.planes, (size_t)3 * Np * s.K * sizeof(uint16_t));
  dfree(c, s.ll2, sizeof(float) * Np);
  dfree(c, s.tmask, sizeof(uint32_t) * (Np / 128));
  dfree(c, s.srow, sizeof(long long) * Np);
  s.srow = nullptr;
  s.fmask = s.kbuf = s.tmask = nullptr;
  s.vbuf = s.hist = nullptr;
  s.perm = nullptr;
  s.planes = nullptr;
  s.ll2 = nullptr;
  s.Npad = 0;
  s.K = 0;
}

void free_list_buffers(Ctx* c, TileSched& s) {
  dfree(c, s.lists, sizeof(int) * (size_t)s.chunks * s.lists_nT);
  dfree(c, s.counts, sizeof(int) * (size_t)(s.chunks + 2));
  s.lists = s.counts = nullptr;
  s.chunks = 0;
  s.lists_nT = 0;
}
}  // namespace

int sched_prepare(Ctx* c, long long Npad, int K, int chunks) {
  TileSched& s = c->sched;
  const long long nT = Npad / 128;
  const size_t nb = (size_t)((Npad + kSortBlock - 1) / kSortBlock);
  if (s.Npad != Npad || s.K != K) {
    free_frame_buffers(c, s);
    int rc = dalloc(c, (void**)&s.fmask, sizeof(uint32_t) * Npad, "tile schedule masks");
    if (!rc) rc = dalloc(c, (void**)&s.kbuf, 2 * sizeof(uint32_t) * Npad, "tile schedule sort keys");
    if (!rc) rc = dalloc(c, (void**)&s.vbuf, 2 * sizeof(int) * Npad, "tile schedule sort values");
    if (!rc) rc = dalloc(c, (void**)&s.hist, sizeof(int) * 256 * (nb + 1), "tile schedule histogram");
    if (!rc) rc = dalloc(c, (void**)&s.planes, (size_t)3 * Npad * K * sizeof(uint16_t), "sorted feature planes");
    if (!rc) rc = dalloc(c, (void**)&s.ll2, sizeof(float) * Npad, "sorted frame LSE");
    if (!rc) rc = dalloc(c, (void**)&s.tmask, sizeof(uint32_t) * nT, "tile masks");
    if (!rc) rc = dalloc(c, (void**)&s.srow, sizeof(long long) * Npad, "sorted row frames");

    s.Npad = Npad;  // set before a failure too, so that the sizes of what was allocated are known
    s.K = K;
    if (rc) {
      free_frame_buffers(c, s);
      return rc;
    }
  }
  if (s.chunks != chunks || s.lists_nT != nT) {
    free_list_buffers(c, s);
    s.chunks = chunks;
    s.lists_nT = nT;
    int rc = dalloc(c, (void**)&s.lists, sizeof(int) * (size_t)chunks * nT, "tile lists");
    if (!rc) rc = dalloc(c, (void**)&s.counts, sizeof(int) * (chunks + 2), "tile list counts");
    if (rc) {
      free_list_buffers(c, s);
      return rc;
    }
  }
  if (!s.work) {
    int rc = dalloc(c, (void**)&s.work, sizeof(int4) * kSchedGridMax, "work items");
    if (!rc) rc = dalloc(c, (void**)&s.item_off, sizeof(int) * (kSchedChunksMax + 2), "work item offsets");
    if (rc) return rc;
  }
  if (s.gact_cap < c->M) {
    dfree(c, s.gact, sizeof(int) * (size_t)s.gact_cap);
    s.gact = nullptr;
    s.gact_cap = 0;
    int rc = dalloc(c, (void**)&s.gact, sizeof(int) * c->M, "grouped active list");
    if (rc) return rc;
    s.gact_cap = c->M;
  }
  return GMM_OK;
}

void sched_free(Ctx* c) {
  TileSched& s = c->sched;
  free_frame_buffers(c, s);
  free_list_buffers(c, s);
  dfree(c, s.work, sizeof(int4) * kSchedGridMax);
  dfree(c, s.item_off, sizeof(int) * (kSchedChunksMax + 2));
  dfree(c, s.gact, sizeof(int) * (size_t)s.gact_cap);
  s.work = nullptr;
  s.item_off = nullptr;
  s.gact = nullptr;
  s.gact_cap = 0;
}

void sched_group(Ctx* c, const int* act, int Mact, const int* mact_dev, int chunks, int D, const float* mu) {
  TileSched& s = c->sched;
  cudaMemcpyAsync(s.gact, act, sizeof(int) * c->M, cudaMemcpyDeviceToDevice, c->stream);
  int levels = 0;
  while ((1 << levels) < chunks) ++levels;
  for (int l = 0; l < levels; ++l) {
    GMM_LAUNCH(c, "tc_group_kernel");
    group_level_kernel<<<1 << l, 1024, 0, c->stream>>>(l, mact_dev, Mact, D, mu, s.gact);
  }
}

void sched_sort(Ctx* c, long long Npad, int chunks) {
  TileSched& s = c->sched;
  const int nb = (int)((Npad + kSortBlock - 1) / kSortBlock);
  const int passes = (chunks + 7) / 8;
  const uint32_t* kin = s.fmask;
  const int* vin = nullptr;
  for (int p = 0; p < passes; ++p) {
    uint32_t* kout = s.kbuf + (size_t)(p & 1) * Npad;
    int* vout = s.vbuf + (size_t)(p & 1) * Npad;
    {
      GMM_LAUNCH(c, "tc_sort_hist_kernel");
      radix_hist_kernel<<<nb, 256, 0, c->stream>>>(kin, Npad, 8 * p, s.hist, nb);
    }
    {
      GMM_LAUNCH(c, "tc_sort_scan_kernel");
      radix_scan_digit_kernel<<<256, 1024, 0, c->stream>>>(s.hist, nb, s.hist + 256 * (size_t)nb);
    }
    {
      GMM_LAUNCH(c, "tc_sort_scan_kernel");
      radix_scan_totals_kernel<<<1, 256, 0, c->stream>>>(s.hist + 256 * (size_t)nb);
    }
    {
      GMM_LAUNCH(c, "tc_sort_scatter_kernel");
      radix_scatter_kernel<<<nb, 256, 0, c->stream>>>(kin, vin, kout, vout, Npad, 8 * p, s.hist, nb,
                                                      s.hist + 256 * (size_t)nb);
    }
    kin = kout;
    vin = vout;
  }
  s.perm = s.vbuf + (size_t)((passes - 1) & 1) * Npad;
}

void sched_lists(Ctx* c, long long Npad, int chunks, int grid) {
  TileSched& s = c->sched;
  const int nT = (int)(Npad / 128);
  {
    GMM_LAUNCH(c, "tc_tile_list_kernel");
    tile_list_kernel<<<chunks, 1024, 0, c->stream>>>(s.tmask, nT, s.lists, s.counts);
  }
  {
    GMM_LAUNCH(c, "tc_work_items_kernel");
    work_items_kernel<<<1, 32, 0, c->stream>>>(s.counts, chunks, nT, grid, s.work, s.item_off);
  }
}

void sched_reduce(Ctx* c, int K, int Mrows, int chunks, const int* comp_of_row, const float* cent,
                  const double* part, int flags) {
  GMM_LAUNCH(c, "tc_reduce_kernel");
  const long long tot = (long long)chunks * c->D * 128;
  reduce_items_kernel<<<(int)((tot + 255) / 256), 256, 0, c->stream>>>(c->M, c->D, K, Mrows, chunks,
                                                                       c->sched.item_off, comp_of_row, cent, part,
                                                                       flags, c->stats);
}

}  // namespace gmm
