// Device-side iteration control of the recovery loop (Demo1::Run,
// src/demo1.cc:36-59), so that a whole solve runs as one CUDA graph whose
// iteration body sits under a conditional while node.
//
// k_plan (before each iteration, one thread per signal) computes what the
// reference computes on the host at the start of Iterate: the number of bins
// B = max(2 (k - found) + 1, min_bins), NumBits, the window scalars
// (src/window.cc:28-51, with explicitly rounded FP64 operations so that they
// equal the host's values bit for bit), the thresholds 3 sigma / sqrt(B) and
// sigma / sqrt(B), and takes the iteration's transform and q's from the draw
// table the host filled from the signal's RNG in the reference's order
// (with each trial's row phase e^{2 pi i (b q mod n)/n}, computed there).
// k_finish (after the merge) applies the stop rule: count the iteration, a
// stale one when nothing was found, stop after max_stale_iter stale ones (never
// reset), on a status, or at max_iter; then it sets the while condition to
// "some signal still has work and draws".
//
// Fixed bins: once 2 (k - found) + 1 <= min_bins, every later iteration of a
// signal has bins = min_bins (found never decreases). When every signal of a
// batch is there, the next iteration can be planned ahead ("ahead" plan,
// into a second descriptor array) and its gather/fold run while the current
// iteration decides; k_finish then drops the planned iteration of a signal
// that stopped.
#include <algorithm>

#include "common.cuh"
#include "launch.h"

namespace mpsft {

thread_local bool g_launch_pdl = false;

namespace {

__device__ int32_t NumBitsDev(int32_t n, int32_t bins) {
  if (n < bins) return 1;
  int32_t out = 0;
  while (n >= bins) {
    n >>= 1;
    ++out;
  }
  return out;
}

__device__ inline int32_t NextBins(const SolveCtl &c, const SigIter &it) {
  const int32_t found = *it.tab_count;
  int32_t bins = (c.k - found) * 2 + 1;
  if (bins < c.min_bins) bins = c.min_bins;
  return bins;
}

// max_bins: signals needing more bins wait (the launch shapes of this body
// do not cover them). ahead = 1 plans iteration iter + 1 of a signal in the
// fixed-bins state while iteration iter runs (bins = min_bins; the flags,
// which iteration iter still uses, are cleared by its k_finish instead).
__global__ void k_plan(SolveCtl *__restrict__ ctl, SigIter *__restrict__ its,
                       int nsig, int32_t max_bins, int ahead) {
  PdlEnter(its, kTracePlan);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsig) return;
  SolveCtl &c = ctl[i];
  SigIter &it = its[i];
  const int local = c.iter + ahead - c.draw_base;
  if (c.done || local >= c.draws_avail) {
    it.active = 0;
    return;
  }
  const int32_t bins = ahead ? c.min_bins : NextBins(c, it);
  if (bins > max_bins) {
    it.active = 0;
    return;
  }
  if (ahead && it.fold_alt != nullptr) {
    // the planned iteration folds (and stashes its samples) into the
    // buffers this one's row transforms and re-binning do not read
    void *f = it.fold;
    it.fold = it.fold_alt;
    it.fold_alt = f;
    unsigned char *st = it.stash;
    it.stash = it.stash_alt;
    it.stash_alt = st;
  }
  // Everything that depends on the bins only (and on the signal's constants)
  // stays from the previous iteration when the bins repeat (most late
  // iterations): the window scalars, fixed-point constants and thresholds
  // are a chain of FP64 divisions, square roots and 128-bit divisions, each a
  // long sequence on this part.
  const bool same_bins = it.bins == bins;
  const double B = double(bins);
  if (!same_bins) {
    // Window scalars in the reference's operation order, no contraction.
    const double width = __ddiv_rn(1.0, __dmul_rn(2.0, B));
    const double sq = c.sqrt_c_delta;
    const double sigma_f =
        __ddiv_rn(0.5, __dmul_rn(__dmul_rn(__dmul_rn(B, 2.0), M_SQRT2), sq));
    const double sigma_t = __ddiv_rn(1.0, __dmul_rn(2.0 * M_PI, sigma_f));
    const double tmp =
        __dadd_rn(__dmul_rn(__dmul_rn(2.0 * M_SQRT2, sigma_t), sq), 1.0);
    int32_t f = int32_t(ceil(__ddiv_rn(tmp, B)));
    if (f % 2 == 0) ++f;
    const int32_t bits = NumBitsDev(it.n, bins);
    it.bins = bins;
    it.bits = bits;
    it.rows = 1 + 2 * bits;
    it.folds = f;
    it.p = f * bins;
    it.p2 = (it.p - 1) / 2;
    it.width = width;
    it.sigma_f = sigma_f;
    it.erf_d = __dmul_rn(M_SQRT2 * M_PI, sigma_t);
    SetBinsFixedPoint(&it);
    const double rb = __dsqrt_rn(B);
    it.bin_thr = __ddiv_rn(__dmul_rn(3.0, c.sigma), rb);
    it.sv_thr = __ddiv_rn(c.sigma, rb);
    SetThresholdCopies(&it);
    int l = 0;
    while ((1 << l) < 2 * bins - 1) ++l;
    it.fft_log2m = l;
    it.fft_m = 1 << l;
    if (!c.fp64_path) {
      it.eps_rel = float(c.margin * 5.9604644775390625e-08);  // margin * 2^-24
      it.eps_ms = float(c.margin * double(kEpsRms) * 5.9604644775390625e-08 *
                        0.70710678118654752);  // / sqrt(2)
    } else {
      it.eps_rel = 0.f;
      it.eps_ms = 0.f;
    }
  }
  const int32_t *d = c.draws + size_t(local) * c.draw_stride;
  const double *bq = c.draw_bq + size_t(local) * (c.draw_stride - 4) * 2;
  it.a = d[0];
  it.b = d[1];
  it.c = d[2];
  it.a_inv = d[3];
  it.trials = c.trials;
  SetPhiB(&it);
  for (int t = 0; t < c.trials; ++t) {
    it.q[t] = d[4 + t];
    it.bq_re[t] = bq[2 * t];
    it.bq_im[t] = bq[2 * t + 1];
  }
  it.win_thr = c.win_thr;
  it.force_fp64 = c.force_fp64;
  it.win_slot = -1;
  if (c.win_base != nullptr && !c.force_fp64) {
    // tables from the context's cache: built already, or built now by the
    // one signal of the batch that claims the block
    const int h = bins >> 1;
    const WinBlock wb = WinBlockOf(it.p2, bins, it.fft_m);
    unsigned char *blk = c.win_pool + c.win_base[h];
    it.wt32 = reinterpret_cast<float *>(blk);
    it.wt64 = reinterpret_cast<double *>(blk + wb.wt64);
    it.wtff = reinterpret_cast<float2 *>(blk + wb.wtff);
    it.chirp32 = reinterpret_cast<float2 *>(blk + wb.chirp32);
    it.chat32 = reinterpret_cast<float2 *>(blk + wb.chat32);
    it.r2b64 = reinterpret_cast<double2 *>(blk + wb.r2b64);
    const bool build = c.win_valid[h] == 0 && atomicCAS(&c.win_claim[h], 0, 1) == 0;
    it.tables_valid = build ? 0 : 1;
    if (build) it.win_slot = h;
  } else {
    it.tables_valid = (c.last_bins == bins && !c.force_fp64) ? 1 : 0;
  }
  if (!ahead) {
    it.flags[0] = 0;
    it.flags[1] = 0;
    it.flags[2] = 0;
  }
  it.active = 1;
}

// The while condition: some signal has work (not stopped, draws left) and
// its next iteration's bins lie in (cond_lo, cond_hi] (and, with
// exclude_fixed, exceed its min_bins). its_ahead (or null): the iteration
// planned ahead (pipelined body).
__global__ void __launch_bounds__(1024)
    k_finish(SolveCtl *__restrict__ ctl, SigIter *__restrict__ its, int nsig,
             cudaGraphConditionalHandle handle, int set_condition,
             int32_t cond_lo, int32_t cond_hi, SigIter *__restrict__ its_ahead,
             int exclude_fixed) {
  PdlEnter(its, kTraceFinish);
  int any = 0;
  for (int i = threadIdx.x; i < nsig; i += blockDim.x) {
    SolveCtl &c = ctl[i];
    SigIter &it = its[i];
    if (it.active) {
      // this iteration's spilled candidates, after all others (InsertSpills)
      if (it.flags[4] > 0) InsertSpills(it);
      const int32_t *fl = it.flags;
      c.iter += 1;
      c.near_ties += fl[2];
      if (fl[1] & kStatusUnresolved) c.unresolved += 1;
      c.fp64_iters += it.force_fp64;
      const bool f64 = c.fp64_path || it.force_fp64;
      c.gathers += BinGathers(it, f64);
      c.bin_bytes += BinBytesOf(it, f64);
      if (fl[1] & kStatusCapacity) {
        c.status = kSolveCapacity;
      } else if (fl[1] & kStatusNonFinite) {
        c.status = kSolveNonFinite;
      } else if (int64_t(fl[3]) * 2 > it.tab_cap) {
        c.status = kSolveCapacity;
      }
      if (!fl[0]) c.stale += 1;
      if (c.status == 0 && c.stale < c.max_stale && c.iter >= c.max_iter) {
        c.status = kSolveIterCap;
      }
      if (c.status != 0 || c.stale >= c.max_stale) c.done = 1;
      c.last_bins = it.force_fp64 ? -1 : it.bins;
      // the tables this signal built are complete (every table kernel of
      // the iteration has run)
      if (it.win_slot >= 0) c.win_valid[it.win_slot] = 1;
      it.active = 0;
    }
    if (its_ahead != nullptr) {
      if (c.done) its_ahead[i].active = 0;
      it.flags[0] = 0;
      it.flags[1] = 0;
      it.flags[2] = 0;
    }
    if (!c.done && c.iter - c.draw_base < c.draws_avail) {
      const int32_t nb = NextBins(c, it);
      if (nb > cond_lo && nb <= cond_hi && !(exclude_fixed && nb <= c.min_bins)) {
        any = 1;
      }
    }
  }
  any = __syncthreads_or(any);
  if (threadIdx.x == 0 && set_condition) {
    cudaGraphSetConditional(handle, any ? 1u : 0u);
  }
}

// Holds the stream for `ns` nanoseconds of the global timer (one thread;
// the wait always ends): in profiling runs, the host enqueues the timed
// binning launch and its events meanwhile, so that no host launch gap falls
// between the events.
__global__ void k_delay(unsigned long long ns) {
  unsigned long long t0, t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  do {
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  } while (t - t0 < ns);
}

// dst[0..bytes) = src[0..bytes) with src in device-mapped pinned host memory:
// 16-byte words when both are 16-byte aligned, 4-byte words when 4-byte
// aligned, else bytes; the remainder bytewise.
__global__ void __launch_bounds__(256)
    k_copy_mapped(const unsigned char *__restrict__ src, unsigned char *__restrict__ dst,
                  size_t bytes) {
  PdlEnter();
  const size_t stride = size_t(gridDim.x) * blockDim.x;
  const size_t t0 = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const uintptr_t al = reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst);
  const int w = (al & 15u) == 0 ? 16 : ((al & 3u) == 0 ? 4 : 1);
  const size_t nw = bytes / w;
  if (w == 16) {
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    for (size_t i = t0; i < nw; i += stride) d4[i] = s4[i];
  } else if (w == 4) {
    const uint32_t *s1 = reinterpret_cast<const uint32_t *>(src);
    uint32_t *d1 = reinterpret_cast<uint32_t *>(dst);
    for (size_t i = t0; i < nw; i += stride) d1[i] = s1[i];
  }
  for (size_t i = nw * w + t0; i < bytes; i += stride) dst[i] = src[i];
}

}  // namespace

void LaunchCopyMapped(const void *src_dev, void *dst, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return;
  const size_t words = bytes / 16 + 1;
  const unsigned blocks = unsigned(std::min<size_t>(152, (words + 255) / 256));
  Launch(k_copy_mapped, blocks, 256, 0, s, static_cast<const unsigned char *>(src_dev),
                                       static_cast<unsigned char *>(dst), bytes);
}

void LaunchDelay(unsigned long long ns, cudaStream_t s) {
  k_delay<<<1, 1, 0, s>>>(ns);
}

void LaunchPlan(SolveCtl *ctl, SigIter *its, int nsig, int32_t max_bins,
                cudaStream_t s, bool ahead) {
  Launch(k_plan, (nsig + 127) / 128, 128, 0, s, ctl, its, nsig, max_bins, ahead ? 1 : 0);
}

void LaunchFinish(SolveCtl *ctl, SigIter *its, int nsig,
                  cudaGraphConditionalHandle handle, bool set_condition,
                  int32_t cond_lo, int32_t cond_hi, cudaStream_t s,
                  SigIter *its_ahead, bool exclude_fixed) {
  Launch(k_finish, 1, 1024, 0, s, ctl, its, nsig, handle, set_condition ? 1 : 0,
                              cond_lo, cond_hi, its_ahead, exclude_fixed ? 1 : 0);
}

bool ControlKernelsLaunchable() {
  int a = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_finish, 1024, 0);
  return a > 0;
}

}  // namespace mpsft
