// Host engine of the C ABI declared in include/mpsft.h.
//
// Per iteration of every active signal the host computes the scalars the
// reference computes on the host side of Iterate (bins, NumBits, the window
// scalars, the thresholds of Demo1::Run) and draws the transform and the q's
// from the signal's RNG in the reference's order (src/iterate.cc:92-104);
// everything proportional to n, p, bins or the mode count runs on the GPU:
//   window tables -> Bluestein tables -> mode buckets -> gather/fold ->
//   size-B FFT -> decide (subtract, energy, pencils, coefficient) -> merge.
// One small device-to-host copy per iteration returns the found flag, the
// status bits and the mode count that drive the reference's stop rule.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <utility>
#include <vector>

#include "../../include/mpsft.h"
#include "internal.h"
#include "launch.h"

using namespace mpsft;

namespace {

// FP32 near-tie margin: the safety factor on the FP32 error model of the bins
// (kEpsRms, kEpsRowMax, kEpsValue in units of 2^-24; the rms of the bins is
// estimated as sqrt(mean|x|^2 / (2 bins))).
constexpr double kDefaultNearTieMargin = 2.0;



int Fail(mpsft_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->err = msg;
  return code;
}

#define MPSFT_CUDA(ctx, call)                                                  \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      return Fail(ctx, MPSFT_ERR_CUDA,                                         \
                  std::string(#call) + ": " + cudaGetErrorString(e_));         \
    }                                                                          \
  } while (0)

}  // namespace

// Integer and window helpers shared with the other host translation units
// (declared in internal.h).
namespace mpsft {

bool IsPow2(int64_t n) { return n > 0 && (n & (n - 1)) == 0; }

uint64_t MulModU64(uint64_t a, uint64_t b, uint64_t m) {
  return uint64_t((unsigned __int128)a * b % m);
}
uint64_t PowModU64(uint64_t b, uint64_t e, uint64_t m) {
  uint64_t r = 1 % m;
  b %= m;
  while (e) {
    if (e & 1) r = MulModU64(r, b, m);
    b = MulModU64(b, b, m);
    e >>= 1;
  }
  return r;
}
// Deterministic Miller-Rabin, exact for n < 3.2e9 with bases 2, 3, 5, 7.
bool IsPrime(int64_t n) {
  if (n < 2) return false;
  for (int64_t p : {2, 3, 5, 7, 11, 13}) {
    if (n % p == 0) return n == p;
  }
  uint64_t d = uint64_t(n) - 1;
  int r = 0;
  while ((d & 1) == 0) {
    d >>= 1;
    ++r;
  }
  for (uint64_t a : {2ull, 3ull, 5ull, 7ull}) {
    uint64_t x = PowModU64(a, d, uint64_t(n));
    if (x == 1 || x == uint64_t(n) - 1) continue;
    bool comp = true;
    for (int i = 1; i < r; ++i) {
      x = MulModU64(x, x, uint64_t(n));
      if (x == uint64_t(n) - 1) {
        comp = false;
        break;
      }
    }
    if (comp) return false;
  }
  return true;
}

// a^{-1} mod m by the extended Euclidean algorithm; 0 if not invertible.
int32_t InverseMod(int64_t a, int64_t m) {
  int64_t r0 = m, r1 = ((a % m) + m) % m, s0 = 0, s1 = 1;
  while (r1 != 0) {
    const int64_t qt = r0 / r1;
    int64_t t = r0 - qt * r1;
    r0 = r1;
    r1 = t;
    t = s0 - qt * s1;
    s0 = s1;
    s1 = t;
  }
  if (r0 != 1) return 0;
  return int32_t(((s0 % m) + m) % m);
}

int32_t NumBits(int32_t n, int32_t bins) {
  if (n < bins) return 1;
  int32_t out = 0;
  while (n >= bins) {
    n >>= 1;
    ++out;
  }
  return out;
}

// Window scalars, in the reference's operation order (src/window.cc:28-51).
WinParams MakeWindow(int32_t bins, double delta) {
  WinParams w;
  w.width = 1.0 / (2.0 * bins);
  const double sq = std::sqrt(-std::log(delta));
  w.sigma_f = 0.5 / (bins * 2.0 * M_SQRT2 * sq);
  w.sigma_t = 1.0 / ((2.0 * M_PI) * w.sigma_f);
  const double tmp = 2.0 * M_SQRT2 * w.sigma_t * sq + 1;
  int32_t f = int32_t(std::ceil(tmp / double(bins)));
  if (f % 2 == 0) ++f;
  w.folds = f;
  w.p = f * bins;
  w.p2 = (w.p - 1) / 2;
  w.erf_d = M_SQRT2 * M_PI * w.sigma_t;
  return w;
}

int FFTLog2(int32_t bins) {
  int l = 0;
  while ((1 << l) < 2 * bins - 1) ++l;
  return l;
}

bool SupportedN(int64_t n) {
  return n >= 3 && n <= INT32_MAX && (IsPow2(n) || IsPrime(n));
}

}  // namespace mpsft

namespace {

// Transform(n) (src/integer.cc:44-49): a, b, c drawn in that order; a is made
// odd for power-of-two n so that it is invertible.
Transform DrawTransform(mpsft_rng *rng, int32_t n) {
  Transform t;
  t.a = (rng->Draw() % (n - 1)) + 1;
  t.b = rng->Draw() % n;
  t.c = rng->Draw() % n;
  if (IsPow2(n)) t.a |= 1;
  t.a_inv = InverseMod(t.a, n);
  return t;
}

int CheckN(mpsft_ctx *ctx, int64_t n) {
  if (n < 3 || n > INT32_MAX) {
    return Fail(ctx, MPSFT_ERR_INVALID, "n must be in [3, 2^31 - 1]");
  }
  if (!IsPow2(n) && !IsPrime(n)) {
    return Fail(ctx, MPSFT_ERR_UNSUPPORTED_N,
                "n must be prime or a power of two (the permutation needs an "
                "invertible a)");
  }
  return MPSFT_OK;
}

// Precision policy of the FP32 path: a signal stays on the FP32 kernels
// while the FP32 rounding of its bins (eps, about 16 * 2^-24 * rms) is below
// 1% of its noise thresholds; otherwise (very high SNR) rounding would decide
// near the thresholds, and the iteration runs on the FP64 kernels. The ratio
// eps / threshold does not depend on the number of bins: it is an SNR test
// (about 90 dB with the reference's thresholds 3 sigma/sqrt(B), sigma/sqrt(B)).
constexpr double kPrecisionRatio = 0.01;
// The policy's mean |x|^2, estimated from 256 evenly spread runs of this
// many samples (the near-tie bound itself takes each row's own rms, measured
// by the row transforms, so the policy needs no exact energy)
constexpr int kPolicySample = 256;

// Precision-policy decision for one signal (FP32 calls): true when its FP32
// rounding is not small against its noise thresholds. The ratio does not
// depend on the number of bins, so it is taken once per solve.
bool PolicyForcesFP64(double margin, int32_t bins, double energy,
                      double bin_thr, double sv_thr) {
  const double m = margin > 0 ? margin : kDefaultNearTieMargin;
  // the bound's rms term for a typical row: a row's own rms is about 2/3 of
  // the signal-wide sqrt(energy / (2 bins))
  const double eps = m * kEpsRms * (2.0 / 3.0) * std::ldexp(1.0, -24) /
                     std::sqrt(2.0 * bins) * std::sqrt(energy);
  double scale = 0;
  if (bin_thr > 0) scale = bin_thr;
  if (sv_thr > 0) scale = scale > 0 ? std::min(scale, sv_thr) : sv_thr;
  return scale > 0 && eps > kPrecisionRatio * scale &&
         (1 << FFTLog2(bins)) <= kMaxFFT64;
}

// FP32 error-model scalars of an iteration with `bins` bins.
void SetNearTie(SigIter *it, bool fp64, double margin, int32_t bins,
                bool force) {
  it->force_fp64 = force ? 1 : 0;
  if (fp64) {
    it->force_fp64 = 0;
    it->eps_ms = 0;
    it->eps_rel = 0;
    return;
  }
  const double m = margin > 0 ? margin : kDefaultNearTieMargin;
  it->eps_rel = float(m * std::ldexp(1.0, -24));
  it->eps_ms = float(m * kEpsRms * std::ldexp(1.0, -24) / std::sqrt(2.0));
}

// mean |x|^2 of the signals (device values, one synchronisation)
int ReadEnergy(mpsft_ctx *ctx, const double *d_energy, int nsig,
               std::vector<double> *out) {
  out->assign(nsig, 0.0);
  MPSFT_CUDA(ctx, cudaMemcpy2DAsync(out->data(), sizeof(double), d_energy,
                                    sizeof(double) * kEnergyStride,
                                    sizeof(double), nsig,
                                    cudaMemcpyDeviceToHost, ctx->stream));
  MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MPSFT_OK;
}

// ---------------------------------------------------------------- buffers
struct Carve {
  unsigned char *base;
  size_t off = 0;
  template <typename T> T *take(size_t count) {
    off = (off + 255) & ~size_t(255);
    T *p = reinterpret_cast<T *>(base ? base + off : nullptr);
    off += count * sizeof(T);
    return p;
  }
};

// Buffer shape of one signal for a whole call.
struct Shape {
  int32_t n = 0, bins_cap = 0, rows_cap = 0, trials = 1, p2_cap = 0;
  int32_t m_cap = 0, tab_cap = 0;
  bool fp64 = false;
  bool fp32_bins = false;  // FP32 pass bins in ubuf32 (solves, iterations)
  int64_t stash_cap = 0;   // complex64 samples per stash buffer (0: none)
};

void CarveSignal(Carve &cv, const Shape &s, SigIter *it, int32_t **ctl) {
  it->wt32 = cv.take<float>(size_t(s.p2_cap) + 1);
  it->wt64 = cv.take<double>(size_t(s.p2_cap) + 1);
  it->wtff = cv.take<float2>(size_t(s.p2_cap) + 1);
  const size_t cells = size_t(s.trials) * s.rows_cap * s.bins_cap;
  // 16-byte cells: the FP32 path may redo an iteration in FP64
  it->fold = cv.take<double2>(cells);
  it->fold_alt = s.fp32_bins ? cv.take<double2>(cells) : nullptr;
  it->stash = it->stash_alt = nullptr;
  it->stash_cap = 0;
  if (s.stash_cap > 0) {
    const size_t sb = kStashHeader + sizeof(float2) * size_t(s.stash_cap);
    it->stash = cv.take<unsigned char>(sb);
    it->stash_alt = cv.take<unsigned char>(sb);
    it->stash_cap = s.stash_cap;
  }
  it->ubuf = cv.take<double2>(cells);
  it->ubuf32 = s.fp32_bins ? cv.take<float2>(cells) : nullptr;
  it->row_max = cv.take<float>(size_t(s.trials) * s.rows_cap);
  it->row_ms = cv.take<float>(size_t(s.trials) * s.rows_cap);
  it->chirp32 = cv.take<float2>(s.bins_cap);
  it->chat32 = cv.take<float2>(s.m_cap);
  it->chirp64 = cv.take<double2>(s.bins_cap);
  it->chat64 = cv.take<double2>(s.m_cap);
  it->r2b64 = s.fp32_bins ? cv.take<double2>(2 * size_t(s.bins_cap)) : nullptr;
  it->esc_part =
      cv.take<double2>(size_t(kMaxListed) * s.trials * s.rows_cap * kRebinChunks);
  it->esc_sum = cv.take<double2>(size_t(kMaxListed) * s.trials * s.rows_cap);
  it->esc_msub = cv.take<double2>(size_t(kMaxListed) * s.trials * s.rows_cap);
  it->esc_cnt = cv.take<int32_t>(size_t(kMaxListed) * s.trials * s.rows_cap);
  it->tab_key = cv.take<int32_t>(s.tab_cap);
  it->tab_coef = cv.take<double2>(s.tab_cap);
  it->tab_err = cv.take<double>(s.tab_cap);
  it->tab_cap = s.tab_cap;
  it->occ_list = cv.take<int32_t>(s.tab_cap);
  it->mode_bin = cv.take<int32_t>(s.tab_cap);
  it->mode_k1 = cv.take<int32_t>(s.tab_cap);

  it->mode_base = cv.take<double2>(size_t(s.tab_cap) * s.trials);

  it->mode_base32 = cv.take<float2>(size_t(s.tab_cap) * s.trials);

  it->mode_errw = cv.take<float>(s.tab_cap);
  it->ph_k = PhaseTableK(s.n);
  it->ph_lo = cv.take<double2>(size_t(1) << it->ph_k);
  it->ph_hi = cv.take<double2>(size_t(PhaseTableHi(s.n)));
  it->ph_build = 1;
  it->bkt_count = cv.take<int32_t>(s.bins_cap);
  it->bkt_start = cv.take<int32_t>(s.bins_cap);
  it->bkt_list = cv.take<int32_t>(s.tab_cap);
  it->cand_valid = cv.take<int32_t>(s.bins_cap);
  it->cand_k0 = cv.take<int32_t>(s.bins_cap);
  it->cand_coef = cv.take<double2>(s.bins_cap);
  it->cand_err = cv.take<double>(s.bins_cap);
  // the listed bins' phase-step powers (s^k, k < 64, and s^64), evaluated
  // once per bin by the FP32 decide that lists it
  it->esc_pow = s.fp32_bins ? cv.take<float4>(size_t(kMaxListed) * 64) : nullptr;
  it->esc_step = s.fp32_bins ? cv.take<double2>(kMaxListed) : nullptr;
  it->esc_list = cv.take<int32_t>(kMaxListed);
  it->esc_mask = cv.take<uint32_t>(kMaxListed);
  it->esc_cap = kMaxListed;
  it->spill_beta = cv.take<int32_t>(kSpillCap);
  it->spill_k0 = cv.take<int32_t>(kSpillCap);
  it->spill_coef = cv.take<double2>(kSpillCap);
  it->spill_err = cv.take<double>(kSpillCap);
  *ctl = cv.take<int32_t>(kCtlWords);
  it->flags = *ctl;
  it->tab_count = *ctl + 3;
  it->bins_cap = s.bins_cap;
}

int EnsureArena(mpsft_ctx *ctx, size_t bytes) {
  if (ctx->arena_size >= bytes) return MPSFT_OK;
  if (ctx->arena) {
    cudaStreamSynchronize(ctx->stream);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->graph) cudaGraphDestroy(ctx->graph);
    ctx->graph_exec = nullptr;
    ctx->graph = nullptr;
    ctx->graph_key.clear();
    cudaFree(ctx->arena);
    ctx->arena = nullptr;
    ctx->arena_size = 0;
  }
  const size_t want = bytes + (bytes >> 3);
  if (cudaMalloc(&ctx->arena, want) != cudaSuccess) {
    cudaGetLastError();
    return Fail(ctx, MPSFT_ERR_NOMEM, "device allocation of the work arena failed");
  }
  ctx->arena_size = want;
  return MPSFT_OK;
}

int EnsureHostCtl(mpsft_ctx *ctx, size_t words) {
  if (ctx->h_ctl_n >= words) return MPSFT_OK;
  if (ctx->h_ctl) cudaFreeHost(ctx->h_ctl);
  ctx->h_ctl = nullptr;
  MPSFT_CUDA(ctx, cudaMallocHost(&ctx->h_ctl, words * sizeof(int32_t)));
  ctx->h_ctl_n = words;
  return MPSFT_OK;
}

// Pinned host staging for a call's results (the solve state and the
// tables' entries, copied from the device after the graph with one wait).
int EnsureHostStage(mpsft_ctx *ctx, size_t bytes) {
  if (ctx->h_stage_n >= bytes) return MPSFT_OK;
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  ctx->h_stage = nullptr;
  ctx->h_stage_n = 0;
  MPSFT_CUDA(ctx, cudaMallocHost(&ctx->h_stage, bytes));
  ctx->h_stage_n = bytes;
  return MPSFT_OK;
}

// A solve call's results, the same layout on the device (arena) and in the
// host staging: the solve state, the tables' entry counts and sorted flags,
// then the packed keys and coefficients (room for max_cap per signal).
struct ResultStage {
  size_t ctl = 0, counts = 0, sorted = 0, keys = 0, coefs = 0, bytes = 0;
  int nsig = 0, max_cap = 0;
  unsigned char *dev = nullptr;
  mutable size_t est = 0;  // entries copied with the header (LaunchResults)
  ResultStage(int n, int cap) : nsig(n), max_cap(cap) {
    auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
    counts = up(ctl + sizeof(SolveCtl) * size_t(nsig));
    sorted = up(counts + sizeof(int32_t) * size_t(nsig));
    keys = up(sorted + sizeof(int32_t) * size_t(nsig));
    coefs = up(keys + sizeof(int32_t) * size_t(cap) * nsig);
    bytes = up(coefs + sizeof(double2) * size_t(cap) * nsig);
  }
  size_t entries() const { return size_t(max_cap) * nsig; }
  template <typename T> T *at(unsigned char *base, size_t off) const {
    return reinterpret_cast<T *>(base + off);
  }
};

// The solve state and every table's entries (k_export_tables) into the
// device staging, then their copies to the host: the header and the first
// `est` entries (the last call's count and a quarter more), so that one wait
// usually covers the results (FinishResults copies any rest).
int LaunchResults(mpsft_ctx *ctx, const SigIter *d_its, const ResultStage &rs) {
  size_t *est = &rs.est;
  unsigned char *d = rs.dev;
  LaunchCopyMapped(ctx->d_solve_ctl, rs.at<SolveCtl>(d, rs.ctl),
                   sizeof(SolveCtl) * rs.nsig, ctx->stream);
  LaunchExportTables(d_its, rs.nsig, rs.max_cap, rs.at<int32_t>(d, rs.keys),
                     rs.at<double2>(d, rs.coefs), rs.at<int32_t>(d, rs.counts),
                     rs.at<int32_t>(d, rs.sorted), ctx->stream);
  *est = std::min(rs.entries(), std::max<size_t>(ctx->res_est, 256 * size_t(rs.nsig)));
  MPSFT_CUDA(ctx, cudaMemcpyAsync(ctx->h_stage, d, rs.keys, cudaMemcpyDeviceToHost,
                                  ctx->stream));
  MPSFT_CUDA(ctx, cudaMemcpyAsync(ctx->h_stage + rs.keys, d + rs.keys,
                                  sizeof(int32_t) * *est, cudaMemcpyDeviceToHost,
                                  ctx->stream));
  MPSFT_CUDA(ctx, cudaMemcpyAsync(ctx->h_stage + rs.coefs, d + rs.coefs,
                                  sizeof(double2) * *est, cudaMemcpyDeviceToHost,
                                  ctx->stream));
  return MPSFT_OK;
}

// After the wait: the entries past the first `est` when the tables grew past
// the estimate (one more wait), and the next call's estimate.
int FinishResults(mpsft_ctx *ctx, const ResultStage &rs) {
  const size_t est = rs.est;
  const int32_t *counts = rs.at<int32_t>(ctx->h_stage, rs.counts);
  size_t total = 0;
  for (int i = 0; i < rs.nsig; ++i) total += size_t(counts[i]);
  total = std::min(total, rs.entries());
  if (total > est) {
    unsigned char *d = rs.dev;
    MPSFT_CUDA(ctx, cudaMemcpyAsync(ctx->h_stage + rs.keys + sizeof(int32_t) * est,
                                    d + rs.keys + sizeof(int32_t) * est,
                                    sizeof(int32_t) * (total - est),
                                    cudaMemcpyDeviceToHost, ctx->stream));
    MPSFT_CUDA(ctx, cudaMemcpyAsync(ctx->h_stage + rs.coefs + sizeof(double2) * est,
                                    d + rs.coefs + sizeof(double2) * est,
                                    sizeof(double2) * (total - est),
                                    cudaMemcpyDeviceToHost, ctx->stream));
    MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  ctx->res_est = total + total / 4 + 256;
  return MPSFT_OK;
}

// A solve's small host -> device transfers (iteration descriptors, draw
// tables, solve state) go through pinned, device-mapped staging and a copy
// kernel rather than the copy engines: a caller streaming the next batch's
// signals in on another stream keeps the engines busy with gigabytes, and a
// DMA copy queued behind those would hold the solve's start back. The
// staging is a bump allocator, reset at the start of a call and after each
// stream synchronisation that retires the uploads before it.
int EnsureUploadStage(mpsft_ctx *ctx, size_t bytes) {
  if (ctx->h_up_n >= bytes) return MPSFT_OK;
  if (ctx->h_up) {
    MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFreeHost(ctx->h_up);
  }
  ctx->h_up = nullptr;
  ctx->d_up = nullptr;
  ctx->h_up_n = 0;
  ctx->up_off = 0;
  const size_t want = bytes + (bytes >> 2) + 4096;
  MPSFT_CUDA(ctx, cudaHostAlloc(&ctx->h_up, want, cudaHostAllocMapped));
  void *dp = nullptr;
  MPSFT_CUDA(ctx, cudaHostGetDevicePointer(&dp, ctx->h_up, 0));
  ctx->d_up = static_cast<unsigned char *>(dp);
  ctx->h_up_n = want;
  return MPSFT_OK;
}

int Upload(mpsft_ctx *ctx, void *dst, const void *src, size_t bytes,
           cudaStream_t s) {
  if (bytes == 0) return MPSFT_OK;
  const size_t off = (ctx->up_off + 255) & ~size_t(255);
  if (off + bytes > ctx->h_up_n) {
    // (only when the caller did not reserve enough: retire the pending
    // uploads and start over in a larger stage)
    MPSFT_CUDA(ctx, cudaStreamSynchronize(s));
    ctx->up_off = 0;
    int rc = EnsureUploadStage(ctx, bytes);
    if (rc) return rc;
    return Upload(ctx, dst, src, bytes, s);
  }
  std::memcpy(ctx->h_up + off, src, bytes);
  ctx->up_off = off + bytes;
  LaunchCopyMapped(ctx->d_up + off, dst, bytes, s);
  ++ctx->up_launches;
  MPSFT_CUDA(ctx, cudaGetLastError());
  return MPSFT_OK;
}

// Table cache for odd bins in [bmin, bmax] and window delta (see mpsft_ctx);
// *out gets the device pointers, or nulls when the cache would exceed its
// budget (the solve then builds per-signal tables).
constexpr size_t kWinCacheBudget = size_t(1) << 30;
struct WinCacheRefs {
  const int64_t *base = nullptr;
  unsigned char *pool = nullptr;
  int32_t *valid = nullptr, *claim = nullptr;
};

int EnsureWinCache(mpsft_ctx *ctx, double delta, int32_t bmin, int32_t bmax,
                   WinCacheRefs *out) {
  *out = WinCacheRefs{};
  const bool fits = ctx->win_dev && ctx->win_delta == delta &&
                    bmin >= ctx->win_bmin && bmax <= ctx->win_bmax;
  if (!fits) {
    if (ctx->win_dev && ctx->win_delta == delta) {
      bmin = std::min(bmin, ctx->win_bmin);
      bmax = std::max(bmax, ctx->win_bmax);
    }
    const int32_t h_n = (bmax >> 1) + 1;
    std::vector<int64_t> base(h_n, 0);
    int64_t pool = 0;
    for (int32_t b = bmin | 1; b <= bmax; b += 2) {
      const WinParams w = MakeWindow(b, delta);
      base[b >> 1] = pool;
      pool += WinBlockOf(w.p2, b, 1 << FFTLog2(b)).bytes;
    }
    if (size_t(pool) > kWinCacheBudget) return MPSFT_OK;
    const size_t head = size_t(Align16(8 * int64_t(h_n)) + 2 * Align16(4 * int64_t(h_n)));
    const size_t bytes = head + size_t(pool);
    if (ctx->win_dev) {
      MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      cudaFree(ctx->win_dev);
      ctx->win_dev = nullptr;
      ctx->win_bytes = 0;
    }
    if (cudaMalloc(&ctx->win_dev, bytes) != cudaSuccess) {
      cudaGetLastError();
      ctx->win_dev = nullptr;
      return MPSFT_OK;  // no cache: per-signal tables
    }
    ctx->win_bytes = bytes;
    ctx->win_delta = delta;
    ctx->win_bmin = bmin;
    ctx->win_bmax = bmax;
    MPSFT_CUDA(ctx, cudaMemcpyAsync(ctx->win_dev, base.data(), sizeof(int64_t) * h_n,
                                    cudaMemcpyHostToDevice, ctx->stream));
    MPSFT_CUDA(ctx, cudaMemsetAsync(ctx->win_dev + Align16(8 * int64_t(h_n)), 0,
                                    2 * Align16(4 * int64_t(h_n)), ctx->stream));
    // pageable source: complete before the vector goes away
    MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  const int32_t h_n = (ctx->win_bmax >> 1) + 1;
  unsigned char *d = ctx->win_dev;
  out->base = reinterpret_cast<const int64_t *>(d);
  out->valid = reinterpret_cast<int32_t *>(d + Align16(8 * int64_t(h_n)));
  out->claim = reinterpret_cast<int32_t *>(d + Align16(8 * int64_t(h_n)) +
                                           Align16(4 * int64_t(h_n)));
  out->pool = d + Align16(8 * int64_t(h_n)) + 2 * Align16(4 * int64_t(h_n));
  // one builder per block and solve: claims start over
  MPSFT_CUDA(ctx, cudaMemsetAsync(out->claim, 0, sizeof(int32_t) * h_n, ctx->stream));
  return MPSFT_OK;
}

int32_t NextPow2(int64_t v) {
  int32_t p = 1;
  while (p < v) p <<= 1;
  return p;
}

}  // namespace

namespace mpsft {

// Fills the per-iteration scalars of it for (bins, bits, transform, q's).
// bq = e^{2 pi i (b q mod n)/n}, as Sinusoid(MulMod(b, q, n) / n); always
// computed here on the host so that every loop uses the same values.
void RowPhase(int32_t b, int32_t q, int32_t n, double *re, double *im) {
  const int64_t m = (int64_t(b) * q) % n;
  const double f = double(m) / double(n) * (2.0 * M_PI);
  *re = std::cos(f);
  *im = std::sin(f);
}

void FillIter(SigIter *it, const mpsft_signal *sig, int32_t bins, int32_t bits,
              double delta, const Transform &tf, const int32_t *q,
              int32_t trials) {
  FillIter(it, sig, bins, bits, MakeWindow(bins, delta), tf, q, trials);
}

void FillIter(SigIter *it, const mpsft_signal *sig, int32_t bins, int32_t bits,
              const WinParams &w, const Transform &tf, const int32_t *q,
              int32_t trials) {
  it->x = sig->d_x;
  it->n = int32_t(sig->n);
  it->bins = bins;
  it->bits = bits;
  it->rows = 1 + 2 * bits;
  it->p = w.p;
  it->p2 = w.p2;
  it->folds = w.folds;
  it->a = tf.a;
  it->b = tf.b;
  it->c = tf.c;
  it->a_inv = tf.a_inv;
  it->phase_shift = -1;
  if (IsPow2(sig->n)) {
    int k = 0;
    while ((int64_t(1) << k) < sig->n) ++k;
    it->phase_shift = 32 - k;
  }
  it->trials = trials;
  it->active = 1;
  for (int t = 0; t < trials; ++t) {
    it->q[t] = q[t];
    RowPhase(tf.b, q[t], it->n, &it->bq_re[t], &it->bq_im[t]);
  }
  it->width = w.width;
  it->sigma_f = w.sigma_f;
  it->erf_d = w.erf_d;
  SetFixedPoint(it);
  it->fft_log2m = FFTLog2(bins);
  it->fft_m = 1 << it->fft_log2m;
}

}  // namespace mpsft

namespace {

int CheckWindow(mpsft_ctx *ctx, int32_t bins, double delta, bool fp64) {
  if (bins <= 0 || bins % 2 == 0) {
    return Fail(ctx, MPSFT_ERR_INVALID, "bins must be odd and positive");
  }
  if (!(delta > 0 && delta < 1)) {
    return Fail(ctx, MPSFT_ERR_INVALID, "window_delta must be in (0, 1)");
  }
  const WinParams w = MakeWindow(bins, delta);
  if (w.folds > kFoldLanes * kMaxFoldsPerLane) {
    return Fail(ctx, MPSFT_ERR_INVALID, "window_delta too small (p/bins > 80)");
  }
  const int m = 1 << FFTLog2(bins);
  if (m > (fp64 ? kMaxFFT64 : kMaxFFT)) {
    return Fail(ctx, MPSFT_ERR_INVALID,
                fp64 ? "bins too large for the FP64 path (max 4096)"
                     : "bins too large (max 8192)");
  }
  return MPSFT_OK;
}

// Records the binning launch between an event pair when profiling.
struct BinTimer {
  mpsft_ctx *ctx;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> used;
  // per timed launch: 0 = the iteration's binning, 1 = its FP64 redo (the
  // signals an FP32 call runs on the FP64 kernels)
  std::vector<int> tags;
  size_t next = 0;
  int Begin(int tag = 0) {
    if (!ctx->profiling) return MPSFT_OK;
    tags.push_back(tag);
    while (ctx->events.size() < 2 * (next + 1)) {
      cudaEvent_t e;
      MPSFT_CUDA(ctx, cudaEventCreate(&e));
      ctx->events.push_back(e);
    }
    MPSFT_CUDA(ctx, cudaEventRecord(ctx->events[2 * next], ctx->stream));
    return MPSFT_OK;
  }
  int End() {
    if (!ctx->profiling) return MPSFT_OK;
    MPSFT_CUDA(ctx, cudaEventRecord(ctx->events[2 * next + 1], ctx->stream));
    used.emplace_back(ctx->events[2 * next], ctx->events[2 * next + 1]);
    ++next;
    return MPSFT_OK;
  }
  double TotalMs() {
    double tot = 0;
    for (auto &p : used) {
      float ms = 0;
      cudaEventElapsedTime(&ms, p.first, p.second);
      tot += ms;
    }
    return tot;
  }
};

int64_t BinBytes(const SigIter &it, bool fp64) { return BinBytesOf(it, fp64); }

// Launch sequence of one iteration for nsig signals whose SigIter array is
// already on the device.

// Launch maxima of one iteration (grid sizes and shared memory).
struct Maxima {
  int bins = 0, bits = 0, trials = 0, p2 = 0, m = 0, rows = 0, cap = 0;
  int64_t n = 0;
  // bins of the launch-shape lookup (FoldShapeFor): the bins the solve
  // graph's phase sizes its launches for; 0 = bins
  int tune_bins = 0;
};

int CeilLog2(int64_t v) {
  int l = 0;
  while ((int64_t(1) << l) < v) ++l;
  return l;
}

// The bins a solve graph sizes an iteration's launches for (its phase's
// largest bins: the batch's largest, or small_bins once every signal needs at
// most that many, GraphLoop), so that a host-driven loop and the autotuner
// look up the launch shape the graph uses.
int32_t PhaseBins(int32_t bins, int32_t bins_cap, int32_t min_bins_max) {
  const int32_t small_bins = (4 * min_bins_max) | 1;
  return (bins_cap > small_bins && bins <= small_bins) ? small_bins : bins_cap;
}

// The FP32 fold's launch shape for a launch of nsig signals (largest bins
// and length given): the forced shape, else the autotuner's entry for the
// launch's classes, else the default shape 0.
int FoldShapeFor(const mpsft_ctx *ctx, int max_bins, int64_t max_n, int nsig,
                 bool c128) {
  if (ctx->force_shape >= 0) return ctx->force_shape;
  const int kb = CeilLog2(max_bins), kn = CeilLog2(max_n), ks = CeilLog2(nsig);
  for (const auto &e : ctx->tuning) {
    if (e.bins_log2 == kb && e.n_log2 == kn && e.nsig_log2 == ks &&
        e.c128 == (c128 ? 1 : 0)) {
      return e.shape;
    }
  }
  return 0;
}

Maxima MaximaOf(const std::vector<SigIter> &h_its) {
  Maxima mx;
  for (const SigIter &it : h_its) {
    if (!it.active) continue;
    mx.bins = std::max(mx.bins, it.bins);
    mx.bits = std::max(mx.bits, it.bits);
    mx.trials = std::max(mx.trials, it.trials);
    mx.p2 = std::max(mx.p2, it.p2);
    mx.m = std::max(mx.m, it.fft_m);
    mx.rows = std::max(mx.rows, it.rows);
    mx.cap = std::max(mx.cap, it.tab_cap);
    mx.n = std::max<int64_t>(mx.n, it.n);
  }
  return mx;
}

// The kernels of one iteration of every active signal, on stream s (and the
// context's side stream, forked from and joined back into s). any_forced:
// some signal of an FP32 call takes the FP64 kernels (precision policy).
// The fixed-bins phase's pipelined body: while this iteration decides, the
// next one (descriptors its_ahead) is planned and gathered/folded on the
// prefold stream, into the second fold buffer (only this iteration's row FFT
// reads the first).
struct Ahead {
  SigIter *its_ahead;
  SolveCtl *ctl;
  int32_t plan_max;
};

int LaunchIterationKernels(mpsft_ctx *ctx, const SigIter *d_its, int nsig,
                           const Maxima &mx, bool x_c128, bool fp64,
                           bool any_forced, BinTimer *timer, int64_t *launched,
                           cudaStream_t s, const Ahead *ahead = nullptr) {
  if (mx.bins == 0) return MPSFT_OK;
  // fork: tables, mode preparation and bucketing on the side stream while
  // the window and the gather/fold run on the main one; the row FFT waits
  // for the Bluestein tables only, the decisions for the rest (ahead: the
  // tables are the phase prologue's, and this iteration's fold ran in the
  // previous body)
  MPSFT_CUDA(ctx, cudaEventRecord(ctx->ev_fork, s));
  MPSFT_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
  if (ahead) {
    // the next iteration's plan (at fixed bins it reads nothing this
    // iteration writes; the stop rule waits for it) and its gather/fold, into
    // the other fold buffer (k_plan swapped them), from the start of the body
    // on the prefold stream, beside all of this iteration. Its window and
    // Bluestein tables are those of the phase's prologue: every iteration of
    // the phase has min_bins bins.
    MPSFT_CUDA(ctx, cudaStreamWaitEvent(ctx->pre, ctx->ev_fork, 0));
    LaunchPlan(ahead->ctl, ahead->its_ahead, nsig, ahead->plan_max, ctx->pre, true);
    MPSFT_CUDA(ctx, cudaEventRecord(ctx->ev_plan_p, ctx->pre));
    LaunchBinFold(ahead->its_ahead, nsig, mx.bins, mx.bits, mx.trials, x_c128, false,
                  ctx->pre, false,
                  FoldShapeFor(ctx, mx.tune_bins > 0 ? mx.tune_bins : mx.bins, mx.n,
                               nsig, x_c128));
    MPSFT_CUDA(ctx, cudaEventRecord(ctx->ev_join_p, ctx->pre));
  }
  if (!ahead) {
    LaunchBluesteinSetup(d_its, nsig, mx.m, fp64, ctx->tw32, ctx->tw64, ctx->side);
    MPSFT_CUDA(ctx, cudaEventRecord(ctx->ev_blue, ctx->side));
  }
  // mode preparation and bucketing in one kernel
  LaunchBucket(d_its, nsig, mx.bins, mx.cap, ctx->side, true);
  MPSFT_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->side));
  // FP32 path: the FP64 window tables (for the near-tie re-binning and the
  // FP64 kernels) are built on the low-priority stream and joined only
  // before the re-binning; the binning uses an FP32 evaluation
  if (!fp64) {
    MPSFT_CUDA(ctx, cudaStreamWaitEvent(ctx->side64, ctx->ev_fork, 0));
    LaunchWindow64(d_its, nsig, mx.p2, ctx->side64);
    MPSFT_CUDA(ctx, cudaEventRecord(ctx->ev_join64, ctx->side64));
  }
  if (fp64) {
    LaunchWindow(d_its, nsig, mx.p2, s);
  } else if (!ahead) {
    LaunchWindow32(d_its, nsig, mx.p2, s);
  }
  if (timer && ctx->profiling) {
    // profiling: the binning alone on the GPU (the side streams' kernels
    // first), and its launch enqueued while a short delay kernel holds the
    // stream, so that its events time the kernel, not a host launch gap
    MPSFT_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_join, 0));
    if (!fp64) MPSFT_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_join64, 0));
    LaunchDelay(20000, s);
  }
  if (timer) {
    int rc = timer->Begin();
    if (rc) return rc;
  }
  const int shape = FoldShapeFor(ctx, mx.tune_bins > 0 ? mx.tune_bins : mx.bins,
                                 mx.n, nsig, x_c128);
  if (!ahead) {
    LaunchBinFold(d_its, nsig, mx.bins, mx.bits, mx.trials, x_c128, fp64, s, false,
                  shape);
  }
  if (timer) {
    int rc = timer->End();
    if (rc) return rc;
  }
  if (!ahead) MPSFT_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_blue, 0));
  LaunchRowFFT(d_its, nsig, mx.rows, mx.trials, mx.m, fp64, ctx->tw32, ctx->tw64,
               s);
  MPSFT_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_join, 0));  // join
  // near ties of the FP32 pass: listed bins re-binned and re-decided in
  // FP64; signals that the precision policy sends to FP64 (and signals whose
  // near-tie list overflowed) run the FP64 kernels (redo). Without redo the
  // other bins' merge runs beside the re-binning: the FP32 decide holds the
  // listed bins back and their FP64 decision merges them.
  const bool redo = !fp64 && any_forced && mx.m <= kMaxFFT64;
  const bool side_merge = !fp64 && !redo;
  LaunchDecide(d_its, nsig, mx.bins, mx.trials, !fp64, false, s, false, side_merge);
  // Bluestein setup, mode preparation with bucketing, window(s), fold, FFT,
  // decide (ahead: the next iteration's plan and fold, bucketing, FP64
  // window, FFT, decide)
  if (launched) *launched += ahead ? 6 : (fp64 ? 6 : 7);
  if (!fp64) {
    // side stream: the listed bins' FP64 mode terms (before any merge
    // changes a coefficient), then the merge of the other bins, beside the
    // re-binning
    MPSFT_CUDA(ctx, cudaEventRecord(ctx->ev_fork_l, s));
    MPSFT_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_fork_l, 0));
    LaunchListedTerms(d_its, nsig, mx.trials, ctx->side);
    MPSFT_CUDA(ctx, cudaEventRecord(ctx->ev_join_l, ctx->side));
    if (side_merge) {
      LaunchMerge(d_its, nsig, mx.bins, ctx->side);
      MPSFT_CUDA(ctx, cudaEventRecord(ctx->ev_join_m, ctx->side));
    }
    MPSFT_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_join64, 0));
    LaunchRebin(d_its, nsig, kMaxListed, x_c128, false, s);
    MPSFT_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_join_l, 0));
    LaunchDecideListed(d_its, nsig, mx.trials, redo, side_merge, s);
    if (launched) *launched += 3;  // mode terms, re-binning, FP64 decisions
    if (redo) {
      LaunchModePrep(d_its, nsig, mx.cap, s, true);
      LaunchBluesteinSetup(d_its, nsig, mx.m, true, ctx->tw32, ctx->tw64, s, true);
      if (timer && ctx->profiling) LaunchDelay(20000, s);
      if (timer) {
        int rc = timer->Begin(1);
        if (rc) return rc;
      }
      LaunchBinFold(d_its, nsig, mx.bins, mx.bits, mx.trials, x_c128, true, s,
                    true);
      if (timer) {
        int rc = timer->End();
        if (rc) return rc;
      }
      LaunchRowFFT(d_its, nsig, mx.rows, mx.trials, mx.m, true, ctx->tw32,
                   ctx->tw64, s, true);
      LaunchDecide(d_its, nsig, mx.bins, mx.trials, false, false, s, true);
      if (launched) *launched += 5;
    }
  }
  if (side_merge) {
    MPSFT_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_join_m, 0));
  } else {
    LaunchMerge(d_its, nsig, mx.bins, s);
  }
  if (launched) *launched += 1;
  MPSFT_CUDA(ctx, cudaGetLastError());
  return MPSFT_OK;
}

int LaunchIteration(mpsft_ctx *ctx, const SigIter *d_its, int nsig,
                    const std::vector<SigIter> &h_its, bool x_c128, bool fp64,
                    BinTimer *timer, int64_t *launched = nullptr,
                    int32_t tune_bins = 0) {
  bool any_forced = false;
  for (const SigIter &it : h_its) any_forced |= it.active && it.force_fp64;
  Maxima mx = MaximaOf(h_its);
  mx.tune_bins = tune_bins;
  const int rc = LaunchIterationKernels(ctx, d_its, nsig, mx, x_c128, fp64, any_forced,
                                        timer, launched, ctx->stream);
  if (rc != MPSFT_OK) return rc;
  // (in the solve graph, k_finish inserts the spilled candidates)
  LaunchInsertSpills(d_its, nsig, ctx->stream);
  if (launched) *launched += 1;
  MPSFT_CUDA(ctx, cudaGetLastError());
  return MPSFT_OK;
}

struct ModeOut {
  std::vector<std::pair<int32_t, double2>> modes;
};

int DownloadTable(mpsft_ctx *ctx, const SigIter &it,
                  std::vector<std::pair<int32_t, double2>> *out) {
  std::vector<int32_t> keys(it.tab_cap);
  std::vector<double2> coefs(it.tab_cap);
  MPSFT_CUDA(ctx, cudaMemcpyAsync(keys.data(), it.tab_key,
                                  sizeof(int32_t) * it.tab_cap,
                                  cudaMemcpyDeviceToHost, ctx->stream));
  MPSFT_CUDA(ctx, cudaMemcpyAsync(coefs.data(), it.tab_coef,
                                  sizeof(double2) * it.tab_cap,
                                  cudaMemcpyDeviceToHost, ctx->stream));
  MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  out->clear();
  for (int i = 0; i < it.tab_cap; ++i) {
    if (keys[i] != kEmptyKey) out->emplace_back(keys[i], coefs[i]);
  }
  std::sort(out->begin(), out->end(),
            [](const std::pair<int32_t, double2> &l,
               const std::pair<int32_t, double2> &r) { return l.first < r.first; });
  return MPSFT_OK;
}

int ClearTable(mpsft_ctx *ctx, const SigIter &it, int32_t *ctl) {
  MPSFT_CUDA(ctx, cudaMemsetAsync(it.tab_key, 0xFF,
                                  sizeof(int32_t) * it.tab_cap, ctx->stream));
  MPSFT_CUDA(ctx, cudaMemsetAsync(it.tab_coef, 0, sizeof(double2) * it.tab_cap,
                                  ctx->stream));
  MPSFT_CUDA(ctx, cudaMemsetAsync(it.tab_err, 0, sizeof(double) * it.tab_cap,
                                  ctx->stream));
  MPSFT_CUDA(ctx, cudaMemsetAsync(ctl, 0, sizeof(int32_t) * kCtlWords,
                                  ctx->stream));
  return MPSFT_OK;
}

int CheckSignal(mpsft_ctx *ctx, const mpsft_signal *sig) {
  if (!sig || !sig->d_x) return Fail(ctx, MPSFT_ERR_INVALID, "null signal");
  if (sig->ctx != ctx) {
    return Fail(ctx, MPSFT_ERR_INVALID, "signal belongs to another context");
  }
  return CheckN(ctx, sig->n);
}

constexpr int kDrawChunk = 32;  // iterations of draws uploaded at a time
constexpr int kTimelineCapacity = 1 << 14;  // kernel entries of a timeline
constexpr int kGraphUnavailable = -100;
static_assert(int(kSolveCapacity) == int(MPSFT_ERR_CAPACITY) &&
                  int(kSolveIterCap) == int(MPSFT_ERR_ITER_CAP) &&
                  int(kSolveNonFinite) == int(MPSFT_ERR_NONFINITE),
              "device stop codes are the ABI's status codes");

// Fills draws for iterations [base, base + kDrawChunk) of one signal from its
// RNG, in the reference's order: a, b, c (Transform), then one q per trial;
// bq gets each trial's row phase (re, im) at [(j * (stride - 4) + t) * 2].
void FillDraws(mpsft_rng *rng, int32_t n, int32_t trials, int stride,
               int32_t *out, double *bq) {
  for (int j = 0; j < kDrawChunk; ++j) {
    const Transform tf = DrawTransform(rng, n);
    int32_t *d = out + size_t(j) * stride;
    double *p = bq + size_t(j) * (stride - 4) * 2;
    d[0] = tf.a;
    d[1] = tf.b;
    d[2] = tf.c;
    d[3] = tf.a_inv;
    for (int t = 0; t < trials; ++t) {
      d[4 + t] = rng->Draw() % n;
      RowPhase(tf.b, d[4 + t], n, &p[2 * t], &p[2 * t + 1]);
    }
  }
}

// Host side of the solve graph's draw tables: the first kDrawChunk
// iterations' draws of every signal, its initial device state (SolveCtl) and
// the RNG states to rewind to. Filled while the GPU computes the signal
// energies (nothing here depends on them; force_fp64 is set afterwards).
struct DrawTables {
  int tmax = 1, stride = 5;
  size_t bq_per = 0;
  std::vector<SolveCtl> hc;
  std::vector<int32_t> hd;
  std::vector<double> hb;
  // working copies of the callers' generators: the draws come from these,
  // and the callers' own generators take the used draws afterwards
  // (mpsft_rng::pending), so that an error leaves them untouched
  std::vector<mpsft_rng> work;
};

void PrepareDraws(mpsft_ctx *ctx, const mpsft_signal *const *sigs,
                  const mpsft_solve_options *opts, int nsig,
                  mpsft_rng *const *rngs, bool fp64, DrawTables *dt) {
  dt->tmax = 1;
  for (int i = 0; i < nsig; ++i) dt->tmax = std::max(dt->tmax, opts[i].trials);
  const int stride = dt->stride = 4 + dt->tmax;
  dt->bq_per = size_t(kDrawChunk) * dt->tmax * 2;
  dt->hc.assign(nsig, SolveCtl{});
  dt->hd.assign(size_t(nsig) * kDrawChunk * stride, 0);
  dt->hb.assign(nsig * dt->bq_per, 0.0);
  dt->work.resize(nsig);
  auto fill = [&](int i) {
    const mpsft_solve_options &o = opts[i];
    SolveCtl &c = dt->hc[i];
    std::memset(&c, 0, sizeof(c));
    c.k = o.k;
    c.min_bins = o.min_bins;
    c.trials = o.trials;
    c.draw_stride = stride;
    c.max_stale = o.max_stale_iter;
    c.max_iter = o.max_iter > 0 ? o.max_iter : 64 + 8 * o.k;
    c.fp64_path = fp64 ? 1 : 0;
    c.sigma = o.sigma;
    c.sqrt_c_delta = std::sqrt(-std::log(o.window_delta));
    c.win_thr = o.window_threshold;
    c.margin = o.near_tie_margin > 0 ? o.near_tie_margin : kDefaultNearTieMargin;
    c.draws = ctx->d_draws + size_t(i) * kDrawChunk * stride;
    c.draw_bq = ctx->d_draw_bq + i * dt->bq_per;
    c.draw_base = 0;
    c.draws_avail = kDrawChunk;
    c.last_bins = -1;
    dt->work[i] = *rngs[i];
    FillDraws(&dt->work[i], int32_t(sigs[i]->n), o.trials, stride,
              dt->hd.data() + size_t(i) * kDrawChunk * stride,
              dt->hb.data() + i * dt->bq_per);
  };
  // each signal's draws come from its own generator: the signals are filled
  // side by side, in chunks, by the context's host threads and this one
  constexpr int kPoolMin = 16, kPoolWorkers = 3, kChunk = 8;
  if (nsig < kPoolMin) {
    for (int i = 0; i < nsig; ++i) fill(i);
    return;
  }
  if (!ctx->pool) ctx->pool = std::make_unique<HostPool>(kPoolWorkers);
  const int chunks = (nsig + kChunk - 1) / kChunk;
  ctx->pool->Run(chunks, [&](int ch) {
    for (int i = ch * kChunk; i < std::min(nsig, (ch + 1) * kChunk); ++i) fill(i);
  });
}

// The solve as a CUDA graph: a while node whose body is one iteration of
// every signal (k_plan, the iteration kernels, k_finish). The host only
// refills draw tables; the loop ends when every signal has stopped. The RNGs
// are left exactly where the reference's loop would leave them.
int GraphLoop(mpsft_ctx *ctx, const mpsft_signal *const *sigs,
              const mpsft_solve_options *opts, int nsig,
              mpsft_rng *const *rngs, const std::vector<Shape> &shapes,
              SigIter *d_its, SigIter *d_its_ahead, std::vector<SigIter> *its,
              DrawTables *dt,
              const std::vector<int32_t> &force, bool any_forced, bool fp64,
              bool x_c128, int64_t *launches, const ResultStage &rs,
              std::vector<SolveCtl> *ctl_out) {
  const int tmax = dt->tmax;
  Maxima mx;
  for (int i = 0; i < nsig; ++i) {
    const Shape &s = shapes[i];
    mx.bins = std::max(mx.bins, s.bins_cap);
    mx.bits = std::max(mx.bits, (s.rows_cap - 1) / 2);
    mx.rows = std::max(mx.rows, s.rows_cap);
    mx.p2 = std::max(mx.p2, s.p2_cap);
    mx.m = std::max(mx.m, s.m_cap);
    mx.cap = std::max(mx.cap, s.tab_cap);
    mx.n = std::max<int64_t>(mx.n, s.n);
  }
  mx.trials = tmax;
  const int stride = dt->stride;
  // static fields of the iteration descriptors (k_plan fills the rest)
  for (int i = 0; i < nsig; ++i) {
    SigIter &it = (*its)[i];
    it.x = sigs[i]->d_x;
    it.n = int32_t(sigs[i]->n);
    it.phase_shift = -1;
    if (IsPow2(sigs[i]->n)) {
      int k = 0;
      while ((int64_t(1) << k) < sigs[i]->n) ++k;
      it.phase_shift = 32 - k;
    }
    it.trials = opts[i].trials;
    it.active = 0;
    it.trace = i == 0 ? ctx->trace : nullptr;
    it.trace_count = i == 0 ? ctx->trace_count : nullptr;
    it.trace_cap = kTimelineCapacity;
  }
  {
    int rc = Upload(ctx, d_its, its->data(), sizeof(SigIter) * nsig, ctx->stream);
    if (rc == MPSFT_OK) {
      rc = Upload(ctx, d_its_ahead, its->data(), sizeof(SigIter) * nsig, ctx->stream);
    }
    if (rc) return rc;
  }
  std::vector<SolveCtl> &hc = dt->hc;
  std::vector<int32_t> &hd = dt->hd;
  std::vector<double> &hb = dt->hb;
  const size_t bq_per = dt->bq_per;
  for (int i = 0; i < nsig; ++i) hc[i].force_fp64 = force[i];
  {
    int rc = Upload(ctx, ctx->d_draws, hd.data(), sizeof(int32_t) * hd.size(), ctx->stream);
    if (rc == MPSFT_OK) {
      rc = Upload(ctx, ctx->d_draw_bq, hb.data(), sizeof(double) * hb.size(), ctx->stream);
    }
    if (rc == MPSFT_OK) {
      rc = Upload(ctx, ctx->d_solve_ctl, hc.data(), sizeof(SolveCtl) * nsig, ctx->stream);
    }
    if (rc) return rc;
  }
  // late-iteration phase: bins up to small_bins (a few times min_bins)
  int32_t min_bins_max = 1;
  int32_t min_bins_min = INT32_MAX;
  for (int i = 0; i < nsig; ++i) {
    min_bins_max = std::max(min_bins_max, opts[i].min_bins);
    min_bins_min = std::min(min_bins_min, opts[i].min_bins);
  }
  const int32_t small_bins = (4 * min_bins_max) | 1;
  const bool two_phase = mx.bins > small_bins;
  Maxima mx_small = mx;
  if (two_phase) {
    mx_small.bins = small_bins;
    mx_small.m = 1 << FFTLog2(small_bins);
    mx_small.p2 = 0;
    // (once per distinct window delta; a batch usually shares one)
    std::vector<double> deltas;
    for (int i = 0; i < nsig; ++i) {
      const double d = opts[i].window_delta;
      if (std::find(deltas.begin(), deltas.end(), d) != deltas.end()) continue;
      deltas.push_back(d);
      for (int32_t bb = min_bins_min | 1; bb <= small_bins; bb += 2) {
        mx_small.p2 = std::max(mx_small.p2, MakeWindow(bb, d).p2);
      }
    }
  }
  // the fixed-bins phase runs pipelined on the FP32 path without FP64 redo
  const bool pipe = !fp64 && !(any_forced && mx.m <= kMaxFFT64);
  // graph (rebuilt when the launch shape or the arena changes)
  const std::vector<int64_t> key = {
      int64_t(reinterpret_cast<uintptr_t>(ctx->arena)), nsig, mx.bins, mx.bits,
      mx.rows, mx.p2, mx.m, mx.cap, mx.trials, fp64, x_c128, any_forced,
      small_bins, mx_small.p2, pipe, ctx->tuning_version, ctx->force_shape};
  if (ctx->graph_key != key || ctx->graph_exec == nullptr) {
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->graph) cudaGraphDestroy(ctx->graph);
    ctx->graph_exec = nullptr;
    ctx->graph = nullptr;
    ctx->graph_key.clear();
    MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaGraph_t g = nullptr;
    MPSFT_CUDA(ctx, cudaGraphCreate(&g, 0));
    ctx->graph = g;
    // One while node per phase: the first runs every signal with launch
    // shapes for the largest bins; once no signal needs more than small_bins,
    // the second runs with shapes for small_bins (the late iterations, where
    // most of a solve's iterations are, then launch no idle blocks). With
    // pipelining, the second ends when every signal with work is at fixed
    // bins (min_bins from then on), and a third runs the rest with the next
    // iteration's plan and gather/fold beside the current one's decisions,
    // after a prologue that plans and folds its first iteration.
    struct Phase {
      Maxima shape;
      int32_t plan_max, cond_lo, cond_hi;
      bool exclude_fixed, pipelined;
    };
    std::vector<Phase> phases;
    if (two_phase) {
      phases.push_back({mx, INT32_MAX, small_bins, INT32_MAX, false, false});
      phases.push_back({mx_small, small_bins, 0, small_bins, pipe, false});
    } else {
      phases.push_back({mx, INT32_MAX, 0, INT32_MAX, pipe, false});
    }
    if (pipe) {
      Phase last = phases.back();
      last.exclude_fixed = false;
      last.pipelined = true;
      // every signal with work is at its min_bins: the row transforms are no
      // longer than those of the largest min_bins (small bins take the direct
      // DFT, LaunchRowFFT)
      last.shape.m = std::min(last.shape.m, 1 << FFTLog2(min_bins_max));
      phases.push_back(last);
    }
    int rc = MPSFT_OK;
    cudaError_t ce = cudaSuccess;
    int64_t per_body = 1;
    // the captured kernels use programmatic dependent launch
    struct PdlScope {
      PdlScope() { g_launch_pdl = true; }
      ~PdlScope() { g_launch_pdl = false; }
    } pdl_scope;
    cudaGraphNode_t prev = nullptr;
    for (const Phase &ph : phases) {
      if (ph.pipelined) {
        // prologue: plan, fold and Bluestein tables of the phase's first
        // iteration
        cudaGraph_t pg = nullptr;
        MPSFT_CUDA(ctx, cudaGraphCreate(&pg, 0));
        ce = cudaStreamBeginCaptureToGraph(ctx->cap, pg, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal);
        if (ce == cudaSuccess) {
          LaunchPlan(ctx->d_solve_ctl, d_its, nsig, ph.plan_max, ctx->cap);
          LaunchWindow32(d_its, nsig, ph.shape.p2, ctx->cap);
          LaunchBinFold(d_its, nsig, ph.shape.bins, ph.shape.bits, ph.shape.trials,
                        x_c128, false, ctx->cap, false,
                        FoldShapeFor(ctx, ph.shape.bins, ph.shape.n, nsig, x_c128));
          LaunchBluesteinSetup(d_its, nsig, ph.shape.m, false, ctx->tw32, ctx->tw64,
                               ctx->cap);
          cudaGraph_t captured = nullptr;
          ce = cudaStreamEndCapture(ctx->cap, &captured);
        }
        cudaGraphNode_t child = nullptr;
        if (ce == cudaSuccess) {
          ce = cudaGraphAddChildGraphNode(&child, g, prev ? &prev : nullptr,
                                          prev ? 1 : 0, pg);
        }
        cudaGraphDestroy(pg);  // the node holds its own copy
        if (ce != cudaSuccess) break;
        prev = child;
      }
      cudaGraphConditionalHandle handle;
      MPSFT_CUDA(ctx, cudaGraphConditionalHandleCreate(&handle, g, 1,
                                                       cudaGraphCondAssignDefault));
      // the params union has no default constructor: zeroed raw storage
      alignas(cudaGraphNodeParams) unsigned char pbuf[sizeof(cudaGraphNodeParams)];
      std::memset(pbuf, 0, sizeof(pbuf));
      cudaGraphNodeParams &p = *reinterpret_cast<cudaGraphNodeParams *>(pbuf);
      p.type = cudaGraphNodeTypeConditional;
      p.conditional.handle = handle;
      p.conditional.type = cudaGraphCondTypeWhile;
      p.conditional.size = 1;
      cudaGraphNode_t node;
      MPSFT_CUDA(ctx, cudaGraphAddNode(&node, g, prev ? &prev : nullptr, nullptr,
                                       prev ? 1 : 0, &p));
      prev = node;
      cudaGraph_t body = p.conditional.phGraph_out[0];
      MPSFT_CUDA(ctx, cudaStreamBeginCaptureToGraph(ctx->cap, body, nullptr, nullptr,
                                                    0, cudaStreamCaptureModeThreadLocal));
      if (!ph.pipelined) LaunchPlan(ctx->d_solve_ctl, d_its, nsig, ph.plan_max, ctx->cap);
      per_body = 1;
      const Ahead ah{d_its_ahead, ctx->d_solve_ctl, ph.plan_max};
      rc = LaunchIterationKernels(ctx, d_its, nsig, ph.shape, x_c128, fp64,
                                  any_forced, nullptr, &per_body, ctx->cap,
                                  ph.pipelined ? &ah : nullptr);
      cudaError_t we = cudaSuccess;
      if (ph.pipelined) {
        // the stop rule after the plan ahead has read the solve state; the
        // planned descriptors become current once the next fold is done
        we = cudaStreamWaitEvent(ctx->cap, ctx->ev_plan_p, 0);
        LaunchFinish(ctx->d_solve_ctl, d_its, nsig, handle, true, ph.cond_lo,
                     ph.cond_hi, ctx->cap, d_its_ahead, false);
        if (we == cudaSuccess) we = cudaStreamWaitEvent(ctx->cap, ctx->ev_join_p, 0);
        LaunchCopyMapped(d_its_ahead, d_its, sizeof(SigIter) * nsig, ctx->cap);
        per_body += 1;
      } else {
        LaunchFinish(ctx->d_solve_ctl, d_its, nsig, handle, true, ph.cond_lo,
                     ph.cond_hi, ctx->cap, nullptr, ph.exclude_fixed);
      }
      cudaGraph_t captured = nullptr;
      ce = cudaStreamEndCapture(ctx->cap, &captured);
      if (ce == cudaSuccess) ce = we;
      if (rc != MPSFT_OK || ce != cudaSuccess) break;
    }
    cudaGraphExec_t exec = nullptr;
    cudaError_t ie = cudaErrorUnknown;
    // the side stream's priority was captured into its kernel nodes
    if (rc == MPSFT_OK && ce == cudaSuccess) {
      ie = cudaGraphInstantiate(&exec, g, cudaGraphInstantiateFlagUseNodePriority);
    }
    if (rc != MPSFT_OK || ce != cudaSuccess || ie != cudaSuccess) {
      // no graph on this device / driver: the host loop takes over
      cudaGetLastError();
      cudaGraphDestroy(g);
      ctx->graph = nullptr;
      ctx->graph_unavailable = true;
      return kGraphUnavailable;
    }
    ctx->graph_exec = exec;
    ctx->graph_key = key;
    ctx->graph_body_kernels = per_body + 1;
  }
  // run until every signal has stopped; refill draw tables in between
  const int max_launches = 4 + (hc[0].max_iter + kDrawChunk - 1) / kDrawChunk * 2;
  int64_t body_runs = 0;
  std::vector<int32_t> prev_iter(nsig, 0);
  for (int launch = 0;; ++launch) {
    if (launch > 8 + max_launches * nsig) {
      return Fail(ctx, MPSFT_ERR_ITER_CAP, "solve graph did not converge");
    }
    MPSFT_CUDA(ctx, cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    MPSFT_CUDA(ctx, cudaEventRecord(ctx->ev_loop1, ctx->stream));
    // the solve state and, for the usual case that every signal has
    // stopped, the results with it: one wait per graph launch
    int rc = LaunchResults(ctx, d_its, rs);
    if (rc) return rc;
    *launches += 2;
    MPSFT_CUDA(ctx, cudaGetLastError());
    MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    std::memcpy(hc.data(), rs.at<SolveCtl>(ctx->h_stage, rs.ctl), sizeof(SolveCtl) * nsig);
    ctx->up_off = 0;  // every upload so far has been consumed
    int32_t most = 0;
    bool all_done = true, refilled = false;
    for (int i = 0; i < nsig; ++i) {
      most = std::max(most, hc[i].iter - prev_iter[i]);
      prev_iter[i] = hc[i].iter;
      if (hc[i].done) continue;
      all_done = false;
      if (hc[i].iter - hc[i].draw_base >= hc[i].draws_avail) {
        // the next kDrawChunk iterations continue this signal's RNG stream
        FillDraws(&dt->work[i], int32_t(sigs[i]->n), opts[i].trials, stride,
                  hd.data() + size_t(i) * kDrawChunk * stride,
                  hb.data() + i * bq_per);
        const int32_t window[2] = {hc[i].iter, kDrawChunk};
        int rc = Upload(ctx, ctx->d_draws + size_t(i) * kDrawChunk * stride,
                        hd.data() + size_t(i) * kDrawChunk * stride,
                        sizeof(int32_t) * kDrawChunk * stride, ctx->stream);
        if (rc == MPSFT_OK) {
          rc = Upload(ctx, ctx->d_draw_bq + i * bq_per, hb.data() + i * bq_per,
                      sizeof(double) * bq_per, ctx->stream);
        }
        if (rc == MPSFT_OK) {
          rc = Upload(ctx, &ctx->d_solve_ctl[i].draw_base, window, sizeof(window),
                      ctx->stream);
        }
        if (rc) return rc;
        refilled = true;
      }
    }
    body_runs += most;
    if (all_done) break;
    if (!refilled) {
      return Fail(ctx, MPSFT_ERR_CUDA, "solve graph stopped with work left");
    }
  }
  *launches += body_runs * ctx->graph_body_kernels;
  *ctl_out = hc;
  // each caller's generator takes exactly the used draws, 3 + trials per
  // iteration (DrawTransform's a, b, c, then the q's), before its next draw
  for (int i = 0; i < nsig; ++i) {
    rngs[i]->pending += int64_t(hc[i].iter) * (3 + opts[i].trials);
  }
  return MPSFT_OK;
}

// Results of every signal one after another in two arrays (signal i at
// [offsets[i], offsets[i + 1])), for mpsft_solve_batched_packed.
struct PackedOut {
  int32_t *k;
  double *c;
  int64_t cap;
  int64_t *offsets;
};

// One batched solve; the core of mpsft_solve, mpsft_solve_batched and
// mpsft_solve_batched_packed (packed: out_k, out_c, cap are unused).
int SolveMany(mpsft_ctx *ctx, const mpsft_signal *const *sigs,
              const mpsft_solve_options *opts, int32_t nsig,
              mpsft_rng *const *rngs, int32_t *const *out_k,
              double *const *out_c, const int32_t *cap, int32_t *count,
              mpsft_stats *stats, const PackedOut *packed = nullptr) {
  if (nsig <= 0) return Fail(ctx, MPSFT_ERR_INVALID, "no signals");
  const bool fp64 = opts[0].precision == MPSFT_PREC_FP64;
  const bool x_c128 = sigs[0]->dtype == MPSFT_C128;
  std::vector<Shape> shapes(nsig);
  size_t bytes = 0;
  for (int i = 0; i < nsig; ++i) {
    const mpsft_solve_options &o = opts[i];
    int rc = CheckSignal(ctx, sigs[i]);
    if (rc) return rc;
    if (!rngs[i]) return Fail(ctx, MPSFT_ERR_INVALID, "null rng");
    if ((o.precision == MPSFT_PREC_FP64) != fp64) {
      return Fail(ctx, MPSFT_ERR_INVALID, "all signals must share a precision");
    }
    if ((sigs[i]->dtype == MPSFT_C128) != x_c128) {
      return Fail(ctx, MPSFT_ERR_INVALID, "all signals must share a dtype");
    }
    if (o.trials < 1 || o.trials % 2 == 0 || o.trials > kMaxTrials) {
      return Fail(ctx, MPSFT_ERR_INVALID, "trials must be odd and <= 15");
    }
    if (o.k < 0 || o.min_bins < 1 || o.max_stale_iter < 1) {
      return Fail(ctx, MPSFT_ERR_INVALID, "bad k, min_bins or max_stale_iter");
    }
    if (!(o.window_threshold > 0)) {
      return Fail(ctx, MPSFT_ERR_INVALID, "window_threshold must be > 0");
    }
    const int32_t n = int32_t(sigs[i]->n);
    const int64_t bmax64 = std::max<int64_t>(2 * int64_t(o.k) + 1, o.min_bins);
    if (bmax64 > INT32_MAX) return Fail(ctx, MPSFT_ERR_INVALID, "k too large");
    Shape &s = shapes[i];
    s.n = n;
    s.bins_cap = int32_t(bmax64);
    // Window CHECKs an odd number of bins (src/window.cc:33); B is
    // 2(k - found) + 1 or min_bins, so min_bins must be odd.
    if (o.min_bins % 2 == 0) {
      return Fail(ctx, MPSFT_ERR_INVALID, "min_bins must be odd");
    }
    for (int32_t bb : {s.bins_cap, std::min(s.bins_cap, o.min_bins)}) {
      rc = CheckWindow(ctx, bb, o.window_delta, fp64);
      if (rc) return rc;
    }
    s.rows_cap = 1 + 2 * NumBits(n, std::min(s.bins_cap, o.min_bins));
    s.trials = o.trials;
    s.p2_cap = std::max(MakeWindow(s.bins_cap, o.window_delta).p2,
                        MakeWindow(std::min(s.bins_cap, o.min_bins),
                                   o.window_delta).p2);
    s.m_cap = 1 << FFTLog2(s.bins_cap);
    s.tab_cap = o.mode_capacity > 0
                    ? NextPow2(o.mode_capacity)
                    : NextPow2(std::max<int64_t>(64, 2 * (int64_t(o.k) + s.bins_cap)));
    if (s.tab_cap > kMaxTableCap) {
      return Fail(ctx, MPSFT_ERR_INVALID, "mode table larger than 32768 slots");
    }
    s.fp64 = fp64;
    s.fp32_bins = !fp64;
    // complex64 FP32 solves stash the fold's gathered samples (StashRows)
    if (!fp64 && !x_c128) {
      s.stash_cap = int64_t(s.trials) *
                    std::max<int64_t>(2 * int64_t(s.p2_cap) + 1,
                                      std::min<int64_t>(n / 8, kStashMaxSamples));
    }
    Carve probe{nullptr};
    SigIter dummy{};
    int32_t *ctl = nullptr;
    CarveSignal(probe, s, &dummy, &ctl);
    bytes += probe.off + 256;
  }
  bytes += 2 * (sizeof(SigIter) * nsig + 256);
  bytes += (sizeof(double) * kEnergyStride + sizeof(void *) + sizeof(int64_t)) *
               nsig + 1024;
  int max_trials_all = 1;
  for (int i = 0; i < nsig; ++i) max_trials_all = std::max(max_trials_all, opts[i].trials);
  bytes += (sizeof(SolveCtl) +
            sizeof(int32_t) * kDrawChunk * (4 + max_trials_all) +
            sizeof(double) * kDrawChunk * max_trials_all * 2) * nsig + 2048;
  constexpr int kTimelineCap = kTimelineCapacity;
  bytes += 2 * sizeof(unsigned long long) * kTimelineCap + 512;
  int max_cap = 1;
  for (int i = 0; i < nsig; ++i) max_cap = std::max(max_cap, shapes[i].tab_cap);
  // the results' staging (solve state, tables' entries), on the device and
  // in pinned host memory
  ResultStage rs(nsig, max_cap);
  bytes += rs.bytes + 256;
  int rc = EnsureArena(ctx, bytes);
  if (rc) return rc;
  rc = EnsureHostStage(ctx, rs.bytes);
  if (rc) return rc;
  rc = EnsureHostCtl(ctx, size_t(kCtlWords) * nsig);
  if (rc) return rc;

  Carve cv{ctx->arena};
  SigIter *d_its = cv.take<SigIter>(nsig);
  SigIter *d_its_ahead = cv.take<SigIter>(nsig);  // fixed-bins phase
  double *d_energy = cv.take<double>(size_t(kEnergyStride) * nsig);
  const void **d_xs = cv.take<const void *>(nsig);
  int64_t *d_ns = cv.take<int64_t>(nsig);
  ctx->d_solve_ctl = cv.take<SolveCtl>(nsig);
  unsigned long long *d_trace = cv.take<unsigned long long>(2 * kTimelineCap);
  uint32_t *d_trace_count = cv.take<uint32_t>(1);
  ctx->d_draws = cv.take<int32_t>(size_t(nsig) * kDrawChunk * (4 + max_trials_all));
  ctx->d_draw_bq = cv.take<double>(size_t(nsig) * kDrawChunk * max_trials_all * 2);
  rs.dev = cv.take<unsigned char>(rs.bytes);
  std::vector<SigIter> its(nsig);
  std::vector<int32_t *> ctls(nsig);
  int64_t phase_entries = 1;
  for (int i = 0; i < nsig; ++i) {
    std::memset(&its[i], 0, sizeof(SigIter));
    CarveSignal(cv, shapes[i], &its[i], &ctls[i]);
    its[i].n = int32_t(sigs[i]->n);
    phase_entries = std::max(phase_entries, PhaseTableEntries(sigs[i]->n));
  }
  // the signals of the first one's length share the context's phase tables
  // of that length (built once, by the first of them, when the length is
  // new); other lengths build their own
  {
    const int64_t n0 = sigs[0]->n;
    const size_t lo = size_t(1) << PhaseTableK(n0), hi = size_t(PhaseTableHi(n0));
    const bool fresh = ctx->ph_cache_n != n0;
    if (fresh) {
      if (ctx->ph_cache) cudaFree(ctx->ph_cache);
      ctx->ph_cache = nullptr;
      ctx->ph_cache_n = 0;
      MPSFT_CUDA(ctx, cudaMalloc(&ctx->ph_cache, sizeof(double2) * (lo + hi)));
    }
    bool first = true;
    for (int i = 0; i < nsig; ++i) {
      if (sigs[i]->n != n0) continue;
      its[i].ph_lo = ctx->ph_cache;
      its[i].ph_hi = ctx->ph_cache + lo;
      its[i].ph_build = fresh && first ? 1 : 0;
      first = false;
    }
  }
  // the call's small uploads (descriptors three times, signal pointers and
  // lengths, draw tables, solve state) fit the staging without a wait
  rc = EnsureUploadStage(
      ctx, 3 * sizeof(SigIter) * nsig + 16 * size_t(nsig) +
               size_t(nsig) * kDrawChunk * (4 + max_trials_all) * sizeof(int32_t) +
               size_t(nsig) * kDrawChunk * max_trials_all * 2 * sizeof(double) +
               sizeof(SolveCtl) * nsig + 16 * 256);
  if (rc) return rc;
  ctx->up_off = 0;
  ctx->up_launches = 0;
  // empty tables and the FP64 unit-phase tables (per signal length, for the
  // whole call)
  rc = Upload(ctx, d_its, its.data(), sizeof(SigIter) * nsig, ctx->stream);
  if (rc) return rc;
  LaunchClearTables(d_its, nsig, max_cap, ctx->stream);
  bool any_phase = false;
  for (int i = 0; i < nsig; ++i) any_phase |= its[i].ph_build != 0;
  if (any_phase) LaunchPhaseTables(d_its, nsig, phase_entries, ctx->stream);
  MPSFT_CUDA(ctx, cudaGetLastError());
  ctx->ph_cache_n = sigs[0]->n;  // the shared tables are built (or were)
  bool host_loop = ctx->profiling || ctx->graph_unavailable;
  std::vector<double> energy(nsig, 0.0);
  DrawTables draws;
  if (!fp64) {
    // an estimate of every signal's mean |x|^2 for the precision policy
    std::vector<const void *> h_xs(nsig);
    std::vector<int64_t> h_ns(nsig);
    for (int i = 0; i < nsig; ++i) {
      h_xs[i] = sigs[i]->d_x;
      h_ns[i] = sigs[i]->n;
    }
    rc = Upload(ctx, d_xs, h_xs.data(), sizeof(void *) * nsig, ctx->stream);
    if (rc) return rc;
    rc = Upload(ctx, d_ns, h_ns.data(), sizeof(int64_t) * nsig, ctx->stream);
    if (rc) return rc;
    LaunchEnergy(d_xs, d_ns, nsig, x_c128, d_energy, ctx->stream, kPolicySample);
    // the host's share of the solve graph runs while the GPU reads x
    if (!host_loop) PrepareDraws(ctx, sigs, opts, nsig, rngs, fp64, &draws);
    rc = ReadEnergy(ctx, d_energy, nsig, &energy);
    if (rc) return rc;
  } else if (!host_loop) {
    PrepareDraws(ctx, sigs, opts, nsig, rngs, fp64, &draws);
  }
  // precision policy, once per solve (FP32 calls)
  std::vector<int32_t> force(nsig, 0);
  bool any_forced = false;
  for (int i = 0; i < nsig; ++i) {
    const mpsft_solve_options &o = opts[i];
    const int32_t b0 = shapes[i].bins_cap;
    force[i] = !fp64 && PolicyForcesFP64(o.near_tie_margin, b0, energy[i],
                                         3.0 * o.sigma / std::sqrt(double(b0)),
                                         o.sigma / std::sqrt(double(b0)));
    any_forced |= force[i] != 0;
  }
  struct Run {
    int32_t iter = 0, stale = 0, found = 0, status = MPSFT_OK;
    bool done = false;
    int64_t gathers = 0, bin_bytes = 0;
    int32_t near_ties = 0, unresolved = 0, fp64_iters = 0;
    int32_t last_bins = -1;  // bins of the previous iteration (tables reuse)
  };
  std::vector<Run> run(nsig);
  BinTimer timer{ctx};
  int64_t launches = 0;
  if (!host_loop && !fp64) {
    // the FP32 tables from the context's cache when the batch shares one
    // window delta
    bool one_delta = true;
    int32_t bmin = INT32_MAX, bmax = 1;
    for (int i = 0; i < nsig; ++i) {
      one_delta = one_delta && opts[i].window_delta == opts[0].window_delta;
      bmin = std::min(bmin, std::min(shapes[i].bins_cap, opts[i].min_bins));
      bmax = std::max(bmax, shapes[i].bins_cap);
    }
    WinCacheRefs wc;
    if (one_delta) {
      rc = EnsureWinCache(ctx, opts[0].window_delta, bmin, bmax, &wc);
      if (rc) return rc;
    }
    for (int i = 0; i < nsig; ++i) {
      draws.hc[i].win_base = wc.base;
      draws.hc[i].win_pool = wc.pool;
      draws.hc[i].win_valid = wc.valid;
      draws.hc[i].win_claim = wc.claim;
    }
  }
  ctx->timeline.clear();
  ctx->trace = nullptr;
  ctx->trace_count = nullptr;
  if (!host_loop && ctx->timeline_on) {
    MPSFT_CUDA(ctx, cudaMemsetAsync(d_trace_count, 0, sizeof(uint32_t), ctx->stream));
    ctx->trace = d_trace;
    ctx->trace_count = d_trace_count;
  }
  MPSFT_CUDA(ctx, cudaEventRecord(ctx->ev_loop0, ctx->stream));
  std::vector<SolveCtl> h_ctl;
  if (!host_loop) {
    rc = GraphLoop(ctx, sigs, opts, nsig, rngs, shapes, d_its, d_its_ahead, &its, &draws,
                   force, any_forced, fp64, x_c128, &launches, rs, &h_ctl);
    if (rc == kGraphUnavailable) {
      // no iteration ran and the tables are untouched; the RNGs are back
      // where they were
      host_loop = true;
    } else if (rc) {
      return rc;
    }
  }
  if (!host_loop) {
    // (the graph's solve state and results are in the staging already)
    if (ctx->trace != nullptr) {
      uint32_t cnt = 0;
      MPSFT_CUDA(ctx, cudaMemcpy(&cnt, d_trace_count, sizeof(cnt),
                                 cudaMemcpyDeviceToHost));
      cnt = std::min<uint32_t>(cnt, kTimelineCap);
      ctx->timeline.resize(2 * size_t(cnt));
      if (cnt > 0) {
        MPSFT_CUDA(ctx, cudaMemcpy(ctx->timeline.data(), d_trace,
                                   sizeof(unsigned long long) * ctx->timeline.size(),
                                   cudaMemcpyDeviceToHost));
      }
    }
    for (int i = 0; i < nsig; ++i) {
      Run &r = run[i];
      const SolveCtl &c = h_ctl[i];
      r.iter = c.iter;
      r.stale = c.stale;
      r.status = c.status;
      r.gathers = c.gathers;
      r.bin_bytes = c.bin_bytes;
      r.near_ties = c.near_ties;
      r.unresolved = c.unresolved;
      r.fp64_iters = c.fp64_iters;
    }
  }
  int active = host_loop ? nsig : 0;
  if (ctx->profiling) ctx->bin_launches.clear();
  // per iteration: the binning launch's signals, and those of its FP64 redo
  std::vector<std::pair<mpsft_bin_launch, mpsft_bin_launch>> iter_recs;
  while (active > 0) {
    mpsft_bin_launch rec[2] = {};
    for (int k = 0; k < 2; ++k) {
      rec[k].iteration = int32_t(iter_recs.size());
      rec[k].min_bins = INT32_MAX;
      rec[k].precision = (fp64 || k == 1) ? MPSFT_PREC_FP64 : MPSFT_PREC_FP32;
    }
    for (int i = 0; i < nsig; ++i) {
      SigIter &it = its[i];
      if (run[i].done) {
        it.active = 0;
        continue;
      }
      const mpsft_solve_options &o = opts[i];
      const int32_t n = int32_t(sigs[i]->n);
      const int32_t bins =
          std::max<int32_t>((o.k - run[i].found) * 2 + 1, o.min_bins);
      const int32_t bits = NumBits(n, bins);
      const Transform tf = DrawTransform(rngs[i], n);
      int32_t q[kMaxTrials];
      for (int t = 0; t < o.trials; ++t) q[t] = rngs[i]->Draw() % n;
      FillIter(&it, sigs[i], bins, bits, o.window_delta, tf, q, o.trials);
      it.bin_thr = 3.0 * o.sigma / std::sqrt(double(bins));
      it.sv_thr = 1.0 * o.sigma / std::sqrt(double(bins));
      SetThresholdCopies(&it);
      it.win_thr = o.window_threshold;
      SetNearTie(&it, fp64, o.near_tie_margin, bins, force[i] != 0);
      run[i].fp64_iters += it.force_fp64;
      // same bins as the last iteration: window and Bluestein tables stand
      // (a forced FP64 iteration leaves the FP32 tables unbuilt)
      it.tables_valid = (run[i].last_bins == bins && !it.force_fp64) ? 1 : 0;
      run[i].last_bins = it.force_fp64 ? -1 : bins;
      run[i].gathers += BinGathers(it, fp64 || it.force_fp64);
      run[i].bin_bytes += BinBytes(it, fp64 || it.force_fp64);
      mpsft_bin_launch &r = rec[it.force_fp64 ? 1 : 0];
      r.signals += 1;
      r.max_bins = std::max(r.max_bins, bins);
      r.min_bins = std::min(r.min_bins, bins);
      r.gathers += BinGathers(it, fp64 || it.force_fp64);
      r.bytes += BinBytes(it, fp64 || it.force_fp64);
    }
    if (ctx->profiling) iter_recs.emplace_back(rec[0], rec[1]);
    MPSFT_CUDA(ctx, cudaMemcpyAsync(d_its, its.data(), sizeof(SigIter) * nsig,
                                    cudaMemcpyHostToDevice, ctx->stream));
    for (int i = 0; i < nsig; ++i) {
      if (!run[i].done) {
        MPSFT_CUDA(ctx, cudaMemsetAsync(ctls[i], 0, sizeof(int32_t) * 3,
                                        ctx->stream));
      }
    }
    // the launch shape the solve graph would use for this iteration
    int32_t bins_now = 0, bins_cap = 0, min_bins_max = 1;
    for (int i = 0; i < nsig; ++i) {
      bins_cap = std::max(bins_cap, shapes[i].bins_cap);
      min_bins_max = std::max(min_bins_max, opts[i].min_bins);
      if (its[i].active) bins_now = std::max(bins_now, its[i].bins);
    }
    rc = LaunchIteration(ctx, d_its, nsig, its, x_c128, fp64, &timer, &launches,
                         PhaseBins(bins_now, bins_cap, min_bins_max));
    if (rc) return rc;
    for (int i = 0; i < nsig; ++i) {
      MPSFT_CUDA(ctx, cudaMemcpyAsync(ctx->h_ctl + kCtlWords * i, ctls[i],
                                      sizeof(int32_t) * kCtlWords,
                                      cudaMemcpyDeviceToHost, ctx->stream));
    }
    MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < nsig; ++i) {
      if (run[i].done) continue;
      const mpsft_solve_options &o = opts[i];
      const int32_t *c = ctx->h_ctl + kCtlWords * i;
      Run &r = run[i];
      r.iter += 1;
      r.found = c[3];
      r.near_ties += c[2];
      if (c[1] & kStatusUnresolved) r.unresolved += 1;
      if (c[1] & kStatusCapacity) {
        r.status = MPSFT_ERR_CAPACITY;
      } else if (c[1] & kStatusNonFinite) {
        r.status = MPSFT_ERR_NONFINITE;
      } else if (int64_t(r.found) * 2 > its[i].tab_cap) {
        r.status = MPSFT_ERR_CAPACITY;
      }
      if (!c[0]) r.stale += 1;
      const int32_t max_iter = o.max_iter > 0 ? o.max_iter : 64 + 8 * o.k;
      if (r.status == MPSFT_OK && r.stale < o.max_stale_iter &&
          r.iter >= max_iter) {
        r.status = MPSFT_ERR_ITER_CAP;
      }
      if (r.status != MPSFT_OK || r.stale >= o.max_stale_iter) {
        r.done = true;
        --active;
      }
    }
  }
  if (host_loop) {
    MPSFT_CUDA(ctx, cudaEventRecord(ctx->ev_loop1, ctx->stream));
    rc = LaunchResults(ctx, d_its, rs);
    if (rc) return rc;
    launches += 2;
    MPSFT_CUDA(ctx, cudaGetLastError());
  }
  int first_err = MPSFT_OK;
  const double bin_ms = timer.TotalMs();
  if (ctx->profiling) {
    // timed launches in order: each iteration's binning (tag 0), then its
    // FP64 redo when it has one (tag 1); launches that binned no signal
    // (every signal on the other kind of kernel) are left out
    MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    size_t k = 0;
    for (size_t j = 0; j < timer.used.size(); ++j) {
      const bool redo = timer.tags[j] == 1;
      if (!redo) ++k;
      if (k == 0 || k > iter_recs.size()) break;
      mpsft_bin_launch r = redo ? iter_recs[k - 1].second : iter_recs[k - 1].first;
      if (r.signals == 0) continue;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, timer.used[j].first, timer.used[j].second);
      r.ms = ms;
      ctx->bin_launches.push_back(r);
    }
  }
  // the call's own kernels outside the loop: table clearing, phase tables,
  // the energy pair (FP32) and the upload copies
  launches += 1 + (any_phase ? 1 : 0) + (fp64 ? 0 : 2) + ctx->up_launches;
  // every table's entries (k_export_tables, with the solve state) in the
  // host staging: counts and sorted flags, then the packed keys and
  // coefficients, signal after signal
  MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  rc = FinishResults(ctx, rs);
  if (rc) return rc;
  const int32_t *counts = rs.at<int32_t>(ctx->h_stage, rs.counts);
  const int32_t *sorted = rs.at<int32_t>(ctx->h_stage, rs.sorted);
  const int32_t *h_keys = rs.at<int32_t>(ctx->h_stage, rs.keys);
  const double2 *h_coefs = rs.at<double2>(ctx->h_stage, rs.coefs);
  size_t res_off = 0;  // signal i's entries in the staging
  int64_t packed_off = 0;
  float loop_ms = 0.f;
  MPSFT_CUDA(ctx, cudaEventElapsedTime(&loop_ms, ctx->ev_loop0, ctx->ev_loop1));
  for (int i = 0; i < nsig; ++i) {
    const int32_t *ki = h_keys + res_off;
    const double2 *ci = h_coefs + res_off;
    res_off += size_t(counts[i]);
    std::vector<int32_t> order;
    if (!sorted[i]) {
      order.resize(counts[i]);
      for (int32_t j = 0; j < counts[i]; ++j) order[j] = j;
      std::sort(order.begin(), order.end(),
                [ki](int32_t l, int32_t r) { return ki[l] < ki[r]; });
    }
    int st = run[i].status;
    const int32_t m = counts[i];
    int32_t room = 0;
    int32_t *dk = nullptr;
    double *dc = nullptr;
    if (packed) {
      room = int32_t(std::min<int64_t>(packed->cap - packed_off, INT32_MAX));
      dk = packed->k + packed_off;
      dc = packed->c + 2 * packed_off;
      packed->offsets[i] = packed_off;
    } else {
      room = cap[i];
      dk = out_k[i];
      dc = out_c[i];
    }
    if (m > room) st = st ? st : MPSFT_ERR_CAPACITY;
    const int32_t w = std::min(m, room);
    if (sorted[i]) {
      // (re, im) pairs of doubles: the staging's layout is the caller's
      std::memcpy(dk, ki, sizeof(int32_t) * size_t(w));
      std::memcpy(dc, ci, sizeof(double2) * size_t(w));
    } else {
      for (int32_t j = 0; j < w; ++j) {
        const int32_t s = order[j];
        dk[j] = ki[s];
        dc[2 * j] = ci[s].x;
        dc[2 * j + 1] = ci[s].y;
      }
    }
    if (packed) {
      packed_off += w;
      packed->offsets[i + 1] = packed_off;
    }
    count[i] = m;
    if (stats) {
      mpsft_stats &s = stats[i];
      std::memset(&s, 0, sizeof(s));
      s.iterations = run[i].iter;
      s.found = m;
      s.gathers = run[i].gathers;
      s.bin_bytes = run[i].bin_bytes;
      s.bin_launches = int32_t(timer.used.size());
      s.bin_ms = bin_ms;
      s.status = st;
      s.kernel_launches = launches;
      s.escalated = run[i].near_ties;
      s.unresolved = run[i].unresolved;
      s.fp64_iterations = run[i].fp64_iters;
      s.loop_ms = loop_ms;
    }
    if (st && !first_err) {
      first_err = st;
      char buf[160];
      std::snprintf(buf, sizeof(buf), "signal %d: %s after %d iterations", i,
                    mpsft_status_string(st), run[i].iter);
      ctx->err = buf;
    }
  }
  return first_err;
}

}  // namespace

// ===================================================================== ABI
extern "C" {

const char *mpsft_status_string(int status) {
  switch (status) {
    case MPSFT_OK: return "ok";
    case MPSFT_ERR_INVALID: return "invalid argument";
    case MPSFT_ERR_UNSUPPORTED_N: return "unsupported n";
    case MPSFT_ERR_CUDA: return "CUDA error";
    case MPSFT_ERR_CAPACITY: return "capacity exceeded";
    case MPSFT_ERR_ITER_CAP: return "iteration cap reached";
    case MPSFT_ERR_NONFINITE: return "non-finite values in the bins";
    case MPSFT_ERR_NOMEM: return "out of device memory";
    default: return "unknown status";
  }
}

int mpsft_ctx_create(int device, mpsft_ctx **out) {
  if (!out) return MPSFT_ERR_INVALID;
  *out = nullptr;
  mpsft_ctx *ctx = new mpsft_ctx;
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking);
  int prio_least = 0, prio_greatest = 0;
  if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  if (e == cudaSuccess) {
    e = cudaStreamCreateWithPriority(&ctx->side, cudaStreamNonBlocking, prio_greatest);
  }
  if (e == cudaSuccess) {
    e = cudaStreamCreateWithPriority(&ctx->side64, cudaStreamNonBlocking, prio_least);
  }
  if (e == cudaSuccess) {
    e = cudaStreamCreateWithPriority(&ctx->pre, cudaStreamNonBlocking, prio_least);
  }
  // the solve graph's main chain sits between the two side streams
  if (e == cudaSuccess) {
    e = cudaStreamCreateWithPriority(&ctx->cap, cudaStreamNonBlocking,
                                     (prio_least + prio_greatest) / 2);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_loop0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_loop1);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_blue, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join64, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_fork_l, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join_l, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join_m, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_plan_p, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join_p, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->tw32, sizeof(float2) * kTwiddleEntries);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->tw64, sizeof(double2) * kTwiddleEntries);
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return MPSFT_ERR_CUDA;
  }
  ctx->stream = ctx->own;
  if (!(WindowKernelsLaunchable() && FftKernelsLaunchable() &&
        DecideKernelsLaunchable() && RebinKernelsLaunchable() &&
        ControlKernelsLaunchable())) {
    cudaGetLastError();
    mpsft_ctx_destroy(ctx);
    return MPSFT_ERR_CUDA;
  }
  LaunchTwiddles(ctx->tw32, ctx->tw64, ctx->stream);
  e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    mpsft_ctx_destroy(ctx);
    return MPSFT_ERR_CUDA;
  }
  *out = ctx;
  return MPSFT_OK;
}

int mpsft_ctx_destroy(mpsft_ctx *ctx) {
  if (!ctx) return MPSFT_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (cudaEvent_t e : ctx->events) cudaEventDestroy(e);
  if (ctx->arena) cudaFree(ctx->arena);
  if (ctx->h_ctl) cudaFreeHost(ctx->h_ctl);
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  if (ctx->h_up) cudaFreeHost(ctx->h_up);
  if (ctx->tw32) cudaFree(ctx->tw32);
  if (ctx->tw64) cudaFree(ctx->tw64);
  if (ctx->win_dev) cudaFree(ctx->win_dev);
  if (ctx->ph_cache) cudaFree(ctx->ph_cache);
  if (ctx->side64) {
    cudaStreamSynchronize(ctx->side64);
    cudaStreamDestroy(ctx->side64);
  }
  if (ctx->side) {
    cudaStreamSynchronize(ctx->side);
    cudaStreamDestroy(ctx->side);
  }
  if (ctx->pre) {
    cudaStreamSynchronize(ctx->pre);
    cudaStreamDestroy(ctx->pre);
  }
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  if (ctx->cap) cudaStreamDestroy(ctx->cap);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_loop0) cudaEventDestroy(ctx->ev_loop0);
  if (ctx->ev_loop1) cudaEventDestroy(ctx->ev_loop1);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->ev_blue) cudaEventDestroy(ctx->ev_blue);
  if (ctx->ev_join64) cudaEventDestroy(ctx->ev_join64);
  if (ctx->ev_fork_l) cudaEventDestroy(ctx->ev_fork_l);
  if (ctx->ev_join_l) cudaEventDestroy(ctx->ev_join_l);
  if (ctx->ev_join_m) cudaEventDestroy(ctx->ev_join_m);
  if (ctx->ev_plan_p) cudaEventDestroy(ctx->ev_plan_p);
  if (ctx->ev_join_p) cudaEventDestroy(ctx->ev_join_p);
  if (ctx->own) cudaStreamDestroy(ctx->own);
  delete ctx;
  return MPSFT_OK;
}

int mpsft_ctx_set_stream(mpsft_ctx *ctx, void *stream) {
  if (!ctx) return MPSFT_ERR_INVALID;
  ctx->stream = stream ? reinterpret_cast<cudaStream_t>(stream) : ctx->own;
  return MPSFT_OK;
}

int mpsft_ctx_set_profiling(mpsft_ctx *ctx, int enable) {
  if (!ctx) return MPSFT_ERR_INVALID;
  ctx->profiling = enable != 0;
  return MPSFT_OK;
}

int mpsft_ctx_bin_launches(const mpsft_ctx *ctx, mpsft_bin_launch *out,
                           int32_t cap, int32_t *count) {
  if (!ctx || !count || (cap > 0 && !out)) return MPSFT_ERR_INVALID;
  const int32_t total = int32_t(ctx->bin_launches.size());
  for (int32_t j = 0; j < total && j < cap; ++j) out[j] = ctx->bin_launches[j];
  *count = total;
  return MPSFT_OK;
}

const char *mpsft_last_error(const mpsft_ctx *ctx) {
  return ctx ? ctx->err.c_str() : "null context";
}

int mpsft_rng_create(int32_t seed, mpsft_rng **out) {
  if (!out) return MPSFT_ERR_INVALID;
  *out = new mpsft_rng;
  (*out)->Seed(seed);
  return MPSFT_OK;
}
int mpsft_rng_destroy(mpsft_rng *rng) {
  delete rng;
  return MPSFT_OK;
}
int mpsft_rng_seed(mpsft_rng *rng, int32_t seed) {
  if (!rng) return MPSFT_ERR_INVALID;
  // RandomSeed (src/base.cc:52) reseeds the engine only: a normal draw the
  // distribution holds back (the second of a pair) survives the reseed
  rng->Seed(seed);
  return MPSFT_OK;
}
int mpsft_rng_seed_many(mpsft_rng *const *rngs, const int32_t *seeds,
                        int32_t count) {
  if (count < 0 || (count > 0 && (!rngs || !seeds))) return MPSFT_ERR_INVALID;
  for (int32_t i = 0; i < count; ++i) {
    if (!rngs[i]) return MPSFT_ERR_INVALID;
  }
  for (int32_t i = 0; i < count; ++i) rngs[i]->Seed(seeds[i]);
  return MPSFT_OK;
}
int32_t mpsft_rng_int32(mpsft_rng *rng) { return rng ? rng->Draw() : -1; }

int mpsft_rng_normals(mpsft_rng *rng, int64_t count, double *out) {
  if (!rng || count < 0) return MPSFT_ERR_INVALID;
  for (int64_t i = 0; i < count; ++i) {
    const double v = rng->Normal();
    if (out) out[i] = v;
  }
  return MPSFT_OK;
}

int32_t mpsft_num_bits(int32_t n, int32_t bins) {
  return bins > 0 ? NumBits(n, bins) : 0;
}

int32_t mpsft_window_support(int32_t n, int32_t bins, double delta) {
  (void)n;
  if (bins <= 0 || bins % 2 == 0 || !(delta > 0 && delta < 1)) return 0;
  return MakeWindow(bins, delta).p;
}

void mpsft_solve_options_default(mpsft_solve_options *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->trials = 1;
  o->min_bins = 101;
  o->window_delta = 1e-6;
  o->window_threshold = 0.1;
  o->max_stale_iter = 3;
  o->precision = MPSFT_PREC_FP32;
}

int mpsft_signal_upload(mpsft_ctx *ctx, const void *x_host, int64_t n,
                        int dtype, mpsft_signal **out) {
  if (!ctx || !x_host || !out) return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  if (dtype != MPSFT_C64 && dtype != MPSFT_C128) {
    return Fail(ctx, MPSFT_ERR_INVALID, "dtype must be MPSFT_C64 or MPSFT_C128");
  }
  int rc = CheckN(ctx, n);
  if (rc) return rc;
  const size_t bytes = size_t(n) * (dtype == MPSFT_C64 ? 8 : 16);
  mpsft_signal *s = new mpsft_signal;
  s->ctx = ctx;
  s->n = n;
  s->dtype = dtype;
  s->owned = true;
  if (cudaMalloc(&s->d_x, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete s;
    return Fail(ctx, MPSFT_ERR_NOMEM, "device allocation of the signal failed");
  }
  cudaError_t e = cudaMemcpyAsync(s->d_x, x_host, bytes, cudaMemcpyHostToDevice,
                                  ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(s->d_x);
    delete s;
    return Fail(ctx, MPSFT_ERR_CUDA, cudaGetErrorString(e));
  }
  *out = s;
  return MPSFT_OK;
}

int mpsft_signal_wrap_device(mpsft_ctx *ctx, const void *x_device, int64_t n,
                             int dtype, mpsft_signal **out) {
  if (!ctx || !x_device || !out) return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  if (dtype != MPSFT_C64 && dtype != MPSFT_C128) {
    return Fail(ctx, MPSFT_ERR_INVALID, "dtype must be MPSFT_C64 or MPSFT_C128");
  }
  int rc = CheckN(ctx, n);
  if (rc) return rc;
  mpsft_signal *s = new mpsft_signal;
  s->ctx = ctx;
  s->n = n;
  s->dtype = dtype;
  s->owned = false;
  s->d_x = const_cast<void *>(x_device);
  *out = s;
  return MPSFT_OK;
}

int mpsft_signal_free(mpsft_signal *sig) {
  if (!sig) return MPSFT_OK;
  if (sig->owned && sig->d_x) {
    if (sig->ctx) cudaStreamSynchronize(sig->ctx->stream);
    cudaFree(sig->d_x);
  }
  delete sig;
  return MPSFT_OK;
}

int mpsft_signal_write(mpsft_ctx *ctx, mpsft_signal *sig, const void *x_host) {
  if (!ctx || !sig || !x_host) return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  if (sig->ctx != ctx) {
    return Fail(ctx, MPSFT_ERR_INVALID, "signal belongs to another context");
  }
  const size_t bytes = size_t(sig->n) * (sig->dtype == MPSFT_C64 ? 8 : 16);
  MPSFT_CUDA(ctx, cudaMemcpyAsync(sig->d_x, x_host, bytes, cudaMemcpyHostToDevice,
                                  ctx->stream));
  return MPSFT_OK;
}

int mpsft_signal_read(mpsft_ctx *ctx, const mpsft_signal *sig, void *x_host) {
  if (!ctx || !sig || !x_host) return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  if (sig->ctx != ctx) {
    return Fail(ctx, MPSFT_ERR_INVALID, "signal belongs to another context");
  }
  const size_t bytes = size_t(sig->n) * (sig->dtype == MPSFT_C64 ? 8 : 16);
  MPSFT_CUDA(ctx, cudaMemcpyAsync(x_host, sig->d_x, bytes, cudaMemcpyDeviceToHost,
                                  ctx->stream));
  MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MPSFT_OK;
}

int mpsft_signal_write_many(mpsft_ctx *ctx, mpsft_signal *const *sigs,
                            const void *const *x_host, int32_t count,
                            void *stream) {
  if (!ctx || count < 0 || (count > 0 && (!sigs || !x_host))) {
    return MPSFT_ERR_INVALID;
  }
  for (int32_t i = 0; i < count; ++i) {
    if (!sigs[i] || !x_host[i] || sigs[i]->ctx != ctx) return MPSFT_ERR_INVALID;
  }
  // the calling thread may not have selected the context's device
  if (cudaSetDevice(ctx->device) != cudaSuccess) {
    cudaGetLastError();
    return MPSFT_ERR_CUDA;
  }
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  for (int32_t i = 0; i < count; ++i) {
    const mpsft_signal *sig = sigs[i];
    const size_t bytes = size_t(sig->n) * (sig->dtype == MPSFT_C64 ? 8 : 16);
    if (cudaMemcpyAsync(sig->d_x, x_host[i], bytes, cudaMemcpyHostToDevice, st) !=
        cudaSuccess) {
      cudaGetLastError();
      return MPSFT_ERR_CUDA;
    }
  }
  return MPSFT_OK;
}

int mpsft_window_table(mpsft_ctx *ctx, int32_t n, int32_t bins, double delta,
                       double *wt_host, int32_t cap) {
  if (!ctx || !wt_host) return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  int rc = CheckWindow(ctx, bins, delta, false);
  if (rc) return rc;
  const WinParams w = MakeWindow(bins, delta);
  if (cap < w.p) return Fail(ctx, MPSFT_ERR_CAPACITY, "wt buffer smaller than p");
  Shape s;
  s.n = n;
  s.bins_cap = bins;
  s.rows_cap = 1;
  s.p2_cap = w.p2;
  s.m_cap = 1 << FFTLog2(bins);
  s.tab_cap = 64;
  Carve probe{nullptr};
  SigIter it{};
  int32_t *ctl;
  CarveSignal(probe, s, &it, &ctl);
  rc = EnsureArena(ctx, probe.off + sizeof(SigIter) + 512);
  if (rc) return rc;
  Carve cv{ctx->arena};
  SigIter *d_it = cv.take<SigIter>(1);
  std::memset(&it, 0, sizeof(it));
  CarveSignal(cv, s, &it, &ctl);
  it.active = 1;
  it.n = n;
  it.bins = bins;
  it.p = w.p;
  it.p2 = w.p2;
  it.width = w.width;
  it.sigma_f = w.sigma_f;
  MPSFT_CUDA(ctx, cudaMemcpyAsync(d_it, &it, sizeof(it), cudaMemcpyHostToDevice,
                                  ctx->stream));
  LaunchWindow(d_it, 1, w.p2, ctx->stream);
  std::vector<double> half(w.p2 + 1);
  MPSFT_CUDA(ctx, cudaMemcpyAsync(half.data(), it.wt64,
                                  sizeof(double) * (w.p2 + 1),
                                  cudaMemcpyDeviceToHost, ctx->stream));
  MPSFT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int32_t i = 0; i < w.p; ++i) {
    const int32_t t = i <= w.p2 ? i : i - w.p;
    wt_host[i] = half[t < 0 ? -t : t];
  }
  return MPSFT_OK;
}

}  // extern "C"

namespace {

// A caller's window table (the reference's Window::wt(), src/window.h:32,
// filled by src/window.cc:65-69): p entries for t = 0, 1..p2, -p2..-1, p an
// odd multiple of bins, even in t (the kernels read it at |t|), finite.
int CheckWindowTable(mpsft_ctx *ctx, int32_t bins, int32_t p, const double *wt,
                     bool fp64) {
  if (bins <= 0 || bins % 2 == 0) {
    return Fail(ctx, MPSFT_ERR_INVALID, "bins must be odd and positive");
  }
  if (p <= 0 || p % 2 == 0 || p % bins != 0) {
    return Fail(ctx, MPSFT_ERR_INVALID, "p must be an odd multiple of bins");
  }
  if (p / bins > kFoldLanes * kMaxFoldsPerLane) {
    return Fail(ctx, MPSFT_ERR_INVALID, "window too wide (p/bins > 80)");
  }
  const int32_t p2 = (p - 1) / 2;
  for (int32_t i = 0; i <= p2; ++i) {
    if (!std::isfinite(wt[i])) {
      return Fail(ctx, MPSFT_ERR_INVALID, "window table must be finite");
    }
    if (i > 0 && wt[p - i] != wt[i]) {
      return Fail(ctx, MPSFT_ERR_INVALID,
                  "window table must be even (wt[p - i] == wt[i])");
    }
  }
  const int m = 1 << FFTLog2(bins);
  if (m > (fp64 ? kMaxFFT64 : kMaxFFT)) {
    return Fail(ctx, MPSFT_ERR_INVALID,
                fp64 ? "bins too large for the FP64 path (max 4096)"
                     : "bins too large (max 8192)");
  }
  return MPSFT_OK;
}

// The window scalars a binning call needs from a caller's table: the support
// and the width (wt[0] = 1 / (2 bins), src/window.cc:65).
WinParams TableWindow(int32_t bins, int32_t p, const double *wt) {
  WinParams w;
  w.p = p;
  w.p2 = (p - 1) / 2;
  w.folds = p / bins;
  w.width = wt[0];
  return w;
}

// Copies the t >= 0 half of a caller's window table into it's device tables:
// FP64 as given, FP32 rounded, float-float (hi, lo) split; waits for the
// copies (pageable staging).
int UploadWindowTable(mpsft_ctx *ctx, const SigIter &it, const double *wt,
                      cudaStream_t st) {
  const size_t e = size_t(it.p2) + 1;
  std::vector<float> w32(e);
  std::vector<float2> wff(e);
  for (size_t i = 0; i < e; ++i) {
    const float hi = float(wt[i]);
    w32[i] = hi;
    wff[i] = make_float2(hi, float(wt[i] - double(hi)));
  }
  MPSFT_CUDA(ctx, cudaMemcpyAsync(it.wt64, wt, sizeof(double) * e,
                                  cudaMemcpyHostToDevice, st));
  MPSFT_CUDA(ctx, cudaMemcpyAsync(it.wt32, w32.data(), sizeof(float) * e,
                                  cudaMemcpyHostToDevice, st));
  MPSFT_CUDA(ctx, cudaMemcpyAsync(it.wtff, wff.data(), sizeof(float2) * e,
                                  cudaMemcpyHostToDevice, st));
  MPSFT_CUDA(ctx, cudaStreamSynchronize(st));
  return MPSFT_OK;
}

// BinInTime::Run over a window evaluated on the device from delta (wt null)
// or given by the caller as the reference's table (wt: p entries, index order
// t = 0, 1..p2, -p2..-1).
int BinInTimeImpl(mpsft_ctx *ctx, const mpsft_signal *sig, int32_t bins,
                  int32_t bits, double delta, int32_t p, const double *wt,
                  int32_t a, int32_t b, int32_t c, int32_t q, int precision,
                  double *out, int out_on_device) {
  if (!ctx || !out) return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  int rc = CheckSignal(ctx, sig);
  if (rc) return rc;
  const bool fp64 = precision != MPSFT_PREC_FP32;
  if (precision < MPSFT_PREC_FP32 || precision > MPSFT_PREC_FP64_DIRECT) {
    return Fail(ctx, MPSFT_ERR_INVALID, "unknown precision");
  }
  WinParams w;
  if (wt) {
    rc = CheckWindowTable(ctx, bins, p, wt, fp64);
    if (rc) return rc;
    w = TableWindow(bins, p, wt);
  } else {
    rc = CheckWindow(ctx, bins, delta, fp64);
    if (rc) return rc;
    w = MakeWindow(bins, delta);
  }
  if (bits < 0 || bits > kMaxBits) {
    return Fail(ctx, MPSFT_ERR_INVALID, "bits must be in [0, 31]");
  }
  if (int64_t(bins) << (bits > 0 ? bits - 1 : 0) > INT32_MAX) {
    return Fail(ctx, MPSFT_ERR_INVALID, "bins * 2^(bits-1) overflows int32");
  }
  const int32_t n = int32_t(sig->n);
  const bool direct = precision == MPSFT_PREC_FP64_DIRECT;
  Shape s;
  s.n = n;
  s.bins_cap = bins;
  s.rows_cap = 1 + 2 * bits;
  s.trials = 1;
  s.p2_cap = w.p2;
  s.m_cap = 1 << FFTLog2(bins);
  s.tab_cap = 64;
  s.fp64 = fp64;
  Carve probe{nullptr};
  SigIter it{};
  int32_t *ctl;
  CarveSignal(probe, s, &it, &ctl);
  const size_t direct_cells = direct ? size_t(bins) * s.rows_cap * kRebinChunks : 0;
  rc = EnsureArena(ctx, probe.off + sizeof(SigIter) + 1024 +
                            direct_cells * sizeof(double2) +
                            (direct ? (2 * sizeof(int32_t) + sizeof(double2) +
                                       64 * sizeof(float4)) * size_t(bins) +
                                          (sizeof(double2) + sizeof(int32_t)) *
                                              (direct_cells / kRebinChunks) + 2304
                                    : 0));
  if (rc) return rc;
  Carve cv{ctx->arena};
  SigIter *d_it = cv.take<SigIter>(1);
  std::memset(&it, 0, sizeof(it));
  CarveSignal(cv, s, &it, &ctl);
  const Transform tf{a, b, c, InverseMod(a, n)};
  FillIter(&it, sig, bins, bits, w, tf, &q, 1);
  cudaStream_t st = ctx->stream;
  // the window tables: evaluated on the device, or the caller's uploaded
  auto window = [&](bool all64) -> int {
    if (wt) return UploadWindowTable(ctx, it, wt, st);
    if (all64) {
      LaunchWindow(d_it, 1, it.p2, st);
    } else {
      LaunchWindow32(d_it, 1, it.p2, st);
    }
    return MPSFT_OK;
  };
  if (direct) {
    // every bin is a listed bin of the FP64 re-binning kernel
    it.esc_part = cv.take<double2>(direct_cells);
    it.esc_sum = cv.take<double2>(direct_cells / kRebinChunks);
    it.esc_cnt = cv.take<int32_t>(direct_cells / kRebinChunks);
    it.esc_list = cv.take<int32_t>(bins);
    it.esc_pow = cv.take<float4>(size_t(bins) * 64);
    it.esc_step = cv.take<double2>(bins);
    it.esc_mask = nullptr;  // every row of every bin
    it.esc_cap = bins;
    std::vector<int32_t> iota(bins);
    for (int32_t i = 0; i < bins; ++i) iota[i] = i;
    MPSFT_CUDA(ctx, cudaMemcpyAsync(it.esc_list, iota.data(),
                                    sizeof(int32_t) * bins,
                                    cudaMemcpyHostToDevice, st));
    const int32_t h_flags[kCtlWords] = {0, 0, bins, 0};
    MPSFT_CUDA(ctx, cudaMemcpyAsync(ctl, h_flags, sizeof(h_flags),
                                    cudaMemcpyHostToDevice, st));
    MPSFT_CUDA(ctx, cudaMemcpyAsync(d_it, &it, sizeof(it), cudaMemcpyHostToDevice,
                                    st));
    rc = window(true);
    if (rc) return rc;
    LaunchRebin(d_it, 1, bins, sig->dtype == MPSFT_C128, true, st);
    MPSFT_CUDA(ctx, cudaGetLastError());
    std::vector<double2> sum(direct_cells / kRebinChunks);
    MPSFT_CUDA(ctx, cudaMemcpyAsync(sum.data(), it.esc_sum,
                                    sizeof(double2) * sum.size(),
                                    cudaMemcpyDeviceToHost, st));
    MPSFT_CUDA(ctx, cudaStreamSynchronize(st));
    std::vector<double2> res(size_t(it.rows) * bins);
    for (int32_t bb = 0; bb < bins; ++bb) {
      for (int32_t r = 0; r < it.rows; ++r) {
        res[size_t(r) * bins + bb] = sum[size_t(bb) * it.rows + r];
      }
    }
    MPSFT_CUDA(ctx, cudaMemcpy(out, res.data(), sizeof(double2) * res.size(),
                               out_on_device ? cudaMemcpyHostToDevice
                                             : cudaMemcpyHostToHost));
    return MPSFT_OK;
  }
  MPSFT_CUDA(ctx, cudaMemcpyAsync(d_it, &it, sizeof(it), cudaMemcpyHostToDevice,
                                  ctx->stream));
  // the window the solves use: FP64 for the FP64 path, FP32-evaluated for
  // FP32 (a caller's table: as given, and rounded to FP32)
  rc = window(fp64);
  if (rc) return rc;
  LaunchBluesteinSetup(d_it, 1, it.fft_m, fp64, ctx->tw32, ctx->tw64, st);
  BinTimer timer{ctx};
  rc = timer.Begin();
  if (rc) return rc;
  LaunchBinFold(d_it, 1, bins, bits, 1, sig->dtype == MPSFT_C128, fp64, st, false,
                FoldShapeFor(ctx, bins, sig->n, 1, sig->dtype == MPSFT_C128));
  rc = timer.End();
  if (rc) return rc;
  LaunchRowFFT(d_it, 1, it.rows, 1, it.fft_m, fp64, ctx->tw32, ctx->tw64, st);
  MPSFT_CUDA(ctx, cudaGetLastError());
  const size_t row_bytes = sizeof(double2) * size_t(bins);
  MPSFT_CUDA(ctx, cudaMemcpy2DAsync(
                      out, row_bytes, it.ubuf, sizeof(double2) * it.bins_cap,
                      row_bytes, it.rows,
                      out_on_device ? cudaMemcpyDeviceToDevice
                                    : cudaMemcpyDeviceToHost,
                      st));
  MPSFT_CUDA(ctx, cudaStreamSynchronize(st));
  if (ctx->profiling) {
    mpsft_bin_launch rec{};
    rec.signals = 1;
    rec.max_bins = rec.min_bins = bins;
    rec.precision = fp64 ? MPSFT_PREC_FP64 : MPSFT_PREC_FP32;
    rec.gathers = BinGathers(it, fp64);
    rec.bytes = BinBytes(it, fp64);
    rec.ms = timer.TotalMs();
    ctx->bin_launches.assign(1, rec);
  }
  return MPSFT_OK;
}

// BinInFreq::Run: subtracts the modes' window responses from a host bin
// matrix. wf null: responses evaluated on the device from delta; otherwise
// wf[i] is mode i's response (the caller's Window::SampleInFreq), folded into
// its coefficient here as the reference's wf * coef.
int BinInFreqImpl(mpsft_ctx *ctx, int32_t n, int32_t bins, int32_t bits,
                  double delta, int32_t a, int32_t b, int32_t c, int32_t q,
                  const int32_t *k0, const double *coef, const double *wf,
                  int64_t m, double *inout) {
  if (!ctx || !inout || (m > 0 && (!k0 || !coef))) {
    return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  }
  int rc = CheckN(ctx, n);
  if (rc) return rc;
  if (wf) {
    if (bins <= 0 || bins % 2 == 0) {
      return Fail(ctx, MPSFT_ERR_INVALID, "bins must be odd and positive");
    }
    for (int64_t i = 0; i < m; ++i) {
      if (!std::isfinite(wf[i])) {
        return Fail(ctx, MPSFT_ERR_INVALID, "window responses must be finite");
      }
    }
  } else {
    rc = CheckWindow(ctx, bins, delta, false);
    if (rc) return rc;
  }
  if (bits < 0 || bits > kMaxBits || m < 0) {
    return Fail(ctx, MPSFT_ERR_INVALID, "bad bits or mode count");
  }
  Shape s;
  s.n = n;
  s.bins_cap = bins;
  s.rows_cap = 1 + 2 * bits;
  s.trials = 1;
  s.p2_cap = 1;
  s.m_cap = 1;
  s.tab_cap = NextPow2(std::max<int64_t>(64, 2 * m));
  if (s.tab_cap > kMaxTableCap) {
    return Fail(ctx, MPSFT_ERR_CAPACITY, "too many modes");
  }
  Carve probe{nullptr};
  SigIter it{};
  int32_t *ctl;
  CarveSignal(probe, s, &it, &ctl);
  const size_t extra = size_t(m) * (sizeof(int32_t) + sizeof(double2)) + 1024;
  rc = EnsureArena(ctx, probe.off + sizeof(SigIter) + extra);
  if (rc) return rc;
  Carve cv{ctx->arena};
  SigIter *d_it = cv.take<SigIter>(1);
  std::memset(&it, 0, sizeof(it));
  CarveSignal(cv, s, &it, &ctl);
  int32_t *d_k0 = cv.take<int32_t>(size_t(m));
  double2 *d_coef = cv.take<double2>(size_t(m));
  const Transform tf{a, b, c, 0};
  mpsft_signal fake;
  fake.n = n;
  // the window's scalars serve only the device's responses
  FillIter(&it, &fake, bins, bits, wf ? WinParams{} : MakeWindow(bins, delta),
           tf, &q, 1);
  it.x = nullptr;
  it.unit_wf = wf ? 1 : 0;
  cudaStream_t st = ctx->stream;
  MPSFT_CUDA(ctx, cudaMemcpyAsync(d_it, &it, sizeof(it), cudaMemcpyHostToDevice,
                                  st));
  LaunchPhaseTables(d_it, 1, PhaseTableEntries(n), st);
  rc = ClearTable(ctx, it, ctl);
  if (rc) return rc;
  if (m > 0) {
    MPSFT_CUDA(ctx, cudaMemcpyAsync(d_k0, k0, sizeof(int32_t) * m,
                                    cudaMemcpyHostToDevice, st));
    std::vector<double> wc;
    const double *src = coef;
    if (wf) {
      // wf * coef, the reference's first product (src/binner.cc:580)
      wc.resize(2 * size_t(m));
      for (int64_t i = 0; i < m; ++i) {
        wc[2 * i] = coef[2 * i] * wf[i];
        wc[2 * i + 1] = coef[2 * i + 1] * wf[i];
      }
      src = wc.data();
    }
    MPSFT_CUDA(ctx, cudaMemcpyAsync(d_coef, src, sizeof(double2) * m,
                                    cudaMemcpyHostToDevice, st));
    LaunchTableInsert(d_it, d_k0, d_coef, m, st);
    // the pageable source must outlive the copy
    if (wf) MPSFT_CUDA(ctx, cudaStreamSynchronize(st));
  }
  const size_t row_bytes = sizeof(double2) * size_t(bins);
  MPSFT_CUDA(ctx, cudaMemcpy2DAsync(it.ubuf, sizeof(double2) * it.bins_cap,
                                    inout, row_bytes, row_bytes, it.rows,
                                    cudaMemcpyHostToDevice, st));
  LaunchBucket(d_it, 1, bins, s.tab_cap, st, true);
  LaunchDecide(d_it, 1, bins, 1, false, true, st);
  MPSFT_CUDA(ctx, cudaGetLastError());
  MPSFT_CUDA(ctx, cudaMemcpy2DAsync(inout, row_bytes, it.ubuf,
                                    sizeof(double2) * it.bins_cap, row_bytes,
                                    it.rows, cudaMemcpyDeviceToHost, st));
  int32_t h_ctl[kCtlWords];
  MPSFT_CUDA(ctx, cudaMemcpyAsync(h_ctl, ctl, sizeof(h_ctl),
                                  cudaMemcpyDeviceToHost, st));
  MPSFT_CUDA(ctx, cudaStreamSynchronize(st));
  if (h_ctl[1] & kStatusCapacity) {
    return Fail(ctx, MPSFT_ERR_CAPACITY, "mode table full");
  }
  return MPSFT_OK;
}

}  // namespace

extern "C" {

int mpsft_bin_in_time(mpsft_ctx *ctx, const mpsft_signal *sig, int32_t bins,
                      int32_t bits, double delta, int32_t a, int32_t b,
                      int32_t c, int32_t q, int precision, double *out,
                      int out_on_device) {
  return BinInTimeImpl(ctx, sig, bins, bits, delta, 0, nullptr, a, b, c, q,
                       precision, out, out_on_device);
}

int mpsft_bin_in_time_wt(mpsft_ctx *ctx, const mpsft_signal *sig, int32_t bins,
                         int32_t bits, int32_t p, const double *wt, int32_t a,
                         int32_t b, int32_t c, int32_t q, int precision,
                         double *out, int out_on_device) {
  if (!wt) return Fail(ctx, MPSFT_ERR_INVALID, "null window table");
  return BinInTimeImpl(ctx, sig, bins, bits, 0.0, p, wt, a, b, c, q, precision,
                       out, out_on_device);
}

int mpsft_bin_in_freq(mpsft_ctx *ctx, int32_t n, int32_t bins, int32_t bits,
                      double delta, int32_t a, int32_t b, int32_t c, int32_t q,
                      const int32_t *k0, const double *coef, int64_t m,
                      double *inout) {
  return BinInFreqImpl(ctx, n, bins, bits, delta, a, b, c, q, k0, coef, nullptr,
                       m, inout);
}

int mpsft_bin_in_freq_wf(mpsft_ctx *ctx, int32_t n, int32_t bins, int32_t bits,
                         int32_t a, int32_t b, int32_t c, int32_t q,
                         const int32_t *k0, const double *coef, const double *wf,
                         int64_t m, double *inout) {
  if (m > 0 && !wf) return Fail(ctx, MPSFT_ERR_INVALID, "null window responses");
  static const double kNone = 0.0;
  return BinInFreqImpl(ctx, n, bins, bits, 0.0, a, b, c, q, k0, coef,
                       wf ? wf : &kNone, m, inout);
}

}  // extern "C"

namespace {

// Shared setup of mpsft_estimate / mpsft_adjoint: validates, carves one
// signal's buffers plus `extra` bytes, fills and uploads the descriptor, and
// builds the FP64 window, Bluestein and unit-phase tables.
int EstimateSetup(mpsft_ctx *ctx, int32_t n, const void *x,
                  const mpsft_estimate_setup *su, size_t extra, Carve *cv,
                  SigIter *it, SigIter **d_it) {
  if (!su) return Fail(ctx, MPSFT_ERR_INVALID, "null setup");
  int rc = CheckN(ctx, n);
  if (rc) return rc;
  rc = CheckWindow(ctx, su->bins, su->window_delta, true);
  if (rc) return rc;
  if (su->bits < 0 || su->bits > kMaxBits || su->trials < 1 ||
      su->trials > kMaxTrials) {
    return Fail(ctx, MPSFT_ERR_INVALID, "bad bits or trials");
  }
  if (int64_t(su->bins) << (su->bits > 0 ? su->bits - 1 : 0) > INT32_MAX) {
    return Fail(ctx, MPSFT_ERR_INVALID, "bins * 2^(bits-1) overflows int32");
  }
  Shape s;
  s.n = n;
  s.bins_cap = su->bins;
  s.rows_cap = 1 + 2 * su->bits;
  s.trials = su->trials;
  s.p2_cap = MakeWindow(su->bins, su->window_delta).p2;
  s.m_cap = 1 << FFTLog2(su->bins);
  s.tab_cap = 64;
  s.fp64 = true;
  Carve probe{nullptr};
  SigIter tmp{};
  int32_t *ctl;
  CarveSignal(probe, s, &tmp, &ctl);
  rc = EnsureArena(ctx, probe.off + sizeof(SigIter) + extra + 4096);
  if (rc) return rc;
  *cv = Carve{ctx->arena};
  *d_it = cv->take<SigIter>(1);
  std::memset(it, 0, sizeof(*it));
  CarveSignal(*cv, s, it, &ctl);
  mpsft_signal fake{};
  fake.n = n;
  fake.d_x = const_cast<void *>(x);
  const Transform tf{su->a, su->b, su->c, 0};
  FillIter(it, &fake, su->bins, su->bits, su->window_delta, tf, su->q, su->trials);
  cudaStream_t st = ctx->stream;
  MPSFT_CUDA(ctx, cudaMemcpyAsync(*d_it, it, sizeof(SigIter),
                                  cudaMemcpyHostToDevice, st));
  LaunchPhaseTables(*d_it, 1, PhaseTableEntries(n), st);
  LaunchWindow(*d_it, 1, it->p2, st);
  LaunchBluesteinSetup(*d_it, 1, it->fft_m, true, ctx->tw32, ctx->tw64, st);
  MPSFT_CUDA(ctx, cudaGetLastError());
  return MPSFT_OK;
}

}  // namespace

namespace mpsft {
int CtxFail(mpsft_ctx *ctx, int code, const std::string &msg) {
  return Fail(ctx, code, msg);
}
int CtxCheckN(mpsft_ctx *ctx, int64_t n) { return CheckN(ctx, n); }
}  // namespace mpsft

extern "C" {

int mpsft_estimate(mpsft_ctx *ctx, const mpsft_signal *sig,
                   const mpsft_estimate_setup *setup, const int32_t *k0,
                   int64_t m, double *coef) {
  if (!ctx || (m > 0 && (!k0 || !coef)) || m < 0) {
    return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  }
  int rc = CheckSignal(ctx, sig);
  if (rc) return rc;
  Carve cv{nullptr};
  SigIter it;
  SigIter *d_it = nullptr;
  const size_t extra = size_t(m) * (sizeof(int32_t) + sizeof(double2)) + 1024;
  rc = EstimateSetup(ctx, int32_t(sig->n), sig->d_x, setup, extra, &cv, &it, &d_it);
  if (rc) return rc;
  int32_t *d_k0 = cv.take<int32_t>(size_t(m));
  double2 *d_coef = cv.take<double2>(size_t(m));
  cudaStream_t st = ctx->stream;
  LaunchBinFold(d_it, 1, it.bins, it.bits, it.trials, sig->dtype == MPSFT_C128,
                true, st);
  LaunchRowFFT(d_it, 1, it.rows, it.trials, it.fft_m, true, ctx->tw32, ctx->tw64,
               st);
  if (m > 0) {
    MPSFT_CUDA(ctx, cudaMemcpyAsync(d_k0, k0, sizeof(int32_t) * m,
                                    cudaMemcpyHostToDevice, st));
    LaunchEstimate(d_it, d_k0, m, d_coef, st);
  }
  MPSFT_CUDA(ctx, cudaGetLastError());
  if (m > 0) {
    MPSFT_CUDA(ctx, cudaMemcpyAsync(coef, d_coef, sizeof(double2) * m,
                                    cudaMemcpyDeviceToHost, st));
  }
  MPSFT_CUDA(ctx, cudaStreamSynchronize(st));
  return MPSFT_OK;
}

int mpsft_adjoint(mpsft_ctx *ctx, int32_t n, const mpsft_estimate_setup *setup,
                  const int32_t *k0, int64_t m, const double *g, double *dx) {
  if (!ctx || !dx || (m > 0 && (!k0 || !g)) || m < 0) {
    return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  }
  Carve cv{nullptr};
  SigIter it;
  SigIter *d_it = nullptr;
  const size_t extra = size_t(m) * (sizeof(int32_t) + sizeof(double2)) +
                       sizeof(double2) * size_t(n) + 1024;
  int rc = EstimateSetup(ctx, n, nullptr, setup, extra, &cv, &it, &d_it);
  if (rc) return rc;
  int32_t *d_k0 = cv.take<int32_t>(size_t(m));
  double2 *d_g = cv.take<double2>(size_t(m));
  double2 *d_dx = cv.take<double2>(size_t(n));
  cudaStream_t st = ctx->stream;
  const int64_t cells = int64_t(it.trials) * it.rows * it.bins_cap;
  MPSFT_CUDA(ctx, cudaMemsetAsync(it.fold, 0, sizeof(double2) * cells, st));
  MPSFT_CUDA(ctx, cudaMemsetAsync(d_dx, 0, sizeof(double2) * size_t(n), st));
  if (m > 0) {
    MPSFT_CUDA(ctx, cudaMemcpyAsync(d_k0, k0, sizeof(int32_t) * m,
                                    cudaMemcpyHostToDevice, st));
    MPSFT_CUDA(ctx, cudaMemcpyAsync(d_g, g, sizeof(double2) * m,
                                    cudaMemcpyHostToDevice, st));
  }
  LaunchAdjointSpread(d_it, d_k0, d_g, m, st);
  // inverse DFT of every row as conj(DFT(conj(G))): the row transform with
  // unit row factors
  for (int t = 0; t < it.trials; ++t) {
    it.bq_re[t] = 1.0;
    it.bq_im[t] = 0.0;
  }
  MPSFT_CUDA(ctx, cudaMemcpyAsync(d_it, &it, sizeof(SigIter),
                                  cudaMemcpyHostToDevice, st));
  LaunchRowFFT(d_it, 1, it.rows, it.trials, it.fft_m, true, ctx->tw32, ctx->tw64,
               st);
  LaunchAdjointScatter(d_it, int64_t(it.trials) * it.rows * it.p, d_dx, st);
  MPSFT_CUDA(ctx, cudaGetLastError());
  MPSFT_CUDA(ctx, cudaMemcpyAsync(dx, d_dx, sizeof(double2) * size_t(n),
                                  cudaMemcpyDeviceToHost, st));
  MPSFT_CUDA(ctx, cudaStreamSynchronize(st));
  return MPSFT_OK;
}

int mpsft_mat_pencil(mpsft_ctx *ctx, const double *u3, int64_t count,
                     double *sigma, int32_t *vote) {
  if (!ctx || count < 0 || (count > 0 && (!u3 || !sigma || !vote))) {
    return Fail(ctx, MPSFT_ERR_INVALID, "bad argument");
  }
  if (count == 0) return MPSFT_OK;
  const size_t need = size_t(count) * (3 * sizeof(double2) + 2 * sizeof(double) +
                                       sizeof(int32_t)) + 1024;
  int rc = EnsureArena(ctx, need);
  if (rc) return rc;
  Carve cv{ctx->arena};
  double2 *d_u = cv.take<double2>(size_t(count) * 3);
  double *d_s = cv.take<double>(size_t(count) * 2);
  int32_t *d_v = cv.take<int32_t>(size_t(count));
  cudaStream_t st = ctx->stream;
  MPSFT_CUDA(ctx, cudaMemcpyAsync(d_u, u3, sizeof(double2) * 3 * count,
                                  cudaMemcpyHostToDevice, st));
  LaunchPencil(d_u, count, d_s, d_v, st);
  MPSFT_CUDA(ctx, cudaGetLastError());
  MPSFT_CUDA(ctx, cudaMemcpyAsync(sigma, d_s, sizeof(double) * 2 * count,
                                  cudaMemcpyDeviceToHost, st));
  MPSFT_CUDA(ctx, cudaMemcpyAsync(vote, d_v, sizeof(int32_t) * count,
                                  cudaMemcpyDeviceToHost, st));
  MPSFT_CUDA(ctx, cudaStreamSynchronize(st));
  return MPSFT_OK;
}

}  // extern "C"

namespace {

// One Iterate call for a transform and q's drawn by the caller (draw set:
// the draws come from rng after the argument checks, in the reference's
// order).
int IterateImpl(mpsft_ctx *ctx, const mpsft_signal *sig,
                const mpsft_iterate_options *opt, mpsft_rng *rng,
                const Transform *tf_in, const int32_t *q_in, int32_t *mm_k,
                double *mm_c, int32_t *mm_size, int32_t mm_cap, int32_t *found) {
  if (!ctx || !opt || (!rng && !(tf_in && q_in)) || !mm_size || !found ||
      (mm_cap > 0 && (!mm_k || !mm_c))) {
    return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  }
  int rc = CheckSignal(ctx, sig);
  if (rc) return rc;
  const bool fp64 = opt->precision == MPSFT_PREC_FP64;
  if (!(opt->window_threshold > 0)) {
    return Fail(ctx, MPSFT_ERR_INVALID, "window_threshold must be > 0");
  }
  if (opt->trials < 1 || opt->trials % 2 == 0 || opt->trials > kMaxTrials) {
    return Fail(ctx, MPSFT_ERR_INVALID, "trials must be odd and <= 15");
  }
  rc = CheckWindow(ctx, opt->bins, opt->window_delta, fp64);
  if (rc) return rc;
  if (*mm_size < 0 || *mm_size > mm_cap) {
    return Fail(ctx, MPSFT_ERR_INVALID, "mm_size out of range");
  }
  const int32_t n = int32_t(sig->n);
  const int32_t bins = opt->bins;
  const int32_t bits = NumBits(n, bins);
  Shape s;
  s.n = n;
  s.bins_cap = bins;
  s.rows_cap = 1 + 2 * bits;
  s.trials = opt->trials;
  s.p2_cap = MakeWindow(bins, opt->window_delta).p2;
  s.m_cap = 1 << FFTLog2(bins);
  s.tab_cap = NextPow2(std::max<int64_t>(64, 2 * (int64_t(*mm_size) + bins)));
  if (s.tab_cap > kMaxTableCap) {
    return Fail(ctx, MPSFT_ERR_CAPACITY, "mode map larger than the table");
  }
  s.fp64 = fp64;
  s.fp32_bins = !fp64;
  Carve probe{nullptr};
  SigIter it{};
  int32_t *ctl;
  CarveSignal(probe, s, &it, &ctl);
  const int64_t m0 = *mm_size;
  const size_t extra = size_t(m0) * (sizeof(int32_t) + sizeof(double2)) +
                       sizeof(double) * kEnergyStride + 2048;
  rc = EnsureArena(ctx, probe.off + sizeof(SigIter) + extra);
  if (rc) return rc;
  Carve cv{ctx->arena};
  SigIter *d_it = cv.take<SigIter>(1);
  std::memset(&it, 0, sizeof(it));
  CarveSignal(cv, s, &it, &ctl);
  int32_t *d_k0 = cv.take<int32_t>(size_t(m0));
  double2 *d_coef = cv.take<double2>(size_t(m0));
  double *d_energy = cv.take<double>(kEnergyStride);
  const void **d_xs = cv.take<const void *>(1);
  int64_t *d_ns = cv.take<int64_t>(1);
  Transform tf;
  int32_t q[kMaxTrials];
  if (tf_in) {
    tf = *tf_in;
    for (int t = 0; t < opt->trials; ++t) q[t] = q_in[t];
  } else {
    tf = DrawTransform(rng, n);
    for (int t = 0; t < opt->trials; ++t) q[t] = rng->Draw() % n;
  }
  FillIter(&it, sig, bins, bits, opt->window_delta, tf, q, opt->trials);
  it.bin_thr = opt->bin_threshold;
  it.sv_thr = opt->sv_threshold;
  SetThresholdCopies(&it);
  it.win_thr = opt->window_threshold;
  cudaStream_t st = ctx->stream;
  std::vector<double> energy(1, 0.0);
  if (!fp64) {
    const void *h_x = sig->d_x;
    const int64_t h_n = sig->n;
    MPSFT_CUDA(ctx, cudaMemcpyAsync(d_xs, &h_x, sizeof(h_x),
                                    cudaMemcpyHostToDevice, st));
    MPSFT_CUDA(ctx, cudaMemcpyAsync(d_ns, &h_n, sizeof(h_n),
                                    cudaMemcpyHostToDevice, st));
    LaunchEnergy(d_xs, d_ns, 1, sig->dtype == MPSFT_C128, d_energy, st, kPolicySample);
    rc = ReadEnergy(ctx, d_energy, 1, &energy);
    if (rc) return rc;
  }
  SetNearTie(&it, fp64, opt->near_tie_margin, bins,
             !fp64 && PolicyForcesFP64(opt->near_tie_margin, bins, energy[0],
                                       opt->bin_threshold, opt->sv_threshold));
  MPSFT_CUDA(ctx, cudaMemcpyAsync(d_it, &it, sizeof(it), cudaMemcpyHostToDevice,
                                  st));
  LaunchPhaseTables(d_it, 1, PhaseTableEntries(n), st);
  rc = ClearTable(ctx, it, ctl);
  if (rc) return rc;
  if (m0 > 0) {
    MPSFT_CUDA(ctx, cudaMemcpyAsync(d_k0, mm_k, sizeof(int32_t) * m0,
                                    cudaMemcpyHostToDevice, st));
    MPSFT_CUDA(ctx, cudaMemcpyAsync(d_coef, mm_c, sizeof(double2) * m0,
                                    cudaMemcpyHostToDevice, st));
    LaunchTableInsert(d_it, d_k0, d_coef, m0, st);
  }
  std::vector<SigIter> h_its(1, it);
  BinTimer timer{ctx};
  rc = LaunchIteration(ctx, d_it, 1, h_its, sig->dtype == MPSFT_C128, fp64,
                       &timer);
  if (rc) return rc;
  int32_t h_ctl[kCtlWords];
  MPSFT_CUDA(ctx, cudaMemcpyAsync(h_ctl, ctl, sizeof(h_ctl),
                                  cudaMemcpyDeviceToHost, st));
  MPSFT_CUDA(ctx, cudaStreamSynchronize(st));
  if (h_ctl[1] & kStatusCapacity) {
    return Fail(ctx, MPSFT_ERR_CAPACITY, "mode table full");
  }
  if (h_ctl[1] & kStatusNonFinite) {
    return Fail(ctx, MPSFT_ERR_NONFINITE, "non-finite values in the bins");
  }
  std::vector<std::pair<int32_t, double2>> modes;
  rc = DownloadTable(ctx, it, &modes);
  if (rc) return rc;
  if (int64_t(modes.size()) > mm_cap) {
    return Fail(ctx, MPSFT_ERR_CAPACITY, "mode map capacity too small");
  }
  for (size_t j = 0; j < modes.size(); ++j) {
    mm_k[j] = modes[j].first;
    mm_c[2 * j] = modes[j].second.x;
    mm_c[2 * j + 1] = modes[j].second.y;
  }
  *mm_size = int32_t(modes.size());
  *found = h_ctl[0] ? 1 : 0;
  return MPSFT_OK;
}

}  // namespace

extern "C" {

int mpsft_iterate(mpsft_ctx *ctx, const mpsft_signal *sig,
                  const mpsft_iterate_options *opt, mpsft_rng *rng,
                  int32_t *mm_k, double *mm_c, int32_t *mm_size,
                  int32_t mm_cap, int32_t *found) {
  if (!rng) return Fail(ctx, MPSFT_ERR_INVALID, "null rng");
  return IterateImpl(ctx, sig, opt, rng, nullptr, nullptr, mm_k, mm_c, mm_size,
                     mm_cap, found);
}

int mpsft_iterate_draws(mpsft_ctx *ctx, const mpsft_signal *sig,
                        const mpsft_iterate_options *opt, int32_t a, int32_t b,
                        int32_t c, int32_t a_inv, const int32_t *q,
                        int32_t *mm_k, double *mm_c, int32_t *mm_size,
                        int32_t mm_cap, int32_t *found) {
  if (!sig || !q) return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  const int64_t n = sig->n;
  if (a < 0 || a >= n || b < 0 || b >= n || c < 0 || c >= n || a_inv < 0 ||
      a_inv >= n) {
    return Fail(ctx, MPSFT_ERR_INVALID, "transform values must be in [0, n)");
  }
  if (opt && opt->trials >= 1 && opt->trials <= kMaxTrials) {
    for (int t = 0; t < opt->trials; ++t) {
      if (q[t] < 0 || q[t] >= n) {
        return Fail(ctx, MPSFT_ERR_INVALID, "q must be in [0, n)");
      }
    }
  }
  const Transform tf{a, b, c, a_inv};
  return IterateImpl(ctx, sig, opt, nullptr, &tf, q, mm_k, mm_c, mm_size,
                     mm_cap, found);
}

int mpsft_solve(mpsft_ctx *ctx, const mpsft_signal *sig,
                const mpsft_solve_options *opt, mpsft_rng *rng,
                int32_t *out_k, double *out_c, int32_t cap, int32_t *count,
                mpsft_stats *stats) {
  if (!ctx || !opt || !rng || !count || (cap > 0 && (!out_k || !out_c))) {
    return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  }
  const mpsft_signal *sigs[1] = {sig};
  mpsft_rng *rngs[1] = {rng};
  int32_t *ok[1] = {out_k};
  double *oc[1] = {out_c};
  return SolveMany(ctx, sigs, opt, 1, rngs, ok, oc, &cap, count, stats);
}

int mpsft_ctx_set_timeline(mpsft_ctx *ctx, int enable) {
  if (!ctx) return MPSFT_ERR_INVALID;
  ctx->timeline_on = enable != 0;
  return MPSFT_OK;
}

int mpsft_ctx_timeline(const mpsft_ctx *ctx, int32_t *kernel, double *us,
                       int32_t cap, int32_t *count) {
  if (!ctx || !count || (cap > 0 && (!us || !kernel))) return MPSFT_ERR_INVALID;
  const int32_t total = int32_t(ctx->timeline.size() / 2);
  // in start order (the records' slots are taken in arrival order)
  std::vector<std::pair<unsigned long long, int32_t>> r(total);
  for (int32_t j = 0; j < total; ++j) {
    r[j] = {ctx->timeline[2 * j + 1], int32_t(ctx->timeline[2 * j])};
  }
  std::sort(r.begin(), r.end());
  for (int32_t j = 0; j < total && j < cap; ++j) {
    kernel[j] = r[j].second;
    us[j] = 1e-3 * double(r[j].first - r[0].first);
  }
  *count = total;
  return MPSFT_OK;
}

int32_t mpsft_fold_shape_count(void) { return kFoldShapes; }

int mpsft_ctx_set_fold_shape(mpsft_ctx *ctx, int32_t shape) {
  if (!ctx) return MPSFT_ERR_INVALID;
  if (shape < -1 || shape >= kFoldShapes) {
    return Fail(ctx, MPSFT_ERR_INVALID, "no such fold shape");
  }
  ctx->force_shape = shape;
  return MPSFT_OK;
}

int mpsft_autotune(mpsft_ctx *ctx, const mpsft_signal *const *sigs,
                   const mpsft_solve_options *opts, int32_t nsig, int32_t seed,
                   int32_t repeats) {
  if (!ctx || !sigs || !opts || nsig <= 0) {
    return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  }
  for (int i = 0; i < nsig; ++i) {
    if (!sigs[i]) return Fail(ctx, MPSFT_ERR_INVALID, "null signal");
    if (opts[i].precision != MPSFT_PREC_FP32) {
      return Fail(ctx, MPSFT_ERR_INVALID, "the autotuner times FP32 solves");
    }
  }
  repeats = std::max(1, repeats);
  const bool prof = ctx->profiling;
  const int32_t forced = ctx->force_shape;
  // best[shape][launch]: the shortest of the repeats
  std::vector<std::vector<double>> best(kFoldShapes);
  std::vector<mpsft_bin_launch> recs0;
  std::vector<int32_t> caps(nsig), counts(nsig);
  std::vector<std::vector<int32_t>> ok(nsig);
  std::vector<std::vector<double>> oc(nsig);
  std::vector<int32_t *> okp(nsig);
  std::vector<double *> ocp(nsig);
  for (int i = 0; i < nsig; ++i) {
    caps[i] = 4 * opts[i].k + 4096;
    ok[i].resize(caps[i]);
    oc[i].resize(2 * size_t(caps[i]));
    okp[i] = ok[i].data();
    ocp[i] = oc[i].data();
  }
  int rc = MPSFT_OK;
  ctx->profiling = true;
  for (int rep = 0; rep < repeats && rc == MPSFT_OK; ++rep) {
    for (int shape = 0; shape < kFoldShapes && rc == MPSFT_OK; ++shape) {
      ctx->force_shape = shape;
      std::vector<mpsft_rng> rng(nsig);
      std::vector<mpsft_rng *> rp(nsig);
      for (int i = 0; i < nsig; ++i) {
        rng[i].Seed(seed + i);
        rp[i] = &rng[i];
      }
      rc = SolveMany(ctx, sigs, opts, nsig, rp.data(), okp.data(), ocp.data(),
                     caps.data(), counts.data(), nullptr);
      if (rc) break;
      std::vector<double> &b = best[shape];
      const std::vector<mpsft_bin_launch> &r = ctx->bin_launches;
      if (shape == 0 && rep == 0) recs0 = r;
      if (b.empty()) b.assign(r.size(), 1e300);
      for (size_t j = 0; j < r.size() && j < b.size(); ++j) {
        b[j] = std::min(b[j], r[j].ms);
      }
    }
  }
  ctx->profiling = prof;
  ctx->force_shape = forced;
  if (rc) return rc;
  // a launch counts for the bins class its solve graph phase looks up
  int64_t nmax = 0;
  int32_t bins_cap = 0, min_bins_max = 1;
  for (int i = 0; i < nsig; ++i) {
    nmax = std::max<int64_t>(nmax, sigs[i]->n);
    bins_cap = std::max<int32_t>(bins_cap,
                                 std::max(2 * opts[i].k + 1, opts[i].min_bins));
    min_bins_max = std::max(min_bins_max, opts[i].min_bins);
  }
  const bool c128 = sigs[0]->dtype == MPSFT_C128;
  auto key_of = [&](const mpsft_bin_launch &r) {
    return CeilLog2(PhaseBins(r.max_bins, bins_cap, min_bins_max));
  };
  std::vector<int> keys;
  for (const auto &r : recs0) {
    if (r.precision != MPSFT_PREC_FP32) continue;
    const int kb = key_of(r);
    if (std::find(keys.begin(), keys.end(), kb) == keys.end()) keys.push_back(kb);
  }
  // per key: the shape with the least total time over the key's launches
  for (int kb : keys) {
    double tbest = 1e300;
    int sbest = 0;
    for (int shape = 0; shape < kFoldShapes; ++shape) {
      double t = 0;
      for (size_t j = 0; j < recs0.size() && j < best[shape].size(); ++j) {
        if (recs0[j].precision == MPSFT_PREC_FP32 && key_of(recs0[j]) == kb) {
          t += best[shape][j];
        }
      }
      if (t < tbest) {
        tbest = t;
        sbest = shape;
      }
    }
    mpsft_ctx::TuneEntry e{kb, CeilLog2(nmax), CeilLog2(nsig), c128 ? 1 : 0, sbest,
                           float(1e3 * tbest)};
    auto &tab = ctx->tuning;
    tab.erase(std::remove_if(tab.begin(), tab.end(),
                             [&](const mpsft_ctx::TuneEntry &o) {
                               return o.bins_log2 == e.bins_log2 &&
                                      o.n_log2 == e.n_log2 &&
                                      o.nsig_log2 == e.nsig_log2 && o.c128 == e.c128;
                             }),
              tab.end());
    tab.push_back(e);
  }
  ctx->tuning_version += 1;
  return MPSFT_OK;
}

int mpsft_tuning_save(mpsft_ctx *ctx, const char *path) {
  if (!ctx || !path) return MPSFT_ERR_INVALID;
  FILE *f = std::fopen(path, "w");
  if (!f) return Fail(ctx, MPSFT_ERR_INVALID, std::string("cannot write ") + path);
  std::fprintf(f, "# mpsft-gb300 fold launch shapes: bins_log2 n_log2 "
                  "signals_log2 complex128 shape us\n");
  for (const auto &e : ctx->tuning) {
    std::fprintf(f, "%d %d %d %d %d %.3f\n", e.bins_log2, e.n_log2, e.nsig_log2,
                 e.c128, e.shape, double(e.us));
  }
  std::fclose(f);
  return MPSFT_OK;
}

int mpsft_tuning_load(mpsft_ctx *ctx, const char *path) {
  if (!ctx || !path) return MPSFT_ERR_INVALID;
  FILE *f = std::fopen(path, "r");
  if (!f) return Fail(ctx, MPSFT_ERR_INVALID, std::string("cannot read ") + path);
  std::vector<mpsft_ctx::TuneEntry> tab;
  char line[256];
  while (std::fgets(line, sizeof(line), f)) {
    if (line[0] == '#' || line[0] == '\n') continue;
    mpsft_ctx::TuneEntry e{};
    double us = 0;
    if (std::sscanf(line, "%d %d %d %d %d %lf", &e.bins_log2, &e.n_log2,
                    &e.nsig_log2, &e.c128, &e.shape, &us) != 6 ||
        e.shape < 0 || e.shape >= kFoldShapes) {
      std::fclose(f);
      return Fail(ctx, MPSFT_ERR_INVALID, std::string("bad tuning line in ") + path);
    }
    e.us = float(us);
    tab.push_back(e);
  }
  std::fclose(f);
  ctx->tuning = tab;
  ctx->tuning_version += 1;
  return MPSFT_OK;
}

int32_t mpsft_tuning_size(const mpsft_ctx *ctx) {
  return ctx ? int32_t(ctx->tuning.size()) : 0;
}

int mpsft_solve_batched(mpsft_ctx *ctx, const mpsft_signal *const *sigs,
                        const mpsft_solve_options *opts, int32_t nsig,
                        mpsft_rng *const *rngs, int32_t *const *out_k,
                        double *const *out_c, const int32_t *cap,
                        int32_t *count, mpsft_stats *stats) {
  if (!ctx || !sigs || !opts || !rngs || !out_k || !out_c || !cap || !count) {
    return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  }
  return SolveMany(ctx, sigs, opts, nsig, rngs, out_k, out_c, cap, count,
                   stats);
}

int mpsft_solve_batched_packed(mpsft_ctx *ctx, const mpsft_signal *const *sigs,
                               const mpsft_solve_options *opts, int32_t nsig,
                               mpsft_rng *const *rngs, int32_t *out_k, double *out_c,
                               int64_t out_cap, int64_t *offsets, int32_t *count,
                               mpsft_stats *stats) {
  if (!ctx || !sigs || !opts || !rngs || !out_k || !out_c || !offsets || !count ||
      out_cap < 0) {
    return Fail(ctx, MPSFT_ERR_INVALID, "null argument");
  }
  const PackedOut packed{out_k, out_c, out_cap, offsets};
  return SolveMany(ctx, sigs, opts, nsig, rngs, nullptr, nullptr, nullptr, count,
                   stats, &packed);
}

}  // extern "C"
