// Shared definitions of the sm_103a MPSFT kernels and their host launchers.
//
// Data layout in device memory, per signal and iteration (all row-major):
//   x      : n complex samples, complex64 (float2) or complex128 (double2)
//   wt32/64: window at |t| for t in [0, p2] (the window is even), FP32 / FP64
//   fold   : trials x rows x bins_cap complex (FP32 or FP64), folded samples
//   ubuf   : trials x rows x bins_cap complex128, bins after the size-B FFT
//   table  : open-addressing hash of found modes, key k0 (-1 = empty) and
//            complex128 coefficient
//   bucket : per-bin lists of table slots whose mode falls in that bin
//   cand   : per-bin candidate (valid, k0, coefficient) of this iteration
// rows = 1 + 2*bits: row 0 is tau = q, row 2s+1 is q + bins*2^s, row 2s+2 is
// q - bins*2^s (the reference's row order, src/binner.cc:42-50).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mpsft {

constexpr int kMaxTrials = 15;     // odd trials up to 15
constexpr int kMaxBits = 31;       // rows <= 63; a warp lane per bit in decide
constexpr int kFoldLanes = 8;      // threads sharing one (row pair, bin)
constexpr int kMaxFoldsPerLane = 10;  // folds f = p / bins <= 80
constexpr int kMaxFFT = 16384;     // largest Bluestein transform (FP32)
constexpr int kMaxFFTLog2 = 14;
static_assert((1 << kMaxFFTLog2) == kMaxFFT, "transform size");
constexpr int kMaxFFT64 = 8192;    // largest Bluestein transform (FP64)
constexpr int32_t kEmptyKey = -1;
constexpr int kRebinChunks = 16;   // re-binning: at most this many chunks of the support
// chunks of a window support of p samples: runs of at least 16 samples per
// lane (32 lanes per chunk; a short support spreads over several warps, so
// that each lane waits for few rounds of gathers), at most kRebinChunks
constexpr int kStashHeader = 256;   // bytes before a stash buffer's samples
// samples of a stash buffer at most (per trial: max(p, this))
constexpr int64_t kStashMaxSamples = int64_t(1) << 20;
__host__ __device__ inline int RebinChunks(int p) {
  const int c = (p + 511) / 512;
  return c < 1 ? 1 : (c > kRebinChunks ? kRebinChunks : c);
}
constexpr int kMaxListed = 256;    // near-tie bins listed per signal/iteration
constexpr int kRebinMaxSignals = 256;  // signals per FP64 re-binning launch

// found flag, status bits, near ties, mode count, spilled candidates
constexpr int kCtlWords = 5;
// candidates per signal and iteration whose k1 rounded into a neighbouring
// bin's range (inserted after the others, in bin order: InsertSpills)
constexpr int kSpillCap = 16;
// cand_valid of a listed near-tie bin held back from the merge until its FP64
// decision (added to the FP32 pass's 0 or 2)
constexpr int32_t kCandListed = 3;

// Per-signal status bits written by the device.
enum : int32_t {
  kStatusCapacity = 1,   // mode table full
  kStatusNonFinite = 2,  // NaN / Inf in a bin that reached the decisions
  kStatusUnresolved = 4, // near ties left to FP32 (bins too large for FP64 redo)
};

// FP32 near-tie bound, in units of eps_rel = margin * 2^-24: the bins of a
// row carry at most kEpsRms * rms + kEpsRowMax * (largest |U| of the row) +
// kEpsValue * |U| of rounding error, rms the row's own sqrt(mean |U|^2 / 2)
// over its bins (the row transform measures it). Measured on GB300 over 240
// random binnings (n up to 2^22, prime and power of two, 51 to 2001 bins,
// 20 to 80 dB): the largest error is 1.04 of this sum without the margin
// (the same as 8 times the signal-wide rms sqrt(mean |x|^2 / (2 bins)), which
// the rows' own rms is 0.43 to 0.91 of); the margin multiplies it.
constexpr float kEpsRms = 12.0f;
constexpr float kEpsRowMax = 1.0f;
constexpr float kEpsValue = 4.0f;

// Everything a kernel needs about one signal in the current iteration.
// Filled by the host engine and copied to the device once per iteration.
struct SigIter {
  const void *x;
  int32_t n, bins, bits, rows;
  int32_t p, p2, folds;
  int32_t a, b, c, a_inv;
  int32_t phase_shift;  // 32 - log2(n) when n is a power of two, else -1
  // 64-bit fixed-point constants of the FP32 binning (SetFixedPoint):
  // n_inv = floor(2^64 / n) (0 when n is a power of two), phi_b = b/n and
  // psi = 1/(2 bins) in turns, both rounded to 2^-64
  uint64_t n_inv, phi_b, psi;
  // round(2^64 / n) (0 for n = 1): r / n in 64-bit fixed-point turns
  uint64_t n_fix;
  // erf_d / (4 n bins) in FP32: the FP32 window response's argument scale
  float wf_scale;
  double xi_scale;  // 1 / (2 n bins): xi = (2 bins k1 - (2 beta + 1) n) xi_scale
  // FP64 unit phases e^{2 pi i r / n} = ph_hi[r >> ph_k] * ph_lo[r & (2^ph_k - 1)]
  // (built once per call, see PhaseTableK)
  double2 *ph_lo, *ph_hi;
  int32_t ph_k;
  int32_t ph_build;  // 1: k_phase_tables fills ph_lo / ph_hi of this signal
  // FP32 copies of the thresholds (the near-tie windows include their rounding)
  float bin_thr2_f, sv_thr_f;
  int32_t trials;
  int32_t active;
  int32_t q[kMaxTrials];
  double bq_re[kMaxTrials], bq_im[kMaxTrials];  // e^{2 pi i (b q mod n)/n}
  // window
  double width;     // 1 / (2 bins)
  double sigma_f;   // frequency-domain Gaussian width
  double erf_d;     // sqrt(2) * pi * sigma_t, scale of SampleInFreq
  // thresholds (0 = off)
  double bin_thr, sv_thr, win_thr;
  // FFT (Bluestein) size for this bins
  int32_t fft_m, fft_log2m;
  // buffers
  float *wt32;
  double *wt64;
  float2 *wtff;         // wt64 as float-float (hi, lo); may be null
  void *fold;           // FP32: float2, FP64: double2
  // a second fold buffer of the same size: in the fixed-bins phase the next
  // iteration (planned ahead) folds into it while this iteration's row
  // transforms read fold (k_plan swaps the two)
  void *fold_alt;
  // the samples the FP32 fold gathered, for the near-tie re-binning (which
  // then reads them in order instead of gathering them again from x):
  // a header word (1: this iteration's fold wrote them, StashRows rows;
  // 0: it did not) then, for trial tr, stashed row r and -p2 <= t <= p2,
  // sample (tr StashRows + r) p + t + p2, of the input's type. null when
  // unused. stash_alt: the second buffer, for the iteration planned ahead
  // (k_plan swaps the two with fold / fold_alt)
  unsigned char *stash, *stash_alt;
  int64_t stash_cap;  // samples per buffer
  double2 *ubuf;
  // solves and iterations on the FP32 path: the FP32 pass's bins (the row
  // FFT writes here instead of ubuf, which then holds only FP64 bins)
  float2 *ubuf32;
  int32_t bins_cap;     // row stride of fold / ubuf / ubuf32
  // Bluestein tables: chirp = e^{-pi i k^2 / bins} (bins entries) and
  // chat = FFT of the conjugate chirp sequence (fft_m entries), FP32 and FP64
  float2 *chirp32, *chat32;
  double2 *chirp64, *chat64;
  // FP32 path: e^{-pi i r / bins} for r < 2 bins (FP64), the bins-grid half of
  // the near-tie phase steps (the n grid comes from ph_lo / ph_hi); may be null
  double2 *r2b64;
  // mode table
  int32_t *tab_key;
  double2 *tab_coef;
  double *tab_err;      // bound on each coefficient's FP32 rounding error
  int32_t tab_cap;      // power of two
  int32_t *tab_count;   // distinct keys stored = length of occ_list
  int32_t *occ_list;    // occupied slots, in insertion order
  // per-slot quantities of the current permutation (k_mode_prep)
  int32_t *mode_bin;    // bin of the slot's mode, -1 for an empty slot
  int32_t *mode_k1;     // (a k0 + b) mod n
  // FP64 path: [slot * trials + t] = wf * coef * e^{2 pi i (q_t k1 + c k0)/n}
  double2 *mode_base;
  // FP32 path: the same terms in FP32, and per slot the error the mode
  // carries into its bin
  float2 *mode_base32;
  float *mode_errw;
  // bucketing of table modes by bin
  int32_t *bkt_count;   // bins_cap
  int32_t *bkt_start;   // bins_cap
  int32_t *bkt_list;    // tab_cap
  // candidates of this iteration
  int32_t *cand_valid;  // bins_cap
  int32_t *cand_k0;
  double2 *cand_coef;
  double *cand_err;
  // FP32 near-tie detection: bins whose decisions lie within eps_u (the
  // a-priori bound on an FP32 bin's rounding error) plus the error carried by
  // the subtracted modes are listed for FP64 treatment. The bound's rms term
  // of row r is eps_ms * sqrt(row_ms[r]), eps_ms = eps_rel kEpsRms / sqrt(2)
  // (0 on the FP64 path).
  float eps_ms;
  float *row_max;       // [t * rows + r]: max |U| of the row (row transforms)
  float *row_ms;        // [t * rows + r]: mean |U|^2 over the row's bins
  // re-binning of listed bins: [((e * trials + t) * rows + r) * chunks + c]
  // partial sums over chunk c of the window support
  double2 *esc_part;
  // [(e * trials + t) * rows + r]: the chunk partials summed in chunk order
  // (by the warp that finishes the row's last chunk) and the arrival counter
  double2 *esc_sum;
  // [(e * trials + t) * rows + r]: the FP64 sum of the listed bin's found
  // modes in row r (k_listed_terms), subtracted by its FP64 decision
  double2 *esc_msub;
  int32_t *esc_cnt;
  // per listed bin e: s^k, k < 64, with s = e^{2 pi i (b/n - (2 beta + 1)/(2B))}
  // as float-float {re.hi, im.hi, re.lo, im.lo} at [e * 64 + k], and s^64
  // (the direct evaluation of every bin; null in solves and iterations,
  // whose re-binning evaluates them per work item)
  float4 *esc_pow;
  double2 *esc_step;
  // per-value part of the FP32 error bound: eps_rel * (kEpsRowMax * max |U|
  // of the rows involved + kEpsValue * |value|)
  float eps_rel;
  // FP32 path only: 1 when this signal's FP32 rounding is not small against
  // its noise thresholds, so this iteration runs on the FP64 kernels
  int32_t force_fp64;
  // 1 when the window and FP32 Bluestein tables for this iteration's bins are
  // in place (the previous iteration's, the context's table cache, or built
  // in this iteration by another signal of the batch): the table kernels skip
  // this signal
  int32_t tables_valid;
  // table cache slot (bins >> 1) this signal builds in this iteration, or -1
  int32_t win_slot;
  // 1 when the table's coefficients already carry their window responses
  // (wf * coef, from a caller's window), so that the mode terms use wf = 1
  int32_t unit_wf;
  int32_t *esc_list;    // esc_cap bins
  uint32_t *esc_mask;   // per listed bin: bit s set = rows 2s+1, 2s+2 near
  int32_t esc_cap;
  int32_t *flags;       // [0] found, [1] status bits, [2] near-tie bins
                        // flagged this iteration, [3] mode count, [4] spills
  // spilled candidates of this iteration (kSpillCap): bin, k0, coefficient,
  // error bound
  int32_t *spill_beta;
  int32_t *spill_k0;
  double2 *spill_coef;
  double *spill_err;
  // solve-graph timeline (signal 0's descriptor; null = off): the iteration
  // kernels record (kernel id, device clock) at entry, PdlEnter
  unsigned long long *trace;
  uint32_t *trace_count;
  uint32_t trace_cap;
};

// The rows whose gathered samples the FP32 fold stashes this iteration (the
// fold and the re-binning evaluate it alike): every row while the fold
// gathers from at most an eighth of the signal's samples (the gathers then
// hit distinct sectors at the random-gather rate, and the sequential writes
// of the stash take little of the bandwidth), else row 0 alone (read again
// by every listed bin); 0 without a stash.
__host__ __device__ inline int StashRows(const SigIter &it) {
  if (it.stash == nullptr) return 0;
  const int64_t row = int64_t(it.p) * it.trials;
  const int64_t all = row * it.rows;
  if (all <= it.stash_cap && all <= int64_t(it.n) / 8) return it.rows;
  return row <= it.stash_cap ? 1 : 0;
}

// Per-signal state of a solve run on the device (k_plan / k_finish). The
// host fills the configuration and the draw table; the device owns the rest.
enum : int32_t {  // solve status codes (the C ABI's values)
  kSolveCapacity = 4,
  kSolveIterCap = 5,
  kSolveNonFinite = 6,
};
struct SolveCtl {
  // configuration
  int32_t k, min_bins, trials, draw_stride, max_stale, max_iter;
  int32_t fp64_path, force_fp64;
  double sigma, sqrt_c_delta, win_thr, margin;
  // draws: iteration draw_base + j uses draws[j * (4 + T) ...] =
  // a, b, c, a_inv, q_0 .. q_{trials-1}, for j < draws_avail, and
  // draw_bq[(j * T + t) * 2 ...]; T = the largest trials of the batch
  const int32_t *draws;
  const double *draw_bq;  // row phase (re, im) per draw and trial, host-made
  int32_t draw_base, draws_avail;
  // state
  int32_t iter, stale, done, status, last_bins;
  int32_t near_ties, unresolved, fp64_iters;
  int64_t gathers, bin_bytes;
  // the context's table cache (null: per-signal tables): per odd bins B,
  // block win_base[B >> 1] of win_pool holds wt32, wt64, wtff (p2 + 1
  // entries each), chirp32 (B), chat32 (M) and r2b64 (2B), each 16-byte
  // aligned;
  // win_valid marks built blocks, win_claim elects one builder per block
  const int64_t *win_base;
  unsigned char *win_pool;
  int32_t *win_valid, *win_claim;
};

// Byte offsets of the tables inside a table-cache block.
struct WinBlock {
  int64_t wt64, wtff, chirp32, chat32, r2b64, bytes;
};
__host__ __device__ inline int64_t Align16(int64_t v) { return (v + 15) & ~int64_t(15); }
__host__ __device__ inline WinBlock WinBlockOf(int32_t p2, int32_t bins, int32_t m) {
  WinBlock w;
  const int64_t e = int64_t(p2) + 1;
  w.wt64 = Align16(4 * e);
  w.wtff = w.wt64 + Align16(8 * e);
  w.chirp32 = w.wtff + Align16(8 * e);
  w.chat32 = w.chirp32 + Align16(8 * int64_t(bins));
  w.r2b64 = w.chat32 + Align16(8 * int64_t(m));
  w.bytes = w.r2b64 + Align16(32 * int64_t(bins));
  return w;
}

// ---------------------------------------------------------------- helpers
__host__ __device__ inline int64_t PosMod(int64_t v, int64_t n) {
  v %= n;
  return v < 0 ? v + n : v;
}

// The fixed-point constants that depend on n and the bins only (n, bins and
// erf_d set).
__host__ __device__ inline void SetBinsFixedPoint(SigIter *it) {
  const uint64_t n = uint64_t(it->n);
  const bool pow2 = (n & (n - 1)) == 0;
  it->n_inv = pow2 ? 0 : uint64_t(((unsigned __int128)1 << 64) / n);
  const uint64_t twoB = 2 * uint64_t(it->bins);
  it->psi = uint64_t((((unsigned __int128)1 << 64) + twoB / 2) / twoB);
  it->n_fix = n > 1 ? uint64_t((((unsigned __int128)1 << 64) + n / 2) / n) : 0;
  it->wf_scale = float(it->erf_d / (4.0 * double(n) * double(it->bins)));
  it->xi_scale = 1.0 / (2.0 * double(n) * double(it->bins));
}

// phi_b = round(2^64 (b mod n) / n) (n and b set); for n = 2^k it is exactly
// (b mod n) 2^(64 - k), without the 128-bit division.
__host__ __device__ inline void SetPhiB(SigIter *it) {
  const uint64_t n = uint64_t(it->n);
  const uint64_t bm = uint64_t(PosMod(it->b, int64_t(n)));
  if ((n & (n - 1)) == 0) {
#ifdef __CUDA_ARCH__
    const int k = 63 - __clzll(static_cast<long long>(n));
#else
    const int k = __builtin_ctzll(n);
#endif
    it->phi_b = bm << (64 - k);
  } else {
    it->phi_b = uint64_t((((unsigned __int128)bm << 64) + n / 2) / n);
  }
}

// The fixed-point constants of an iteration (n, b, bins and erf_d set).
__host__ __device__ inline void SetFixedPoint(SigIter *it) {
  SetBinsFixedPoint(it);
  SetPhiB(it);
}

// FP32 copies of an iteration's thresholds (bin_thr, sv_thr set).
__host__ __device__ inline void SetThresholdCopies(SigIter *it) {
  it->bin_thr2_f = float(it->bin_thr * it->bin_thr);
  it->sv_thr_f = float(it->sv_thr);
}

// Bits of the low table of the FP64 unit phases: ceil(log2 n) / 2 rounded up,
// so both tables hold about sqrt(n) entries.
__host__ __device__ inline int PhaseTableK(int64_t n) {
  int l = 0;
  while ((int64_t(1) << l) < n) ++l;
  return (l + 1) / 2;
}
__host__ __device__ inline int64_t PhaseTableHi(int64_t n) {
  return ((n - 1) >> PhaseTableK(n)) + 1;
}

// Programmatic dependent launch (the solve graph's kernels): every iteration
// kernel starts here. Launched with programmatic stream serialization, it
// waits until the kernel before it in its stream has completed and its
// writes are visible, then lets the kernel after it launch (its blocks are
// scheduled while this one runs, and wait here in turn). Launched without
// that attribute, both instructions return at once.
__device__ __forceinline__ void PdlEnter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Kernel ids of the timeline (mpsft_ctx_set_timeline).
enum : int32_t {
  kTracePlan = 1, kTraceWindow32, kTraceFold, kTraceBluestein, kTraceModePrep,
  kTraceBucket, kTraceRowFft, kTraceDecide, kTraceListedTerms, kTraceMerge,
  kTraceRebin, kTraceDecideListed, kTraceFinish, kTraceWindow64,
};

// PdlEnter, then (timeline on) the kernel's id and the device clock when its
// first block starts.
__device__ __forceinline__ void PdlEnter(const SigIter *its, int32_t id) {
  PdlEnter();
  if (threadIdx.x == 0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 &&
      its[0].trace != nullptr) {
    const uint32_t slot = atomicAdd(its[0].trace_count, 1u);
    if (slot < its[0].trace_cap) {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      its[0].trace[2 * slot] = uint64_t(id);
      its[0].trace[2 * slot + 1] = t;
    }
  }
}

// v mod n (non-negative) for |v| < 2^63 by Barrett reduction with
// inv = floor(2^64 / n), or a mask when n is a power of two (inv = 0).
__host__ __device__ __forceinline__ uint64_t MulHi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return uint64_t(((unsigned __int128)a * b) >> 64);
#endif
}

struct ModN {
  uint32_t n;
  uint64_t inv;
  __host__ __device__ __forceinline__ uint32_t operator()(int64_t v) const {
    if (inv == 0) return uint32_t(uint64_t(v) & uint64_t(n - 1));
    const bool neg = v < 0;
    const uint64_t a = neg ? uint64_t(-v) : uint64_t(v);
    uint64_t r = a - MulHi64(a, inv) * n;  // r < 3n
    if (r >= n) r -= n;
    if (r >= n) r -= n;
    return uint32_t(neg && r != 0 ? n - r : r);
  }
  // floor(v / n) for 0 <= v < 2^63
  __host__ __device__ __forceinline__ uint64_t quot(int64_t v) const {
    const uint64_t a = uint64_t(v);
    if (inv == 0) {
#ifdef __CUDA_ARCH__
      return a >> (__ffs(int(n)) - 1);
#else
      return a >> __builtin_ctz(n);
#endif
    }
    uint64_t q = MulHi64(a, inv);  // q <= floor(a / n) <= q + 2
    uint64_t r = a - q * n;
    if (r >= n) { r -= n; ++q; }
    if (r >= n) { ++q; }
    return q;
  }
};


// The FFT twiddle table, one block per transform size: W_N^e =
// e^{-2 pi i e / N} (N = 2^L, 1 <= L <= log2 kMaxFFT, e < N / 2) at entry
// 2^(L-1) - 1 + e, so that the lanes of a warp read consecutive entries.
constexpr int kTwiddleEntries = kMaxFFT - 1;
__host__ __device__ constexpr int TwiddleBase(int log2n) { return (1 << (log2n - 1)) - 1; }

// Entry i of the table, in FP64 and rounded to FP32 (every table of the
// library is filled by this): e^{-2 pi i k / kMaxFFT} with k = e kMaxFFT / N.
__device__ inline void TwiddleAt(int i, float2 *tw32, double2 *tw64) {
  const int L = 32 - __clz(i + 1);  // i + 1 in [2^(L-1), 2^L)
  const int k = (i - TwiddleBase(L)) << (kMaxFFTLog2 - L);
  double s, c;
  sincospi(-2.0 * double(k) / double(kMaxFFT), &s, &c);
  tw64[i] = make_double2(c, s);
  tw32[i] = make_float2(float(c), float(s));
}

__device__ inline float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ inline double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ inline double2 cadd(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}
__device__ inline double2 csub(double2 a, double2 b) {
  return make_double2(a.x - b.x, a.y - b.y);
}
__device__ inline double2 cscale(double2 a, double s) {
  return make_double2(a.x * s, a.y * s);
}

// e^{2 pi i m / n} for an exact integer m (any sign), FP64.
__device__ inline double2 UnitPhase64(int64_t m, int64_t n) {
  const int64_t r = PosMod(m, n);
  double s, c;
  sincospi(2.0 * (double(r) / double(n)), &s, &c);
  return make_double2(c, s);
}

// Same in FP32. The residue r = m mod n becomes 32-bit fixed-point turns
// floor(r 2^32 / n) (a shift when n = 2^k, shift = 32 - k), whose signed value
// is the angle reduced to [-1/2, 1/2) turns exactly.
__device__ inline float2 UnitPhase32(int64_t m, int64_t n, int shift) {
  uint32_t ph;
  if (shift >= 0) {
    ph = uint32_t(uint64_t(m) & uint64_t(n - 1)) << shift;
  } else {
    const uint64_t r = uint64_t(PosMod(m, n));
    ph = uint32_t((r << 32) / uint64_t(n));
  }
  float s, c;
  sincospif(2.0f * (float(int32_t(ph)) * 2.3283064365386963e-10f), &s, &c);
  return make_float2(c, s);
}

// e^{2 pi i m / n} from the phase tables (two FP64 table entries and one
// complex product: about 2.5 ulp), m any integer with |m| < 2^63.
__device__ inline double2 Phase64(const SigIter &it, int64_t m) {
  const uint32_t r = ModN{uint32_t(it.n), it.n_inv}(m);
  const double2 h = it.ph_hi[r >> it.ph_k];
  const double2 l = it.ph_lo[r & ((1u << it.ph_k) - 1u)];
  return cmul(h, l);
}

// e^{2 pi i m / n} in FP32: r = m mod n as 32-bit fixed-point turns
// round(r 2^32 / n) (error below 2^-33 turns), whose signed value is the angle
// reduced to [-1/2, 1/2) turns.
__device__ inline float2 Phase32(const SigIter &it, int64_t m) {
  const uint64_t r = ModN{uint32_t(it.n), it.n_inv}(m);
  const uint32_t ph = uint32_t((r * it.n_fix + (uint64_t(1) << 31)) >> 32);
  float s, c;
  sincospif(2.0f * (float(int32_t(ph)) * 2.3283064365386963e-10f), &s, &c);
  return make_float2(c, s);
}

// SampleInFreq (src/window.cc:77-81): window response at offset xi.
__device__ inline double WindowInFreq(const SigIter &it, double xi) {
  const double c = 0.5 * it.width;
  return 0.5 * (erf((xi + c) * it.erf_d) - erf((xi - c) * it.erf_d));
}

// FP64 row-0 terms wf c e^{2 pi i (q_t k1 + c k0)/n} of the mode in table
// slot s (k1 and its bin given) into mode_base (BinInFreqV1::Run,
// src/binner.cc:565-591).
__device__ inline void ModeTerms64(const SigIter &it, int s, int64_t k1, int bin) {
  const double xi = (double(bin) + 0.5) / double(it.bins) - double(k1) / double(it.n);
  const double2 wc =
      it.unit_wf ? it.tab_coef[s] : cscale(it.tab_coef[s], WindowInFreq(it, xi));
  const int32_t key = it.tab_key[s];
  for (int t = 0; t < it.trials; ++t) {
    const int64_t ph = int64_t(it.q[t]) * k1 + int64_t(it.c) * key;
    it.mode_base[size_t(s) * it.trials + t] = cmul(wc, Phase64(it, ph));
  }
}

// 2x2 matrix pencil [[u0, u2], [u1, u0]] (src/freqid.cc:27-48).
// sigma0 = sqrt(largest eigenvalue of A^H A), sigma1 = |det A| / sigma0 (no
// cancellation). With m01 = conj(u0) u2 + conj(u1) u0, the off-diagonal of
// A^H A, the dominant right singular vector is (lmax - m11, conj(m01)) or
// (m01, lmax - m00), so the reference's vote Im(conj(v00) v10) < 0 is exactly
// Im(m01) > 0 (and false when m01 = 0, where v is a unit axis). Returns the
// vote; *im_m01 receives Im(m01) for the near-tie margin.
template <typename T> struct CplxOf;
template <> struct CplxOf<float> { using V = float2; };
template <> struct CplxOf<double> { using V = double2; };

template <typename T, typename V>
__device__ inline bool PencilT(V u0, V u1, V u2, T *s0_out, T *s1_out,
                               T *im_m01) {
  const T m00 = u0.x * u0.x + u0.y * u0.y + u1.x * u1.x + u1.y * u1.y;
  const T m11 = u2.x * u2.x + u2.y * u2.y + u0.x * u0.x + u0.y * u0.y;
  // m01 = conj(u0) u2 + conj(u1) u0
  const T mr = (u0.x * u2.x + u0.y * u2.y) + (u1.x * u0.x + u1.y * u0.y);
  const T mi = (u0.x * u2.y - u0.y * u2.x) + (u1.x * u0.y - u1.y * u0.x);
  const T hd = T(0.5) * (m00 - m11);
  const T r = sqrt(hd * hd + (mr * mr + mi * mi));
  const T lmax = T(0.5) * (m00 + m11) + r;
  const T s0 = sqrt(lmax > T(0) ? lmax : T(0));
  // det = u0 u0 - u2 u1
  const T dr = (u0.x * u0.x - u0.y * u0.y) - (u2.x * u1.x - u2.y * u1.y);
  const T di = (T(2) * u0.x * u0.y) - (u2.x * u1.y + u2.y * u1.x);
  *s0_out = s0;
  *s1_out = s0 > T(0) ? sqrt(dr * dr + di * di) / s0 : T(0);
  *im_m01 = mi;
  return mi > T(0);
}

// The same vote with |det A|^2 and sigma0^2 = lmax instead of sigma1, for a
// threshold test sigma1 / 2 > s as |det|^2 > 4 s^2 lmax.
template <typename T, typename V>
__device__ inline bool PencilSq(V u0, V u1, V u2, T *det2, T *lmax_out,
                                T *im_m01) {
  const T m00 = u0.x * u0.x + u0.y * u0.y + u1.x * u1.x + u1.y * u1.y;
  const T m11 = u2.x * u2.x + u2.y * u2.y + u0.x * u0.x + u0.y * u0.y;
  const T mr = (u0.x * u2.x + u0.y * u2.y) + (u1.x * u0.x + u1.y * u0.y);
  const T mi = (u0.x * u2.y - u0.y * u2.x) + (u1.x * u0.y - u1.y * u0.x);
  const T hd = T(0.5) * (m00 - m11);
  const T lmax = T(0.5) * (m00 + m11) + sqrt(hd * hd + (mr * mr + mi * mi));
  const T dr = (u0.x * u0.x - u0.y * u0.y) - (u2.x * u1.x - u2.y * u1.y);
  const T di = (T(2) * u0.x * u0.y) - (u2.x * u1.y + u2.y * u1.x);
  *det2 = dr * dr + di * di;
  *lmax_out = lmax > T(0) ? lmax : T(0);
  *im_m01 = mi;
  return mi > T(0);
}

__device__ inline bool Pencil(double2 u0, double2 u1, double2 u2,
                              double *s0_out, double *s1_out) {
  double im;
  return PencilT<double, double2>(u0, u1, u2, s0_out, s1_out, &im);
}

// True when signal `it` takes the FP64 kernels of the FP32 path this
// iteration: by the precision policy, or because its near-tie list overflowed.
__device__ inline bool RedoFP64(const SigIter &it) {
  return it.force_fp64 || *(volatile int32_t *)&it.flags[2] > it.esc_cap;
}

// ---- the FP32 binning's row cluster -------------------------------------
// Row r's window covers u = off_r + t, |t| <= p2, of the permuted, modulated
// samples y_u = x[a (q + u) + c] e^{2 pi i (b u / n - u / (2 bins))}, with
// off_r = m bins, m in {0, +-1, +-2, ..., +-2^(bits-1)}. Row 0 and the pair
// groups g = 1..ClusterGroups (m = +-2^(g-1)) have overlapping windows (that
// of m = 2^(g-1) overlaps that of 2^(g-2) while 2^(g-2) <= folds - 1), so
// they are binned together from the union of their windows: each sample of
// the union is gathered once and serves every row whose window covers it.
// The span of the union is folds + 2 Mc bins-steps per bin (Mc the largest
// m of the cluster), kept at most kMaxClusterSpan (shared-memory tile).
constexpr int kMaxClusterSpan = 96;
__host__ __device__ inline int ClusterGroups(int folds, int bits) {
  int s = 0;
  while (s < bits) {
    const int g = s + 1;
    if (g >= 2 && (1 << (g - 2)) > folds - 1) break;
    if (folds + 2 * (1 << (g - 1)) > kMaxClusterSpan) break;
    ++s;
  }
  return s;
}
__host__ __device__ inline int ClusterSpan(int folds, int bits) {
  const int sc = ClusterGroups(folds, bits);
  return folds + (sc > 0 ? 2 << (sc - 1) : 0);
}

// Samples the binning gathers in one iteration: FP32 path, the cluster's
// union (bins * span per trial) plus both rows of every other pair group
// (2 p each); FP64 kernels, every row's p samples.
__host__ __device__ inline int64_t BinGathers(const SigIter &it, bool fp64) {
  if (fp64) return int64_t(it.trials) * it.p * it.rows;
  const int sc = ClusterGroups(it.folds, it.bits);
  return int64_t(it.trials) *
         (int64_t(it.bins) * ClusterSpan(it.folds, it.bits) +
          2 * int64_t(it.bits - sc) * it.p);
}

// Algorithmic bytes of a binning launch for one signal, by the reference's
// gather count (BinInTime reads p samples per row, src/binner.cc:394-507):
// one 32-byte sector per sample of every row's window, the window table and
// the fold output. (The FP32 kernels gather fewer samples, BinGathers.)
__host__ __device__ inline int64_t BinBytesOf(const SigIter &it, bool fp64) {
  return 32 * int64_t(it.trials) * it.p * it.rows +
         int64_t(fp64 ? 8 : 4) * (it.p2 + 1) +
         int64_t(it.trials) * (fp64 ? 16 : 8) * it.rows * it.bins;
}

// Shared-memory keys of k_bucket: half the table (a power of two). The host
// keeps tables at or below kMaxTableCap so that this fits in shared memory
// and slots fit the 20 bits of the sort key.
constexpr int32_t kMaxTableCap = 1 << 15;
__host__ __device__ inline int BucketKeys(int tab_cap) { return tab_cap / 2; }

// Hash slot of a mode key (Fibonacci hashing into a power-of-two table).
__device__ inline uint32_t KeySlot(int32_t k, int32_t cap) {
  return (uint32_t(k) * 2654435769u) & uint32_t(cap - 1);
}

// mm[k0] += coef (and its error bound) in the signal's open-addressing table
// (linear probing; a new key takes the next entry of the insertion list).
__device__ inline void InsertMode(const SigIter &it, int32_t k0, double2 coef,
                                  double err) {
  const int cap = it.tab_cap;
  uint32_t slot = KeySlot(k0, cap);
  for (int probe = 0; probe < cap; ++probe) {
    const int32_t prev = atomicCAS(&it.tab_key[slot], kEmptyKey, k0);
    if (prev == kEmptyKey) {
      it.occ_list[atomicAdd(it.tab_count, 1)] = int32_t(slot);
    }
    if (prev == kEmptyKey || prev == k0) {
      atomicAdd(&it.tab_coef[slot].x, coef.x);
      atomicAdd(&it.tab_coef[slot].y, coef.y);
      if (err != 0.0) atomicAdd(&it.tab_err[slot], err);
      return;
    }
    slot = (slot + 1) & uint32_t(cap - 1);
  }
  atomicOr(&it.flags[1], kStatusCapacity);
}

// The iteration's spilled candidates into the table, in increasing bin
// order, after every other candidate (one thread per signal). A candidate's
// k1 lies in its own bin's range except when it rounds across the bin's edge
// (a mode at the edge, seen by both bins); only then can two candidates of
// one iteration meet in one table entry. The others are added by atomics,
// at most one per entry, and the spills in this fixed order, so the
// coefficients do not depend on the order in which blocks run.
__device__ inline void InsertSpills(const SigIter &it) {
  const int ns = min(it.flags[4], kSpillCap);
  uint32_t left = ns >= 32 ? 0xffffffffu : ((1u << ns) - 1u);
  while (left) {
    int best = __ffs(left) - 1;
    for (uint32_t m = left & (left - 1); m; m &= m - 1) {
      const int j = __ffs(m) - 1;
      if (it.spill_beta[j] < it.spill_beta[best]) best = j;
    }
    InsertMode(it, it.spill_k0[best], it.spill_coef[best], it.spill_err[best]);
    left &= ~(1u << best);
  }
  it.flags[4] = 0;
}

}  // namespace mpsft
