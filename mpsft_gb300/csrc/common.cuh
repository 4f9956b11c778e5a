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
constexpr int kMaxFFT64 = 8192;    // largest Bluestein transform (FP64)
constexpr int32_t kEmptyKey = -1;

// Per-signal status bits written by the device.
enum : int32_t {
  kStatusCapacity = 1,   // mode table full
  kStatusNonFinite = 2,  // NaN / Inf in a bin that reached the decisions
};

// Everything a kernel needs about one signal in the current iteration.
// Filled by the host engine and copied to the device once per iteration.
struct SigIter {
  const void *x;
  int32_t n, bins, bits, rows;
  int32_t p, p2, folds;
  int32_t a, b, c, a_inv;
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
  void *fold;           // FP32: float2, FP64: double2
  double2 *ubuf;
  int32_t bins_cap;     // row stride of fold / ubuf
  void *chirp;          // bins entries, e^{-pi i k^2 / bins} (float2 / double2)
  void *chat;           // fft_m entries, FFT of the conjugate chirp sequence
  // mode table
  int32_t *tab_key;
  double2 *tab_coef;
  int32_t tab_cap;      // power of two
  int32_t *tab_count;   // distinct keys stored
  // bucketing of table modes by bin
  int32_t *bkt_count;   // bins_cap
  int32_t *bkt_start;   // bins_cap
  int32_t *bkt_list;    // tab_cap
  // candidates of this iteration
  int32_t *cand_valid;  // bins_cap
  int32_t *cand_k0;
  double2 *cand_coef;
  int32_t *flags;       // [0] found this iteration, [1] status bits
};

// ---------------------------------------------------------------- helpers
__host__ __device__ inline int64_t PosMod(int64_t v, int64_t n) {
  v %= n;
  return v < 0 ? v + n : v;
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

// SampleInFreq (src/window.cc:77-81): window response at offset xi.
__device__ inline double WindowInFreq(const SigIter &it, double xi) {
  const double c = 0.5 * it.width;
  return 0.5 * (erf((xi + c) * it.erf_d) - erf((xi - c) * it.erf_d));
}

// 2x2 matrix pencil [[u0, u2], [u1, u0]] (src/freqid.cc:27-48), FP64.
// sigma0 = sqrt(largest eigenvalue of A^H A), sigma1 = |det A| / sigma0.
// The vote Im(conj(v00) v10) < 0 of the dominant right singular vector v
// reduces to Im(m01) > 0 with m01 = conj(u0) u2 + conj(u1) u0 (the
// off-diagonal of A^H A); the eigenvector is built the same way as in the
// oracle so that degenerate cases (m01 = 0) agree.
__device__ inline bool Pencil(double2 u0, double2 u1, double2 u2,
                              double *s0_out, double *s1_out) {
  const double m00 = u0.x * u0.x + u0.y * u0.y + u1.x * u1.x + u1.y * u1.y;
  const double m11 = u2.x * u2.x + u2.y * u2.y + u0.x * u0.x + u0.y * u0.y;
  const double2 m01 = cadd(cmul(cconj(u0), u2), cmul(cconj(u1), u0));
  const double hd = 0.5 * (m00 - m11);
  const double nm01 = m01.x * m01.x + m01.y * m01.y;
  const double r = sqrt(hd * hd + nm01);
  const double lmax = 0.5 * (m00 + m11) + r;
  const double s0 = sqrt(lmax > 0 ? lmax : 0.0);
  const double2 det = csub(cmul(u0, u0), cmul(u2, u1));
  const double adet = hypot(det.x, det.y);
  *s0_out = s0;
  *s1_out = s0 > 0 ? adet / s0 : 0.0;
  double2 v0, v1;
  if (nm01 == 0.0) {
    v0 = make_double2(m00 >= m11 ? 1.0 : 0.0, 0.0);
    v1 = make_double2(m00 >= m11 ? 0.0 : 1.0, 0.0);
  } else if (m00 >= m11) {
    v0 = make_double2(lmax - m11, 0.0);
    v1 = cconj(m01);
  } else {
    v0 = m01;
    v1 = make_double2(lmax - m00, 0.0);
  }
  // Im(conj(v0) v1); normalisation does not change its sign.
  return (v0.x * v1.y - v0.y * v1.x) < 0;
}

// Hash slot of a mode key (Fibonacci hashing into a power-of-two table).
__device__ inline uint32_t KeySlot(int32_t k, int32_t cap) {
  return (uint32_t(k) * 2654435769u) & uint32_t(cap - 1);
}

}  // namespace mpsft
