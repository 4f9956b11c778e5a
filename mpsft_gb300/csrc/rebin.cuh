// Preparation of a near-tie bin's re-binning (the FP32 path lists bins whose
// decisions lie within their rounding bound of a threshold): the powers of
// its phase step and cleared arrival counters.
#pragma once

#include "common.cuh"

namespace mpsft {

namespace {

struct FF {
  float hi, lo;
};

__device__ __forceinline__ FF FFOf(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - double(h))};
}

constexpr int kPowLen = 64;  // s^k table length = block of samples (2 per lane)

// e^{2 pi i (m/n - r/(2B))} for residues m mod n and r mod 2B: from the
// phase tables (e^{2 pi i m/n}) and the bins-grid roots r2b64 = e^{-pi i r/B}
// (one product), or by a direct FP64 sincospi where the solve tables are
// absent (the direct evaluation of every bin).
__device__ inline double2 StepPhase(const SigIter &it, int64_t m, int64_t r) {
  if (it.r2b64 != nullptr) return cmul(Phase64(it, m), it.r2b64[r]);
  double s, c;
  sincospi(2.0 * (double(m) / double(it.n) - double(r) / double(2 * int64_t(it.bins))),
           &s, &c);
  return make_double2(c, s);
}

// Phase e^{2 pi i k Delta} from exact integer reductions:
// k Delta = (k b mod n)/n - (k (2 beta + 1) mod 2B)/(2B) (mod 1), for
// 0 <= k <= kPowLen and b = it.b mod n.
__device__ inline double2 PowerOfStep(const SigIter &it, int64_t k, uint32_t b,
                                      int64_t g) {
  const ModN mod{uint32_t(it.n), it.n_inv};
  const int64_t twoB = 2 * int64_t(it.bins);
  return StepPhase(it, mod(k * int64_t(b)), (k * g) % twoB);
}

// Listed bin e: its (trial, row) arrival counters cleared, by the lanes of
// one warp.
__device__ inline void ClearListedBin(const SigIter &it, int e, int lane) {
  for (int i = lane; i < it.trials * it.rows; i += 32) {
    it.esc_cnt[size_t(e) * it.trials * it.rows + i] = 0;
  }
}

// s^k of bin beta's phase step s = e^{2 pi i (b/n - (2 beta + 1)/(2B))}, lane
// k and k + 32, as float-float complex {re.hi, im.hi, re.lo, im.lo}, and
// s^64 in FP64.
__device__ inline void StepPowers(const SigIter &it, int beta, int lane, float4 *p0,
                                  float4 *p1, double2 *s64) {
  const ModN mod{uint32_t(it.n), it.n_inv};
  const uint32_t bm = mod(it.b);
  const int64_t g = 2 * int64_t(beta) + 1;
  const double2 z0 = PowerOfStep(it, lane, bm, g);
  const double2 z1 = PowerOfStep(it, lane + 32, bm, g);
  *s64 = PowerOfStep(it, kPowLen, bm, g);
  FF zr = FFOf(z0.x), zi = FFOf(z0.y);
  *p0 = make_float4(zr.hi, zi.hi, zr.lo, zi.lo);
  zr = FFOf(z1.x);
  zi = FFOf(z1.y);
  *p1 = make_float4(zr.hi, zi.hi, zr.lo, zi.lo);
}

// A listed bin's preparation: its counters, and its phase-step powers once
// into esc_pow / esc_step (by the FP32 decide that lists it; for the direct
// evaluation of every bin, without solve tables, by k_rebin_prep with an
// FP64 sincospi per power).
__device__ __noinline__ void PrepListedBin(const SigIter &it, int e, int beta,
                                           int lane) {
  ClearListedBin(it, e, lane);
  float4 p0, p1;
  double2 s64;
  StepPowers(it, beta, lane, &p0, &p1, &s64);
  it.esc_pow[size_t(e) * kPowLen + lane] = p0;
  it.esc_pow[size_t(e) * kPowLen + lane + 32] = p1;
  if (lane == 0) it.esc_step[e] = s64;
}

}  // namespace

}  // namespace mpsft
