// Preparation of a near-tie bin's re-binning (the FP32 path lists bins whose
// decisions lie within their rounding bound of a threshold): the per-bin
// table of powers of the phase step, its 64th power, cleared arrival
// counters, and the FP64 row-0 terms of the bin's found modes for its FP64
// decision.
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
// k Delta = (k b mod n)/n - (k (2 beta + 1) mod 2B)/(2B) (mod 1).
__device__ inline double2 PowerOfStep(const SigIter &it, int64_t k, int64_t b,
                                      int64_t g) {
  const int64_t n = it.n, twoB = 2 * int64_t(it.bins);
  return StepPhase(it, PosMod(k * b, n), PosMod(k * g, twoB));
}

// Listed bin e (bin beta), one warp: with
// s = e^{2 pi i (b/n - (2 beta + 1)/(2B))}, s^k for k < 64 as float-float
// complex {re.hi, im.hi, re.lo, im.lo} and s^64 in FP64; the (trial, row)
// arrival counters cleared. (A solve's FP64 terms of the bin's found modes
// come from k_listed_terms, beside the re-binning.) Not inlined: the FP32
// decide kernel calls it for the few bins it lists, after their decision.
__device__ __noinline__ void PrepListedBin(const SigIter &it, int e, int beta,
                                           int lane) {
  const int64_t b = PosMod(it.b, int64_t(it.n));
  const int64_t g = 2 * int64_t(beta) + 1;
  for (int i = lane; i < it.trials * it.rows; i += 32) {
    it.esc_cnt[size_t(e) * it.trials * it.rows + i] = 0;
  }
  float4 *pw = it.esc_pow + size_t(e) * kPowLen;
  // lanes 0..31: s^lane and s^(lane + 32); lane 0 also s^64
  const double2 z0 = PowerOfStep(it, lane, b, g);
  const double2 z1 = PowerOfStep(it, lane + 32, b, g);
  const double2 z64 = PowerOfStep(it, kPowLen, b, g);
  FF zr = FFOf(z0.x), zi = FFOf(z0.y);
  pw[lane] = make_float4(zr.hi, zi.hi, zr.lo, zi.lo);
  zr = FFOf(z1.x);
  zi = FFOf(z1.y);
  pw[lane + 32] = make_float4(zr.hi, zi.hi, zr.lo, zi.lo);
  if (lane == 0) it.esc_step[e] = z64;
}

}  // namespace

}  // namespace mpsft
