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

constexpr int kPowLen = 64;  // s^k table length = block of samples

// Phase e^{2 pi i k Delta} from exact integer reductions:
// k Delta = (k b mod n)/n - (k (2 beta + 1) mod 2B)/(2B) (mod 1).
__device__ inline double2 PowerOfStep(int64_t k, int64_t b, int64_t g,
                                      int64_t n, int64_t twoB) {
  const int64_t m = PosMod(k * b, n);
  const int64_t r = PosMod(k * g, twoB);
  double s, c;
  sincospi(2.0 * (double(m) / double(n) - double(r) / double(twoB)), &s, &c);
  return make_double2(c, s);
}

// Listed bin e (bin beta), one warp: with
// s = e^{2 pi i (b/n - (2 beta + 1)/(2B))}, s^k for k < 64 as float-float
// complex {re.hi, im.hi, re.lo, im.lo} and s^64 in FP64; the (trial, row)
// arrival counters cleared; the FP64 terms of the bin's found modes (a
// solve's lists carry a row mask; the direct evaluation of every bin has
// neither modes nor mask). Not inlined: the FP32 decide kernel calls it for
// the few bins it lists, after their decision.
__device__ __noinline__ void PrepListedBin(const SigIter &it, int e, int beta,
                                           int lane) {
  const int64_t n = it.n, twoB = 2 * int64_t(it.bins);
  const int64_t b = PosMod(it.b, n);
  const int64_t g = 2 * int64_t(beta) + 1;
  for (int i = lane; i < it.trials * it.rows; i += 32) {
    it.esc_cnt[size_t(e) * it.trials * it.rows + i] = 0;
  }
  float4 *pw = it.esc_pow + size_t(e) * kPowLen;
  for (int k = lane; k < kPowLen; k += 32) {
    const double2 z = PowerOfStep(k, b, g, n, twoB);
    const FF zr = FFOf(z.x), zi = FFOf(z.y);
    pw[k] = make_float4(zr.hi, zi.hi, zr.lo, zi.lo);
  }
  if (lane == 0) it.esc_step[e] = PowerOfStep(kPowLen, b, g, n, twoB);
  if (it.esc_mask == nullptr) return;
  const int nm = it.bkt_count[beta], st = it.bkt_start[beta];
  for (int i = lane; i < nm; i += 32) {
    const int sl = it.bkt_list[st + i];
    ModeTerms64(it, sl, it.mode_k1[sl], it.mode_bin[sl]);
  }
}

}  // namespace

}  // namespace mpsft
