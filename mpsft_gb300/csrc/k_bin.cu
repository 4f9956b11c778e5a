// Time-domain binning: gather, window, modulate and fold (the part of
// BinInTime::Run before the size-B FFT, src/binner.cc:394-507).
//
// Row tau of the bin matrix is U_tau[k] = e^{2 pi i b q/n} * DFT_B(F_tau)[k]
// with the fold
//   F_tau[beta] = sum_{t = beta mod B, |t| <= p2}
//                 x[(a (tau + t) + c) mod n] * wt(t)
//                 * e^{2 pi i ((b (t + off) mod n)/n - t/(2B))},
// tau = q + off. For the pair q +- off (off = B 2^s) the sample of row q - off
// at -t is x[(a (q - t - off) + c) mod n] * wt(t) * conj(phase(t)), so one
// phase per t serves both rows (the symmetry of BinInTimeV1/V4,
// src/binner.cc:116-138), and it lands in bin (-beta) mod B.
//
// Work decomposition: one CTA per (32 bins, row group, trial, signal); eight
// lanes share a bin and split its f = p/B folds (t, t + 8B, ...). Indices
// step exactly in uint32 (j += a*8B mod n with one conditional subtract), so no
// 64-bit division runs per sample. FP32: the phase is carried in 32-bit
// fixed-point turns (exact reduction mod 1 by wrap-around) and converted only
// for sincospif; products in FP32; the per-lane sums and the 8-lane tree use
// compensated (TwoSum) addition. FP64: per-sample double phase and sincospi,
// plain sums (the straightforward port).
#include "common.cuh"
#include "launch.h"

namespace mpsft {

namespace {

struct CompF {
  float s = 0.f, c = 0.f;
  __device__ void add(float v) {
    const float t = s + v;
    const float bp = t - s;
    c += (s - (t - bp)) + (v - bp);
    s = t;
  }
  __device__ void merge(float os, float oc) {
    const float t = s + os;
    const float bp = t - s;
    c += oc + ((s - (t - bp)) + (os - bp));
    s = t;
  }
};

template <typename TX> __device__ inline float2 to_f2(TX v);
template <> __device__ inline float2 to_f2<float2>(float2 v) { return v; }
template <> __device__ inline float2 to_f2<double2>(double2 v) {
  return make_float2(float(v.x), float(v.y));
}
template <typename TX> __device__ inline double2 to_d2x(TX v);
template <> __device__ inline double2 to_d2x<float2>(float2 v) {
  return make_double2(v.x, v.y);
}
template <> __device__ inline double2 to_d2x<double2>(double2 v) { return v; }

// Per-lane setup shared by both precisions.
struct LaneSetup {
  int cnt;          // folds handled by this lane
  int64_t t;        // first t of this lane
  uint32_t j1, j2;  // gather indices of rows q + off and q - off
  uint32_t m;       // (b (t + off)) mod n
  uint32_t a8, m8;  // per-step increments (step 8B in t)
};

__device__ inline LaneSetup MakeLane(const SigIter &it, int beta, int lane8,
                                     bool valid, int64_t off, int64_t q) {
  LaneSetup L;
  const int B = it.bins;
  const int64_t n = it.n;
  const int f = it.folds;
  // t = beta mod B and |t| <= p2; -p2 = (B + 1)/2 mod B since p = f B, f odd.
  const int tmin = -it.p2 + int(PosMod(int64_t(beta) - (B + 1) / 2, B));
  L.t = tmin + int64_t(lane8) * B;
  L.cnt = (valid && f > lane8) ? (f - lane8 + kFoldLanes - 1) / kFoldLanes : 0;
  const int64_t a = it.a, b = it.b, c = it.c;
  L.j1 = uint32_t(PosMod(a * PosMod(q + L.t + off, n) + c, n));
  L.j2 = uint32_t(PosMod(a * PosMod(q - L.t - off, n) + c, n));
  L.m = uint32_t(PosMod(b * PosMod(L.t + off, n), n));
  const int64_t s8 = PosMod(int64_t(kFoldLanes) * B, n);
  L.a8 = uint32_t(PosMod(a * s8, n));
  L.m8 = uint32_t(PosMod(b * s8, n));
  return L;
}

__device__ inline uint32_t StepUp(uint32_t j, uint32_t d, uint32_t n) {
  j += d;
  return j >= n ? j - n : j;
}
__device__ inline uint32_t StepDown(uint32_t j, uint32_t d, uint32_t n) {
  return j >= d ? j - d : j + (n - d);
}

template <typename TX>
__global__ void __launch_bounds__(256)
    k_bin_fold32(const SigIter *__restrict__ its, int gmax) {
  const SigIter &it = its[blockIdx.z];
  if (!it.active || it.force_fp64) return;
  const int B = it.bins;
  if (int(blockIdx.x) * 32 >= B) return;
  const int g = blockIdx.y % gmax;
  const int tr = blockIdx.y / gmax;
  if (tr >= it.trials || g > it.bits) return;

  const int lane8 = threadIdx.x & (kFoldLanes - 1);
  const int beta = blockIdx.x * 32 + (threadIdx.x >> 3);
  const bool valid = beta < B;
  const uint32_t n = uint32_t(it.n);
  const int64_t off = g == 0 ? 0 : (int64_t(B) << (g - 1));
  const LaneSetup L = MakeLane(it, beta, lane8, valid, off, it.q[tr]);

  // Phase in 32-bit fixed-point turns: m/n - t/(2B). Exact reduction mod 1 by
  // uint32 wrap-around; the step adds (m8/n) * 2^32 rounded (error < 2^-32
  // turns per fold).
  const uint64_t twoB = 2ull * uint64_t(B);
  const uint32_t ph_m = uint32_t((uint64_t(L.m) << 32) / n);
  const uint64_t tmod = uint64_t(PosMod(L.t, int64_t(twoB)));
  const uint32_t ph_t = uint32_t(((tmod << 32) + twoB / 2) / twoB);
  const uint32_t dph = uint32_t(((uint64_t(L.m8) << 32) + n / 2) / n);
  uint32_t ph = ph_m - ph_t;  // lane constant -t/(2B) is unchanged by 8B steps

  const TX *__restrict__ x = reinterpret_cast<const TX *>(it.x);
  const float *__restrict__ wt = it.wt32;
  const bool pair = g > 0;

  TX x1[kMaxFoldsPerLane], x2[kMaxFoldsPerLane];
  uint32_t phs[kMaxFoldsPerLane];
  int ta[kMaxFoldsPerLane];
  {
    uint32_t j1 = L.j1, j2 = L.j2;
    int64_t t = L.t;
#pragma unroll
    for (int k = 0; k < kMaxFoldsPerLane; ++k) {
      if (k < L.cnt) {
        x1[k] = __ldg(&x[j1]);
        if (pair) x2[k] = __ldg(&x[j2]);
        phs[k] = ph;
        ta[k] = int(t < 0 ? -t : t);
        j1 = StepUp(j1, L.a8, n);
        j2 = StepDown(j2, L.a8, n);
        ph += dph;
        t += int64_t(kFoldLanes) * B;
      }
    }
  }
  CompF r1, i1, r2, i2;
#pragma unroll
  for (int k = 0; k < kMaxFoldsPerLane; ++k) {
    if (k < L.cnt) {
      const float phi = float(int32_t(phs[k])) * 2.3283064365386963e-10f;
      float s, c;
      sincospif(2.0f * phi, &s, &c);
      const float w = __ldg(&wt[ta[k]]);
      const float wr = c * w, wi = s * w;
      const float2 v1 = to_f2(x1[k]);
      r1.add(v1.x * wr - v1.y * wi);
      i1.add(v1.x * wi + v1.y * wr);
      if (pair) {
        const float2 v2 = to_f2(x2[k]);
        r2.add(v2.x * wr + v2.y * wi);
        i2.add(v2.y * wr - v2.x * wi);
      }
    }
  }
#pragma unroll
  for (int o = 1; o < kFoldLanes; o <<= 1) {
    r1.merge(__shfl_xor_sync(0xffffffffu, r1.s, o),
             __shfl_xor_sync(0xffffffffu, r1.c, o));
    i1.merge(__shfl_xor_sync(0xffffffffu, i1.s, o),
             __shfl_xor_sync(0xffffffffu, i1.c, o));
    if (pair) {
      r2.merge(__shfl_xor_sync(0xffffffffu, r2.s, o),
               __shfl_xor_sync(0xffffffffu, r2.c, o));
      i2.merge(__shfl_xor_sync(0xffffffffu, i2.s, o),
               __shfl_xor_sync(0xffffffffu, i2.c, o));
    }
  }
  if (lane8 == 0 && valid) {
    float2 *fold = reinterpret_cast<float2 *>(it.fold);
    const size_t base = size_t(tr) * it.rows;
    const int rplus = g == 0 ? 0 : 2 * g - 1;
    fold[(base + rplus) * it.bins_cap + beta] =
        make_float2(r1.s + r1.c, i1.s + i1.c);
    if (pair) {
      const int bneg = beta == 0 ? 0 : B - beta;
      fold[(base + 2 * g) * it.bins_cap + bneg] =
          make_float2(r2.s + r2.c, i2.s + i2.c);
    }
  }
}

// cond: only signals whose iteration is redone in FP64 take part.
template <typename TX>
__global__ void __launch_bounds__(256)
    k_bin_fold64(const SigIter *__restrict__ its, int gmax, int cond) {
  const SigIter &it = its[blockIdx.z];
  if (!it.active) return;
  if (cond ? !RedoFP64(it) : it.force_fp64) return;
  const int B = it.bins;
  if (int(blockIdx.x) * 32 >= B) return;
  const int g = blockIdx.y % gmax;
  const int tr = blockIdx.y / gmax;
  if (tr >= it.trials || g > it.bits) return;

  const int lane8 = threadIdx.x & (kFoldLanes - 1);
  const int beta = blockIdx.x * 32 + (threadIdx.x >> 3);
  const bool valid = beta < B;
  const uint32_t n = uint32_t(it.n);
  const int64_t off = g == 0 ? 0 : (int64_t(B) << (g - 1));
  const LaneSetup L = MakeLane(it, beta, lane8, valid, off, it.q[tr]);
  const int64_t twoB = 2 * int64_t(B);
  // -t/(2B) mod 1 is the same for every fold of this lane.
  const double ct = -double(PosMod(L.t, twoB)) / double(twoB);
  const double inv_n = 1.0 / double(n);

  const TX *__restrict__ x = reinterpret_cast<const TX *>(it.x);
  const double *__restrict__ wt = it.wt64;
  const bool pair = g > 0;

  double r1 = 0, i1 = 0, r2 = 0, i2 = 0;
  uint32_t j1 = L.j1, j2 = L.j2, m = L.m;
  int64_t t = L.t;
  for (int k = 0; k < L.cnt; ++k) {
    const double2 v1 = to_d2x(__ldg(&x[j1]));
    double2 v2 = make_double2(0, 0);
    if (pair) v2 = to_d2x(__ldg(&x[j2]));
    double s, c;
    sincospi(2.0 * (double(m) * inv_n + ct), &s, &c);
    const double w = __ldg(&wt[t < 0 ? -t : t]);
    const double wr = c * w, wi = s * w;
    r1 += v1.x * wr - v1.y * wi;
    i1 += v1.x * wi + v1.y * wr;
    if (pair) {
      r2 += v2.x * wr + v2.y * wi;
      i2 += v2.y * wr - v2.x * wi;
    }
    j1 = StepUp(j1, L.a8, n);
    j2 = StepDown(j2, L.a8, n);
    m = StepUp(m, L.m8, n);
    t += int64_t(kFoldLanes) * B;
  }
#pragma unroll
  for (int o = 1; o < kFoldLanes; o <<= 1) {
    r1 += __shfl_xor_sync(0xffffffffu, r1, o);
    i1 += __shfl_xor_sync(0xffffffffu, i1, o);
    r2 += __shfl_xor_sync(0xffffffffu, r2, o);
    i2 += __shfl_xor_sync(0xffffffffu, i2, o);
  }
  if (lane8 == 0 && valid) {
    double2 *fold = reinterpret_cast<double2 *>(it.fold);
    const size_t base = size_t(tr) * it.rows;
    const int rplus = g == 0 ? 0 : 2 * g - 1;
    fold[(base + rplus) * it.bins_cap + beta] = make_double2(r1, i1);
    if (pair) {
      const int bneg = beta == 0 ? 0 : B - beta;
      fold[(base + 2 * g) * it.bins_cap + bneg] = make_double2(r2, i2);
    }
  }
}

}  // namespace

void LaunchBinFold(const SigIter *d_its, int nsig, int max_bins, int max_bits,
                   int max_trials, bool x_c128, bool fp64, cudaStream_t s,
                   bool cond) {
  const int gmax = max_bits + 1;
  dim3 grid((max_bins + 31) / 32, gmax * max_trials, nsig);
  if (fp64) {
    if (x_c128) {
      k_bin_fold64<double2><<<grid, 256, 0, s>>>(d_its, gmax, cond ? 1 : 0);
    } else {
      k_bin_fold64<float2><<<grid, 256, 0, s>>>(d_its, gmax, cond ? 1 : 0);
    }
  } else {
    if (x_c128) {
      k_bin_fold32<double2><<<grid, 256, 0, s>>>(d_its, gmax);
    } else {
      k_bin_fold32<float2><<<grid, 256, 0, s>>>(d_its, gmax);
    }
  }
}

}  // namespace mpsft
