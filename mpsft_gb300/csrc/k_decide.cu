// Found-mode preparation and bucketing, frequency-domain subtraction of found
// modes, per-bin identification and coefficient estimation, and the merge of
// the new modes into the table.
//
// Reference: BinInFreqV1::Run (src/binner.cc:565-591), the bin loop of
// Iterate (src/iterate.cc:113-175), IdentifyFreq (src/iterate.cc:44-76) and
// MatPencil (src/freqid.cc:27-48).
//
// k_mode_prep (one thread per table slot) evaluates, once per mode and
// iteration, what BinInFreq needs from a mode: k1 = (a k0 + b) mod n, its bin,
// the window response wf (two FP64 erf) and, per trial, the row-0 term
// wf * coef * e^{2 pi i (q k1 + c k0)/n}. k_bucket (one CTA per signal) sorts
// the slots by bin. k_decide then works with one warp per (bin, signal):
// every lane holds row 0, lane s holds rows 2s+1 and 2s+2 (bit s). A bin's
// modes are subtracted in increasing k0, so the result does not depend on the
// table layout. The energy test runs on row 0 before anything else, so bins
// without energy cost a few instructions.
//
// Precision: the FP64 path decides in FP64. The FP32 path decides in FP32 and
// checks every decision against eps, an upper bound on the bins' FP32
// rounding error (plus the error carried by the modes it subtracted); a
// decision closer than eps to its threshold lists the bin for FP64 treatment.
#include <algorithm>

#include "common.cuh"
#include "launch.h"

namespace mpsft {

namespace {

// ---------------------------------------------------------------- prep
// One thread per occupied slot (the table's insertion list): k1 = (a k0 + b)
// mod n and the mode's bin for the bucketing, and the row-0 term
// wf c e^{2 pi i (q_t k1 + c k0)/n} of every trial (BinInFreqV1::Run,
// src/binner.cc:565-591) in FP64 (unit phases from the FP64 tables). The
// FP32 path also gets FP32 terms, computed in FP32, together with the error
// the mode carries into its bin: the coefficient's bound tab_err |wf| plus
// 8 eps_rel |wf c| for the FP32 window response, phase, rounding and
// subtraction (each a few 2^-24 relative).
__device__ inline float WindowInFreq32(const SigIter &it, int64_t k1, int bin) {
  // xi +- 1/(4B) with xi = (bin + 1/2)/B - k1/n, as exact integers over 4nB
  const int64_t n = it.n, B4 = 4 * int64_t(it.bins);
  const int64_t np = (4 * int64_t(bin) + 3) * n - k1 * B4;
  const int64_t nm = (4 * int64_t(bin) + 1) * n - k1 * B4;
  return 0.5f * (erff(float(np) * it.wf_scale) - erff(float(nm) * it.wf_scale));
}

__global__ void k_mode_prep(const SigIter *__restrict__ its, int cond) {
  const SigIter &it = its[blockIdx.y];
  if (!it.active) return;
  if (cond && !RedoFP64(it)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *it.tab_count) return;
  const int s = it.occ_list[i];
  const int32_t key = it.tab_key[s];
  const int64_t n = it.n;
  const int B = it.bins;
  const ModN mod{uint32_t(n), it.n_inv};
  const int64_t k1 = mod(int64_t(it.a) * key + it.b);
  const int bin = int(mod.quot(k1 * B));
  it.mode_k1[s] = int32_t(k1);
  it.mode_bin[s] = bin;
  const bool fp32 = it.eps_rel > 0.f && !it.force_fp64 && !cond;
  if (fp32) {
    const float wf = WindowInFreq32(it, k1, bin);
    const double2 cd = it.tab_coef[s];
    const float2 wc = make_float2(float(cd.x) * wf, float(cd.y) * wf);
    for (int t = 0; t < it.trials; ++t) {
      const int64_t ph = int64_t(it.q[t]) * k1 + int64_t(it.c) * key;
      it.mode_base32[size_t(s) * it.trials + t] = cmulf(wc, Phase32(it, ph));
    }
    it.mode_errw[s] = float(it.tab_err[s]) * fabsf(wf) +
                      8.f * it.eps_rel * sqrtf(wc.x * wc.x + wc.y * wc.y);
  } else {
    ModeTerms64(it, s, k1, bin);
  }
}

// Ascending bitonic sort of keys[0..m) in shared memory (m a power of two),
// by the whole block; ends with a barrier.
__device__ void BitonicSort(unsigned long long *keys, int m) {
  for (int size = 2; size <= m; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;
          const unsigned long long a = keys[i], b = keys[j];
          if ((a > b) == up) {
            keys[i] = b;
            keys[j] = a;
          }
        }
      }
      __syncthreads();
    }
  }
}

// Sorts the occupied slots by (bin, k0): one 64-bit key per slot,
// bin << 51 | k0 << 20 | slot (bins < 2^13, k0 < 2^31, slots < 2^20), bitonic
// sort in shared memory, then per-bin start and count from the run
// boundaries. The subtraction later walks each bin's modes in increasing k0,
// an order that does not depend on the table layout. Thread 0 also evaluates
// this iteration's FP32 error scale eps.
__global__ void __launch_bounds__(1024) k_bucket(const SigIter *__restrict__ its) {
  extern __shared__ unsigned long long keys[];  // pow2 >= occupied slots
  const SigIter &it = its[blockIdx.x];
  if (!it.active) return;
  const int B = it.bins;
  const int occ = *it.tab_count;
  if (threadIdx.x == 0 && it.eps_scale > 0) {
    *it.eps_dev = float(it.eps_scale * sqrt(*it.x_energy));
  }
  // shared keys were sized for half the table (BucketKeys); more occupied
  // slots end the solve with a capacity status instead of overflowing
  if (occ > BucketKeys(it.tab_cap)) {
    if (threadIdx.x == 0) atomicOr(&it.flags[1], kStatusCapacity);
    return;
  }
  int m = 1;
  while (m < occ) m <<= 1;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    unsigned long long k = ~0ull;
    if (i < occ) {
      const int s = it.occ_list[i];
      k = (static_cast<unsigned long long>(it.mode_bin[s]) << 51) |
          (static_cast<unsigned long long>(uint32_t(it.tab_key[s])) << 20) |
          static_cast<unsigned long long>(s);
    }
    keys[i] = k;
  }
  for (int i = threadIdx.x; i < B; i += blockDim.x) it.bkt_count[i] = 0;
  __syncthreads();
  BitonicSort(keys, m);
  __syncthreads();  // also orders the bkt_count zeroing when occ <= 1
  for (int i = threadIdx.x; i < occ; i += blockDim.x) {
    const unsigned long long k = keys[i];
    const int bin = int(k >> 51);
    it.bkt_list[i] = int32_t(k & 0xFFFFFu);
    if (i == 0 || int(keys[i - 1] >> 51) != bin) {
      // first slot of its bin: the run ends at the next bin change
      int e = i + 1;
      while (e < occ && int(keys[e] >> 51) == bin) ++e;
      it.bkt_start[bin] = i;
      it.bkt_count[bin] = e - i;
    }
  }
}

// ---------------------------------------------------------------- decide
template <typename T> struct Ops;
template <> struct Ops<float> {
  using V = float2;
  __device__ static V from(double2 d) { return make_float2(float(d.x), float(d.y)); }
  __device__ static V phase(const SigIter &it, int64_t m) { return Phase32(it, m); }
  // row-0 terms of a found mode, from k_mode_prep's FP32 copies
  template <int TMAX>
  __device__ static void terms(const SigIter &it, int sl, V *out) {
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < it.trials) out[t] = it.mode_base32[size_t(sl) * it.trials + t];
    }
  }
};
template <> struct Ops<double> {
  using V = double2;
  __device__ static V from(double2 d) { return d; }
  __device__ static V phase(const SigIter &it, int64_t m) { return Phase64(it, m); }
  // row-0 terms of a found mode (k_mode_prep's FP64 values)
  template <int TMAX>
  __device__ static void terms(const SigIter &it, int sl, V *out) {
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < it.trials) out[t] = it.mode_base[size_t(sl) * it.trials + t];
    }
  }
};

template <typename V> __device__ inline V vsub2(V a, V b) {
  V r;
  r.x = a.x - b.x;
  r.y = a.y - b.y;
  return r;
}
template <typename V> __device__ inline V vmul2(V a, V b) {
  V r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename V> __device__ inline V vconj2(V a) {
  V r;
  r.x = a.x;
  r.y = -a.y;
  return r;
}
template <typename T, typename V> __device__ inline T vabs2(V a) {
  return sqrt(a.x * a.x + a.y * a.y);
}

__device__ inline void Flag(const SigIter &it, int beta, uint32_t mask) {
  const int pos = atomicAdd(&it.flags[2], 1);
  if (pos < it.esc_cap) {
    it.esc_list[pos] = beta;
    if (it.esc_mask) it.esc_mask[pos] = mask;
  }
}

// Row r of a listed bin is re-binned in FP64 when it is row 0 or belongs to
// a bit whose decisions were near.
__device__ inline bool RowListed(uint32_t mask, int r) {
  return r == 0 || ((mask >> ((r - 1) >> 1)) & 1u);
}

__device__ inline void NoCandidate(const SigIter &it, int beta, int lane) {
  if (lane == 0) it.cand_valid[beta] = 0;
}

// Bin values of (trial t, row r) at bin beta, from the size-B FFT output.
struct FromBins {
  const SigIter &it;
  int beta;
  __device__ double2 get(int t, int r) const {
    return it.ubuf[(size_t(t) * it.rows + r) * it.bins_cap + beta];
  }
};

// Bin values of listed bin e: rows re-binned in FP64 (the chunk partial sums
// in their fixed order), the other rows from the FP32 pass.
struct FromRebin {
  const SigIter &it;
  int e, beta;
  uint32_t mask;
  __device__ double2 get(int t, int r) const {
    if (!RowListed(mask, r)) {
      return it.ubuf[(size_t(t) * it.rows + r) * it.bins_cap + beta];
    }
    return it.esc_sum[(size_t(e) * it.trials + t) * it.rows + r];
  }
};

enum DecideMode { kDecide = 0, kSubtractOnly = 1, kDecideExact = 2 };

// The bin loop body of Iterate for one bin (warp-wide). T = float: the FP32
// path with near-tie detection; T = double: FP64 decisions (the FP64 path, and
// the near-tie bins after their FP64 re-binning).
// k1 = round(n (beta + xi1) / B) with xi1 = (2 xs + 1) / 2^{L+1}, exactly in
// integers: num = n (beta 2^{L+1} + 2 xs + 1) < 2^64, den = B 2^{L+1} < 2^33
// (B 2^{L-1} <= n by the definition of L). The reference evaluates this in
// FP64 (relative error below 2^-52, so at most 2^-21 absolute); when the
// exact value lies within 2^-18 of a half-integer, that FP64 evaluation is
// used instead so that the rounding is the reference's.
__device__ inline int64_t RoundK1(int64_t n, int beta, uint32_t xs, int L, int B) {
  const uint64_t den = uint64_t(B) << (L + 1);
  const uint64_t num =
      uint64_t(n) * ((uint64_t(beta) << (L + 1)) + 2 * uint64_t(xs) + 1);
  const uint64_t q = num / den;
  const uint64_t r = num - q * den;
  const uint64_t d = 2 * r > den ? 2 * r - den : den - 2 * r;  // 2 den |frac - 1/2|
  if (d <= (den >> 17)) {
    const double xi1 = ldexp(2.0 * double(xs) + 1.0, -(L + 1));
    return int64_t(round(double(n) * (double(beta) + xi1) / double(B)));
  }
  return int64_t(q) + (2 * r >= den ? 1 : 0);
}

// The bin loop body of Iterate for one bin (warp-wide). T = float: the FP32
// path with near-tie detection, FP32 arithmetic only (GB300 runs FP64 at a
// small fraction of its FP32 rate): a surviving bin leaves a pending
// candidate (cand_valid = 2: k1 in cand_k0, the unscaled coefficient sum in
// cand_coef, its error bound in cand_err) that the merge finishes in FP64 on
// full warps. T = double: FP64 decisions to the end (the FP64 path, and the
// near-tie bins after their re-binning).
template <typename T, int TMAX, typename Src>
__device__ void DecideBin(const SigIter &it, int beta, const Src &src,
                          int mode) {
  using O = Ops<T>;
  using V = typename O::V;
  const int lane = threadIdx.x & 31;
  const int L = it.bits, TR = it.trials, rows = it.rows;
  const int64_t n = it.n;
  const int B = it.bins;
  const bool has_bit = lane < L;
  const bool fp32 = sizeof(T) == 4;
  const int nm = it.bkt_count[beta];
  const int st = it.bkt_start[beta];

  // ---- row 0 and its mode subtraction (the bin's modes are in increasing k0).
  // The first 32 modes are loaded once, one per lane, and shared by shuffles
  // (the common case); further modes are read directly.
  V u0[TMAX];
#pragma unroll
  for (int t = 0; t < TMAX; ++t) {
    if (t < TR) u0[t] = O::from(src.get(t, 0));
  }
  const int npre = min(nm, 32);
  V pre_base[TMAX];
  float mode_err = 0.f;  // FP32 error carried into this bin by the found modes
  if (lane < npre) {
    const int sl = it.bkt_list[st + lane];
    O::template terms<TMAX>(it, sl, pre_base);
    if (fp32) mode_err = it.mode_errw[sl];
  }
  for (int i = 0; i < nm; ++i) {
    V bs[TMAX];
    if (i < 32) {
#pragma unroll
      for (int t = 0; t < TMAX; ++t) {
        if (t < TR) {
          bs[t].x = __shfl_sync(0xffffffffu, pre_base[t].x, i);
          bs[t].y = __shfl_sync(0xffffffffu, pre_base[t].y, i);
        }
      }
    } else {
      const int sl = it.bkt_list[st + i];
      O::template terms<TMAX>(it, sl, bs);
      if (fp32 && lane == 0) mode_err += it.mode_errw[sl];
    }
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) u0[t] = vsub2(u0[t], bs[t]);
    }
  }
  if (fp32) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mode_err += __shfl_xor_sync(0xffffffffu, mode_err, o);
  }
  // FP32 error bound of this lane's values (see kEpsRms and friends)
  float eps_base = 0.f, rm0 = 0.f, rml = 0.f;
  if (fp32) {
    eps_base = *it.eps_dev + mode_err;
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        const float *rm = it.row_max + size_t(t) * rows;
        rm0 = fmaxf(rm0, rm[0]);
        if (has_bit) rml = fmaxf(rml, fmaxf(rm[2 * lane + 1], rm[2 * lane + 2]));
      }
    }
    rml = fmaxf(rml, rm0);
  }
  bool e_near = false;  // energy decision near its threshold (warp-uniform)

  if (mode != kSubtractOnly) {
    // ---- energy threshold (src/iterate.cc:114-124) on row 0 only
    T e = 0;
    T amax = 0;
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        e += u0[t].x * u0[t].x + u0[t].y * u0[t].y;
        amax = max(amax, vabs2<T, V>(u0[t]));
      }
    }
    e /= T(TR);
    if (!isfinite(e)) {
      if (lane == 0) {
        atomicOr(&it.flags[1], kStatusNonFinite);
        it.cand_valid[beta] = 0;
      }
      return;
    }
    if (fp32 ? it.bin_thr2_f > 0.f : it.bin_thr > 0) {
      T thr2;
      if (fp32) {
        thr2 = it.bin_thr2_f;
        const T eps0 = T(eps_base + it.eps_rel * (kEpsRowMax * rm0 +
                                                  kEpsValue * float(amax)));
        // |d e| <= 2 max|u0| eps + eps^2, plus the threshold's FP32 rounding
        e_near = fabs(e - thr2) <= T(2) * amax * eps0 + eps0 * eps0 +
                                       thr2 * T(1.2e-7);
      } else {
        thr2 = T(it.bin_thr * it.bin_thr);
      }
      if (e < thr2) {
        if (e_near && lane == 0) Flag(it, beta, 0u);
        NoCandidate(it, beta, lane);
        return;
      }
    }
  }

  // ---- rows 2s+1, 2s+2 of this lane's bit and their mode subtraction
  V up[TMAX], um[TMAX];
#pragma unroll
  for (int t = 0; t < TMAX; ++t) {
    if (t < TR) {
      if (has_bit) {
        up[t] = O::from(src.get(t, 2 * lane + 1));
        um[t] = O::from(src.get(t, 2 * lane + 2));
      } else {
        up[t].x = up[t].y = um[t].x = um[t].y = T(0);
      }
    }
  }
  const int64_t off = has_bit ? (int64_t(B) << lane) : 0;
  for (int i = 0; i < nm; ++i) {
    V bs[TMAX];
    if (i < 32) {
#pragma unroll
      for (int t = 0; t < TMAX; ++t) {
        if (t < TR) {
          bs[t].x = __shfl_sync(0xffffffffu, pre_base[t].x, i);
          bs[t].y = __shfl_sync(0xffffffffu, pre_base[t].y, i);
        }
      }
    } else {
      const int sl = it.bkt_list[st + i];
      O::template terms<TMAX>(it, sl, bs);
    }
    if (has_bit) {
      // row factor e^{2 pi i (B 2^s k1 mod n)/n} of this lane's bit
      // (src/binner.cc:584-589)
      const int sl = it.bkt_list[st + i];
      const V fac = O::phase(it, off * int64_t(it.mode_k1[sl]));
#pragma unroll
      for (int t = 0; t < TMAX; ++t) {
        if (t < TR) {
          up[t] = vsub2(up[t], vmul2(bs[t], fac));
          um[t] = vsub2(um[t], vmul2(bs[t], vconj2(fac)));
        }
      }
    }
  }
  if (mode == kSubtractOnly) {
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        double2 *base = it.ubuf + size_t(t) * rows * it.bins_cap;
        if (lane == 0) base[beta] = make_double2(u0[t].x, u0[t].y);
        if (has_bit) {
          base[(2 * lane + 1) * it.bins_cap + beta] = make_double2(up[t].x, up[t].y);
          base[(2 * lane + 2) * it.bins_cap + beta] = make_double2(um[t].x, um[t].y);
        }
      }
    }
    return;
  }

  // ---- non-finite input is reported instead of being voted on
  bool finite = true;
#pragma unroll
  for (int t = 0; t < TMAX; ++t) {
    if (t < TR) {
      finite = finite && isfinite(up[t].x) && isfinite(up[t].y) &&
               isfinite(um[t].x) && isfinite(um[t].y);
    }
  }
  if (__any_sync(0xffffffffu, !finite)) {
    if (lane == 0) {
      atomicOr(&it.flags[1], kStatusNonFinite);
      it.cand_valid[beta] = 0;
    }
    return;
  }

  // ---- IdentifyFreq: per-bit majority of the pencil votes, sv rejection
  int count = 0;
  bool sv_fail = false, near = false;
  if (has_bit) {
    const T sv_thr = fp32 ? T(it.sv_thr_f) : T(it.sv_thr);
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        T s0, s1, im;
        if (fp32) {
          if (PencilT<T, V>(u0[t], up[t], um[t], &s0, &s1, &im)) ++count;
          if (sv_thr > T(0) && s1 * T(0.5) > sv_thr) sv_fail = true;
        } else {
          // sigma1 / 2 > sv_thr as |det|^2 > 4 sv_thr^2 sigma0^2 (one square
          // root instead of three and a division)
          T det2, lmax;
          if (PencilSq<T, V>(u0[t], up[t], um[t], &det2, &lmax, &im)) ++count;
          if (sv_thr > T(0) && det2 > T(4) * sv_thr * sv_thr * lmax) sv_fail = true;
        }
        if (fp32) {
          const T a0 = vabs2<T, V>(u0[t]), a1 = vabs2<T, V>(up[t]),
                  a2 = vabs2<T, V>(um[t]);
          const T eps = T(eps_base + it.eps_rel * (kEpsRowMax * rml +
                                                   kEpsValue * float(max(a0, max(a1, a2)))));
          // |d Im(m01)| <= eps (2|u0| + |u1| + |u2|) + 4 eps^2;
          // |d sigma1| <= ||dA||_2 <= 2 eps, plus the threshold's rounding.
          if (fabs(im) <= eps * (T(2) * a0 + a1 + a2) + T(4) * eps * eps) near = true;
          if (sv_thr > T(0) &&
              fabs(s1 * T(0.5) - sv_thr) <= eps + sv_thr * T(1.2e-7)) {
            near = true;
          }
        }
      }
    }
  }
  if (fp32) {
    const uint32_t near_bits = __ballot_sync(0xffffffffu, has_bit && near);
    if ((near_bits || e_near) && lane == 0) Flag(it, beta, near_bits);
  }
  if (__any_sync(0xffffffffu, sv_fail)) {
    NoCandidate(it, beta, lane);
    return;
  }
  const uint32_t mask = __ballot_sync(0xffffffffu, has_bit && count > TR / 2);
  // bit 0 is the most significant digit of xi
  const uint32_t xs = L > 0 ? (__brev(mask) >> (32 - L)) : 0u;
  // the FP32 path (also in its FP64 kernels) leaves pending candidates that
  // the merge finishes on full warps; the FP64 path finishes them here
  const bool pending = fp32 || it.eps_rel > 0.f;
  int64_t k1;
  double wf = 0.0;
  if (pending) {
    k1 = RoundK1(n, beta, xs, L, B);
  } else {
    const double xi1 = ldexp(2.0 * double(xs) + 1.0, -(L + 1));
    k1 = int64_t(round(double(n) * (double(beta) + xi1) / double(B)));
    const double xi0 = double(k1) / double(n) - (double(beta) + 0.5) / double(B);
    wf = WindowInFreq(it, xi0);
    if (fabs(wf) < it.win_thr) {
      NoCandidate(it, beta, lane);
      return;
    }
  }

  // ---- coefficient (src/iterate.cc:146-171)
  V fac_t[TMAX];
  {
    // lane t evaluates e^{-2 pi i (q_t k1 mod n)/n}; the warp shares it
    V mine;
    mine.x = T(1);
    mine.y = T(0);
    if (lane < TR) mine = O::phase(it, -int64_t(it.q[lane]) * k1);
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        fac_t[t].x = __shfl_sync(0xffffffffu, mine.x, t);
        fac_t[t].y = __shfl_sync(0xffffffffu, mine.y, t);
      }
    }
  }
  V acc;
  acc.x = acc.y = T(0);
  V fac2;
  fac2.x = T(1);
  fac2.y = T(0);
  if (has_bit) fac2 = O::phase(it, -off * k1);
#pragma unroll
  for (int t = 0; t < TMAX; ++t) {
    if (t < TR) {
      if (lane == 0) {
        const V p0 = vmul2(u0[t], fac_t[t]);
        acc.x += p0.x;
        acc.y += p0.y;
      }
      if (has_bit) {
        const V p1 = vmul2(up[t], vmul2(fac_t[t], fac2));
        const V p2 = vmul2(um[t], vmul2(fac_t[t], vconj2(fac2)));
        acc.x += p1.x + p2.x;
        acc.y += p1.y + p2.y;
      }
    }
  }
  T ax = acc.x, ay = acc.y;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ax += __shfl_xor_sync(0xffffffffu, ax, o);
    ay += __shfl_xor_sync(0xffffffffu, ay, o);
  }
  if (fp32) {
    // the coefficient's FP32 error: every averaged value carries at most the
    // bound of the rows involved (the FP32 sums and phases add a few ulp of
    // the largest value, inside the kEpsValue share)
    T amax = 0;
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        amax = max(amax, max(vabs2<T, V>(u0[t]),
                             max(vabs2<T, V>(up[t]), vabs2<T, V>(um[t]))));
      }
    }
    float eps_c = eps_base + it.eps_rel * (kEpsRowMax * rml + kEpsValue * float(amax));
    for (int o = 16; o > 0; o >>= 1) {
      eps_c = fmaxf(eps_c, __shfl_xor_sync(0xffffffffu, eps_c, o));
    }
    if (lane == 0) {
      it.cand_k0[beta] = int32_t(k1);
      it.cand_coef[beta] = make_double2(double(ax), double(ay));
      it.cand_err[beta] = double(eps_c);
      it.cand_valid[beta] = 2;
    }
    return;
  }
  // near-tie bins of the FP32 path: the rows that were not re-binned carry
  // the FP32 binning bound into the coefficient
  double err = 0.0;
  if (!fp32 && mode == kDecideExact) {
    float rm = 0.f, am = 0.f;
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        const float *r = it.row_max + size_t(t) * rows;
        rm = fmaxf(rm, r[0]);
        am = fmaxf(am, float(vabs2<T, V>(u0[t])));
        if (has_bit) {
          rm = fmaxf(rm, fmaxf(r[2 * lane + 1], r[2 * lane + 2]));
          am = fmaxf(am, float(max(vabs2<T, V>(up[t]), vabs2<T, V>(um[t]))));
        }
      }
    }
    float e = *it.eps_dev + it.eps_rel * (kEpsRowMax * rm + kEpsValue * am);
    for (int o = 16; o > 0; o >>= 1) e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, o));
    err = double(e);
  }
  if (pending) {
    if (lane == 0) {
      it.cand_k0[beta] = int32_t(k1);
      it.cand_coef[beta] = make_double2(double(ax), double(ay));
      it.cand_err[beta] = err;
      it.cand_valid[beta] = 2;
    }
    return;
  }
  if (lane == 0) {
    double2 coef = make_double2(double(ax) / double(TR * (1 + 2 * L)),
                                double(ay) / double(TR * (1 + 2 * L)));
    const ModN mod{uint32_t(n), it.n_inv};
    const int32_t k0 = int32_t(mod(int64_t(it.a_inv) * mod(k1 - it.b)));
    coef = cmul(coef, Phase64(it, -int64_t(it.c) * k0));
    coef = make_double2(coef.x / wf, coef.y / wf);
    it.cand_k0[beta] = k0;
    it.cand_coef[beta] = coef;
    it.cand_err[beta] = 0.0;
    it.cand_valid[beta] = 1;
    it.flags[0] = 1;
  }
}

// One warp per bin. cond: only signals whose iteration is redone in FP64
// (more near-tie bins than their list holds) take part.
template <typename T, int TMAX>
__global__ void __launch_bounds__(256)
    k_decide(const SigIter *__restrict__ its, int mode, int cond) {
  const SigIter &it = its[blockIdx.y];
  if (!it.active) return;
  if (cond ? !RedoFP64(it) : it.force_fp64) return;
  const int beta = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (beta >= it.bins) return;
  DecideBin<T, TMAX>(it, beta, FromBins{it, beta}, mode);
}

// One warp per listed near-tie bin: FP64 decision on the FP64 re-binned
// values. Signals whose list overflowed are redone whole instead.
template <int TMAX>
__global__ void __launch_bounds__(256)
    k_decide_listed(const SigIter *__restrict__ its, int redo) {
  const SigIter &it = its[blockIdx.y];
  if (!it.active) return;
  if (it.force_fp64) return;
  const int nf = *(volatile int32_t *)&it.flags[2];
  if (nf > it.esc_cap) {
    // the whole iteration is redone in FP64 when the redo kernels run
    if (!redo && blockIdx.x == 0 && threadIdx.x == 0) {
      atomicOr(&it.flags[1], kStatusUnresolved);
    }
    return;
  }
  const int e = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (e >= nf) return;
  const int beta = it.esc_list[e];
  DecideBin<double, TMAX>(it, beta, FromRebin{it, e, beta, it.esc_mask[e]},
                          kDecideExact);
}

// ---------------------------------------------------------------- merge
__device__ void InsertMode(const SigIter &it, int32_t k0, double2 coef,
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

// Candidates -> table. Pending FP32 candidates are finished here in FP64 on
// full warps (src/iterate.cc:139-171): the window response at
// xi0 = k1/n - (beta + 1/2)/B and its threshold, the average over the
// T (1 + 2L) values, k0 = a^-1 (k1 - b) mod n, the factor e^{-2 pi i c k0/n}
// and the division by the window response.
__global__ void k_merge(const SigIter *__restrict__ its) {
  const SigIter &it = its[blockIdx.y];
  if (!it.active) return;
  const int beta = blockIdx.x * blockDim.x + threadIdx.x;
  if (beta >= it.bins) return;
  const int v = it.cand_valid[beta];
  if (!v) return;
  int32_t k0 = it.cand_k0[beta];
  double2 coef = it.cand_coef[beta];
  double err = it.cand_err[beta];
  if (v == 2) {
    const int64_t n = it.n, k1 = k0;
    const int B = it.bins;
    const double xi0 = double(k1) / double(n) - (double(beta) + 0.5) / double(B);
    const double wf = WindowInFreq(it, xi0);
    if (fabs(wf) < it.win_thr) {
      it.cand_valid[beta] = 0;
      return;
    }
    const double m = double(it.trials * (1 + 2 * it.bits));
    coef = make_double2(coef.x / m, coef.y / m);
    const ModN mod{uint32_t(n), it.n_inv};
    k0 = int32_t(mod(int64_t(it.a_inv) * mod(k1 - it.b)));
    coef = cmul(coef, Phase64(it, -int64_t(it.c) * k0));
    coef = make_double2(coef.x / wf, coef.y / wf);
    err = err / fabs(wf);
    it.cand_k0[beta] = k0;
    it.cand_coef[beta] = coef;
    it.cand_err[beta] = err;
    it.cand_valid[beta] = 1;
  }
  it.flags[0] = 1;
  InsertMode(it, k0, coef, err);
}

__global__ void k_table_insert(const SigIter *__restrict__ it,
                               const int32_t *__restrict__ k0,
                               const double2 *__restrict__ coef, int64_t m) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= m) return;
  InsertMode(*it, k0[i], coef[i], 0.0);
}

__global__ void k_pencil(const double2 *__restrict__ u3, int64_t count,
                         double *sigma, int32_t *vote) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= count) return;
  double s0, s1;
  vote[i] = Pencil(u3[3 * i], u3[3 * i + 1], u3[3 * i + 2], &s0, &s1) ? 1 : 0;
  sigma[2 * i] = s0;
  sigma[2 * i + 1] = s1;
}

// Empty tables and control words of every signal.
__global__ void k_clear_tables(const SigIter *__restrict__ its) {
  const SigIter &it = its[blockIdx.y];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < it.tab_cap) {
    it.tab_key[i] = kEmptyKey;
    it.tab_coef[i] = make_double2(0.0, 0.0);
    it.tab_err[i] = 0.0;
  }
  if (i < kCtlWords) it.flags[i] = 0;
}

// The occupied entries of every table into a staging area, signal s at
// [s * stride, s * stride + count_s), sorted by k0 (one block per signal,
// bitonic sort of (k0, slot) in shared memory); a table with more entries
// than the sort holds (only after a capacity status) is written in insertion
// order and sorted[s] = 0.
__global__ void __launch_bounds__(1024)
    k_export_tables(const SigIter *__restrict__ its, int32_t *keys,
                    double2 *coefs, int32_t *counts, int32_t *sorted, int stride) {
  extern __shared__ unsigned long long sk[];
  const SigIter &it = its[blockIdx.x];
  const int cnt = *it.tab_count;
  const size_t base = size_t(blockIdx.x) * stride;
  const bool fits = cnt <= BucketKeys(it.tab_cap);
  if (threadIdx.x == 0) {
    counts[blockIdx.x] = cnt;
    sorted[blockIdx.x] = fits ? 1 : 0;
  }
  if (!fits) {
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
      const int sl = it.occ_list[i];
      keys[base + i] = it.tab_key[sl];
      coefs[base + i] = it.tab_coef[sl];
    }
    return;
  }
  int m = 1;
  while (m < cnt) m <<= 1;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    unsigned long long k = ~0ull;
    if (i < cnt) {
      const int sl = it.occ_list[i];
      k = (static_cast<unsigned long long>(uint32_t(it.tab_key[sl])) << 32) |
          static_cast<unsigned long long>(uint32_t(sl));
    }
    sk[i] = k;
  }
  __syncthreads();
  BitonicSort(sk, m);
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
    const unsigned long long k = sk[i];
    keys[base + i] = int32_t(k >> 32);
    coefs[base + i] = it.tab_coef[uint32_t(k)];
  }
}

template <typename T, int TMAX>
void LaunchDecideT(const SigIter *d_its, int nsig, int max_bins, int mode,
                   int cond, cudaStream_t s) {
  dim3 grid((max_bins + 7) / 8, nsig);
  k_decide<T, TMAX><<<grid, 256, 0, s>>>(d_its, mode, cond);
}

template <typename T>
void LaunchDecideP(const SigIter *d_its, int nsig, int max_bins, int max_trials,
                   int mode, int cond, cudaStream_t s) {
  if (max_trials <= 1) {
    LaunchDecideT<T, 1>(d_its, nsig, max_bins, mode, cond, s);
  } else if (max_trials <= 5) {
    LaunchDecideT<T, 5>(d_its, nsig, max_bins, mode, cond, s);
  } else {
    LaunchDecideT<T, kMaxTrials>(d_its, nsig, max_bins, mode, cond, s);
  }
}

}  // namespace

void LaunchClearTables(const SigIter *d_its, int nsig, int max_cap,
                       cudaStream_t s) {
  dim3 grid((std::max(max_cap, int(kCtlWords)) + 255) / 256, nsig);
  k_clear_tables<<<grid, 256, 0, s>>>(d_its);
}

void LaunchExportTables(const SigIter *d_its, int nsig, int max_cap,
                        int32_t *keys, double2 *coefs, int32_t *counts,
                        int32_t *sorted, cudaStream_t s) {
  const size_t sm = size_t(BucketKeys(max_cap)) * sizeof(unsigned long long);
  cudaFuncSetAttribute(k_export_tables, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(sm));
  k_export_tables<<<nsig, 1024, sm, s>>>(d_its, keys, coefs, counts, sorted,
                                         max_cap);
}

void LaunchModePrep(const SigIter *d_its, int nsig, int max_cap, cudaStream_t s,
                    bool cond) {
  // the occupied count is only known on the device: cover the whole table,
  // blocks past the count exit at once
  dim3 grid((max_cap + 255) / 256, nsig);
  k_mode_prep<<<grid, 256, 0, s>>>(d_its, cond ? 1 : 0);
}

void LaunchBucket(const SigIter *d_its, int nsig, int max_bins, int max_cap,
                  cudaStream_t s) {
  (void)max_bins;
  const size_t sm = size_t(BucketKeys(max_cap)) * sizeof(unsigned long long);
  cudaFuncSetAttribute(k_bucket, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(sm));
  k_bucket<<<nsig, 1024, sm, s>>>(d_its);
}

void LaunchDecide(const SigIter *d_its, int nsig, int max_bins, int max_trials,
                  bool fp32, bool subtract_only, cudaStream_t s, bool cond) {
  const int mode = subtract_only ? kSubtractOnly : kDecide;
  if (fp32) {
    LaunchDecideP<float>(d_its, nsig, max_bins, max_trials, mode, 0, s);
  } else {
    LaunchDecideP<double>(d_its, nsig, max_bins, max_trials, mode, cond ? 1 : 0,
                          s);
  }
}

void LaunchDecideListed(const SigIter *d_its, int nsig, int max_trials,
                        bool redo, cudaStream_t s) {
  dim3 grid((kMaxListed + 7) / 8, nsig);
  const int r = redo ? 1 : 0;
  if (max_trials <= 1) {
    k_decide_listed<1><<<grid, 256, 0, s>>>(d_its, r);
  } else if (max_trials <= 5) {
    k_decide_listed<5><<<grid, 256, 0, s>>>(d_its, r);
  } else {
    k_decide_listed<kMaxTrials><<<grid, 256, 0, s>>>(d_its, r);
  }
}

void LaunchMerge(const SigIter *d_its, int nsig, int max_bins,
                 cudaStream_t s) {
  dim3 grid((max_bins + 255) / 256, nsig);
  k_merge<<<grid, 256, 0, s>>>(d_its);
}

void LaunchTableInsert(const SigIter *d_it, const int32_t *k0,
                       const double2 *coef, int64_t m, cudaStream_t s) {
  if (m <= 0) return;
  k_table_insert<<<unsigned((m + 255) / 256), 256, 0, s>>>(d_it, k0, coef, m);
}

void LaunchPencil(const double2 *u3, int64_t count, double *sigma,
                  int32_t *vote, cudaStream_t s) {
  if (count <= 0) return;
  k_pencil<<<unsigned((count + 255) / 256), 256, 0, s>>>(u3, count, sigma,
                                                          vote);
}

bool DecideKernelsLaunchable() {
  int a = 0, b = 0, c = 0, d = 0;
  const size_t smb = size_t(BucketKeys(kMaxTableCap)) * sizeof(unsigned long long);
  cudaFuncSetAttribute(k_bucket, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(smb));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_bucket, 1024, smb);
  int e = 0;
  cudaFuncSetAttribute(k_export_tables, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(smb));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e, k_export_tables, 1024, smb);
  a = a < e ? a : e;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_decide<double, kMaxTrials>, 256, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_decide<float, kMaxTrials>, 256, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d, k_decide_listed<kMaxTrials>, 256, 0);
  return a > 0 && b > 0 && c > 0 && d > 0;
}

}  // namespace mpsft
