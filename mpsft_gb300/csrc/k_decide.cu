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
// One thread per occupied slot (the table's insertion list), so FP64 work
// runs on full warps.
__global__ void k_mode_prep(const SigIter *__restrict__ its) {
  const SigIter &it = its[blockIdx.y];
  if (!it.active) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *it.tab_count) return;
  const int s = it.occ_list[i];
  const int32_t key = it.tab_key[s];
  const int64_t n = it.n;
  const int B = it.bins;
  const int64_t k1 = PosMod(int64_t(it.a) * key + it.b, n);
  const int bin = int(k1 * B / n);
  const double xi = (double(bin) + 0.5) / double(B) - double(k1) / double(n);
  const double wf = WindowInFreq(it, xi);
  const double2 wc = cscale(it.tab_coef[s], wf);
  for (int t = 0; t < it.trials; ++t) {
    const int64_t ph = int64_t(it.q[t]) * k1 + int64_t(it.c) * key;
    it.mode_base[size_t(s) * it.trials + t] = cmul(wc, UnitPhase64(ph, n));
  }
  it.mode_k1[s] = int32_t(k1);
  it.mode_wf[s] = wf;
  it.mode_bin[s] = bin;
}

// Row factors of every found mode: e^{2 pi i (B 2^s k1 mod n)/n} for each bit
// s (the factor BinInFreqV1 applies to rows 2s+1 / 2s+2, src/binner.cc:584-589),
// one thread per (occupied slot, bit).
__global__ void k_mode_fac(const SigIter *__restrict__ its) {
  const SigIter &it = its[blockIdx.y];
  if (!it.active || it.bits <= 0) return;
  const int L = it.bits;
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int i = int(idx / L), s = int(idx % L);
  if (i >= *it.tab_count) return;
  const int sl = it.occ_list[i];
  const int64_t off = int64_t(it.bins) << s;
  it.mode_fac[size_t(sl) * it.fac_stride + s] =
      UnitPhase64(off * int64_t(it.mode_k1[sl]), it.n);
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
  __device__ static V load(const double2 &d) {
    return make_float2(float(d.x), float(d.y));
  }
  __device__ static V from(double2 d) { return make_float2(float(d.x), float(d.y)); }
  __device__ static V phase(int64_t m, int64_t n, int shift) {
    return UnitPhase32(m, n, shift);
  }
};
template <> struct Ops<double> {
  using V = double2;
  __device__ static V load(const double2 &d) { return d; }
  __device__ static V from(double2 d) { return d; }
  __device__ static V phase(int64_t m, int64_t n, int) {
    return UnitPhase64(m, n);
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
    const double2 *p =
        it.esc_part + ((size_t(e) * it.trials + t) * it.rows + r) * kRebinChunks;
    double2 s = p[0];
    for (int c = 1; c < kRebinChunks; ++c) s = cadd(s, p[c]);
    return s;
  }
};

enum DecideMode { kDecide = 0, kSubtractOnly = 1, kDecideExact = 2 };

// The bin loop body of Iterate for one bin (warp-wide). T = float: the FP32
// path with near-tie detection; T = double: FP64 decisions (the FP64 path, and
// the near-tie bins after their FP64 re-binning).
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
  double2 pre_base[TMAX];
  double mode_err = 0;  // FP32 error carried into this bin by the found modes
  if (lane < npre) {
    const int sl = it.bkt_list[st + lane];
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) pre_base[t] = it.mode_base[size_t(sl) * TR + t];
    }
    if (fp32) mode_err = it.tab_err[sl] * fabs(it.mode_wf[sl]);
  }
  for (int i = 0; i < nm; ++i) {
    double2 bs[TMAX];
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
#pragma unroll
      for (int t = 0; t < TMAX; ++t) {
        if (t < TR) bs[t] = it.mode_base[size_t(sl) * TR + t];
      }
      if (fp32 && lane == 0) mode_err += it.tab_err[sl] * fabs(it.mode_wf[sl]);
    }
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) u0[t] = vsub2(u0[t], O::from(bs[t]));
    }
  }
  if (fp32) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mode_err += __shfl_xor_sync(0xffffffffu, mode_err, o);
  }
  // FP32 error bound of this lane's values (see kEpsRms and friends)
  float eps_base = 0.f, rm0 = 0.f, rml = 0.f;
  if (fp32) {
    eps_base = *it.eps_dev + float(mode_err);
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
    if (it.bin_thr > 0) {
      const T thr2 = T(it.bin_thr * it.bin_thr);
      if (fp32) {
        const T eps0 = T(eps_base + it.eps_rel * (kEpsRowMax * rm0 +
                                                  kEpsValue * float(amax)));
        // |d e| <= 2 max|u0| eps + eps^2
        e_near = fabs(e - thr2) <= T(2) * amax * eps0 + eps0 * eps0;
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
    double2 bs[TMAX];
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
#pragma unroll
      for (int t = 0; t < TMAX; ++t) {
        if (t < TR) bs[t] = it.mode_base[size_t(sl) * TR + t];
      }
    }
    if (has_bit) {
      const int sl = it.bkt_list[st + i];
      const V fac = O::from(it.mode_fac[size_t(sl) * it.fac_stride + lane]);
#pragma unroll
      for (int t = 0; t < TMAX; ++t) {
        if (t < TR) {
          const V b = O::from(bs[t]);
          up[t] = vsub2(up[t], vmul2(b, fac));
          um[t] = vsub2(um[t], vmul2(b, vconj2(fac)));
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
    const T sv_thr = T(it.sv_thr);
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        T s0, s1, im;
        if (PencilT<T, V>(u0[t], up[t], um[t], &s0, &s1, &im)) ++count;
        if (sv_thr > T(0) && s1 * T(0.5) > sv_thr) sv_fail = true;
        if (fp32) {
          const T a0 = vabs2<T, V>(u0[t]), a1 = vabs2<T, V>(up[t]),
                  a2 = vabs2<T, V>(um[t]);
          const T eps = T(eps_base + it.eps_rel * (kEpsRowMax * rml +
                                                   kEpsValue * float(max(a0, max(a1, a2)))));
          // |d Im(m01)| <= eps (2|u0| + |u1| + |u2|) + 4 eps^2;
          // |d sigma1| <= ||dA||_2 <= 2 eps.
          if (fabs(im) <= eps * (T(2) * a0 + a1 + a2) + T(4) * eps * eps) near = true;
          if (sv_thr > T(0) && fabs(s1 * T(0.5) - sv_thr) <= eps) near = true;
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
  const double xi1 = ldexp(2.0 * double(xs) + 1.0, -(L + 1));
  const int32_t k1 =
      int32_t(round(double(n) * (double(beta) + xi1) / double(B)));
  const double xi0 = double(k1) / double(n) - (double(beta) + 0.5) / double(B);
  const double wf = WindowInFreq(it, xi0);
  if (fabs(wf) < it.win_thr) {
    NoCandidate(it, beta, lane);
    return;
  }

  // ---- coefficient (src/iterate.cc:146-171)
  V fac_t[TMAX];
  {
    // lane t evaluates e^{-2 pi i (q_t k1 mod n)/n}; the warp shares it
    V mine;
    mine.x = T(1);
    mine.y = T(0);
    if (lane < TR) mine = O::phase(-int64_t(it.q[lane]) * k1, n, it.phase_shift);
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
  if (has_bit) fac2 = O::phase(-off * k1, n, it.phase_shift);
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
  double ax = acc.x, ay = acc.y;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ax += __shfl_xor_sync(0xffffffffu, ax, o);
    ay += __shfl_xor_sync(0xffffffffu, ay, o);
  }
  // the coefficient's FP32 error: every averaged value carries at most the
  // bound of the rows involved
  float eps_c = 0.f;
  if (fp32) {
    T amax = 0;
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        amax = max(amax, max(vabs2<T, V>(u0[t]),
                             max(vabs2<T, V>(up[t]), vabs2<T, V>(um[t]))));
      }
    }
    eps_c = eps_base + it.eps_rel * (kEpsRowMax * rml + kEpsValue * float(amax));
    for (int o = 16; o > 0; o >>= 1) {
      eps_c = fmaxf(eps_c, __shfl_xor_sync(0xffffffffu, eps_c, o));
    }
  }
  if (lane == 0) {
    double2 coef = make_double2(ax / double(TR * (1 + 2 * L)),
                                ay / double(TR * (1 + 2 * L)));
    const int32_t k0 =
        int32_t(PosMod(int64_t(it.a_inv) * (int64_t(k1) - it.b), n));
    coef = cmul(coef, UnitPhase64(-int64_t(it.c) * k0, n));
    coef = make_double2(coef.x / wf, coef.y / wf);
    it.cand_k0[beta] = k0;
    it.cand_coef[beta] = coef;
    it.cand_err[beta] = fp32 ? double(eps_c) / fabs(wf) : 0.0;
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

__global__ void k_merge(const SigIter *__restrict__ its) {
  const SigIter &it = its[blockIdx.y];
  if (!it.active) return;
  const int beta = blockIdx.x * blockDim.x + threadIdx.x;
  if (beta >= it.bins || !it.cand_valid[beta]) return;
  InsertMode(it, it.cand_k0[beta], it.cand_coef[beta], it.cand_err[beta]);
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

void LaunchModePrep(const SigIter *d_its, int nsig, int max_cap, int max_bits,
                    cudaStream_t s) {
  // the occupied count is only known on the device: cover the whole table,
  // blocks past the count exit at once
  dim3 grid((max_cap + 255) / 256, nsig);
  k_mode_prep<<<grid, 256, 0, s>>>(d_its);
  if (max_bits > 0) {
    dim3 grid2(unsigned((int64_t(max_cap) * max_bits + 255) / 256), nsig);
    k_mode_fac<<<grid2, 256, 0, s>>>(d_its);
  }
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

}  // namespace mpsft
