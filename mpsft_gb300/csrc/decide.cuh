// The per-bin decision of an iteration (the bin loop of Iterate,
// src/iterate.cc:113-175, with IdentifyFreq, src/iterate.cc:44-76, MatPencil,
// src/freqid.cc:27-48, and BinInFreqV1's subtraction, src/binner.cc:565-591),
// used by the FP32, FP64 and near-tie (listed bin) decide kernels.
#pragma once

#include "common.cuh"
#include "rebin.cuh"

namespace mpsft {

namespace {

// ---------------------------------------------------------------- decide
template <typename T> struct Ops;
template <> struct Ops<float> {
  using V = float2;
  __device__ static V from(double2 d) { return make_float2(float(d.x), float(d.y)); }
  __device__ static V from(float2 f) { return f; }
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

// Lists bin beta as a near tie (mask: bits whose decisions were near);
// returns its list position, or -1 when the list is full (the iteration is
// then redone in FP64), to every lane. Called by every lane of the bin's warp
// with a warp-uniform condition; the caller prepares the listed bin
// (PrepListedBin) once the decision is done.
__device__ inline int FlagBin(const SigIter &it, int beta, uint32_t mask,
                              int lane) {
  int pos = -1;
  if (lane == 0) {
    pos = atomicAdd(&it.flags[2], 1);
    if (pos < it.esc_cap) {
      it.esc_list[pos] = beta;
      if (it.esc_mask) it.esc_mask[pos] = mask;
    } else {
      pos = -1;
    }
  }
  return __shfl_sync(0xffffffffu, pos, 0);
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

// Bin values of the FP32 pass at bin beta: complex64 from ubuf32 in solves
// and iterations, else the complex128 bins.
struct FromBins32 {
  const SigIter &it;
  int beta;
  __device__ float2 get(int t, int r) const {
    const size_t i = (size_t(t) * it.rows + r) * it.bins_cap + beta;
    if (it.ubuf32 != nullptr) return it.ubuf32[i];
    const double2 d = it.ubuf[i];
    return make_float2(float(d.x), float(d.y));
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
      const size_t i = (size_t(t) * it.rows + r) * it.bins_cap + beta;
      if (it.ubuf32 != nullptr) {
        const float2 f = it.ubuf32[i];
        return make_double2(f.x, f.y);
      }
      return it.ubuf[i];
    }
    return __ldcg(&it.esc_sum[(size_t(e) * it.trials + t) * it.rows + r]);
  }
};

template <typename V> __device__ inline float Abs32(V a) {
  const float x = float(a.x), y = float(a.y);
  return sqrtf(x * x + y * y);
}

enum DecideMode { kDecide = 0, kSubtractOnly = 1, kDecideExact = 2 };

// k1 = round(n (beta + xi1) / B) with xi1 = (2 xs + 1) / 2^{L+1}, exactly in
// integers: num = n (beta 2^{L+1} + 2 xs + 1) < 2^64, den = B 2^{L+1} < 2^33
// (B 2^{L-1} <= n by the definition of L). The reference evaluates this in
// FP64 (relative error below 2^-52, so at most 2^-21 absolute); when the
// exact value lies within 2^-18 of a half-integer, that FP64 evaluation is
// used instead so that the rounding is the reference's.
// No 64-bit division: with Q = floor(num / 2^{L+1}) (< n B < 2^62),
// floor(num / den) = floor(Q / B), estimated from psi = round(2^64 / (2B))
// to within one and corrected exactly.
__host__ __device__ inline int64_t RoundK1(int64_t n, int beta, uint32_t xs, int L,
                                           int B, uint64_t psi) {
  const uint64_t den = uint64_t(B) << (L + 1);
  const uint64_t num =
      uint64_t(n) * ((uint64_t(beta) << (L + 1)) + 2 * uint64_t(xs) + 1);
  const uint64_t Q = num >> (L + 1);
  uint64_t q = MulHi64(2 * Q, psi);  // |2 Q psi / 2^64 - Q / B| < 1/4
  int64_t rq = int64_t(Q) - int64_t(q * uint64_t(B));
  if (rq < 0) {
    --q;
    rq += B;
  } else if (rq >= B) {
    ++q;
    rq -= B;
  }
  const uint64_t r = (uint64_t(rq) << (L + 1)) + (num & ((uint64_t(1) << (L + 1)) - 1));
  const uint64_t d = 2 * r > den ? 2 * r - den : den - 2 * r;  // 2 den |frac - 1/2|
  if (d <= (den >> 17)) {
    const double xi1 = ldexp(2.0 * double(xs) + 1.0, -(L + 1));
    return int64_t(round(double(n) * (double(beta) + xi1) / double(B)));
  }
  return int64_t(q) + (2 * r >= den ? 1 : 0);
}

// The decisions of a bin from its mode-subtracted values (the part of
// DecideBin after the subtraction; also the listed bins' block-wide FP64
// decision): non-finite check, IdentifyFreq, k1, coefficient. Returns the
// near-tie list position (FP32) or listed.
template <typename T, int TMAX>
__device__ __forceinline__ int DecideTail(const SigIter &it, int beta, int mode,
                                          const typename Ops<T>::V *u0,
                                          const typename Ops<T>::V *up,
                                          const typename Ops<T>::V *um,
                                          float eps_base, float rml, bool e_near,
                                          int listed) {
  using O = Ops<T>;
  using V = typename O::V;
  const int lane = threadIdx.x & 31;
  const int L = it.bits, TR = it.trials, rows = it.rows;
  const int64_t n = it.n;
  const int B = it.bins;
  const bool has_bit = lane < L;
  const bool fp32 = sizeof(T) == 4;
  const int64_t off = has_bit ? (int64_t(B) << lane) : 0;
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
    return listed;
  }

  // ---- IdentifyFreq: per-bit majority of the pencil votes, sv rejection
  int count = 0;
  // clear_fail: an sv rejection outside its rounding bound, which rejects the
  // bin whatever the near decisions elsewhere give (no listing needed)
  bool sv_fail = false, near = false, clear_fail = false;
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
          if (sv_thr > T(0)) {
            const bool sv_near = fabs(s1 * T(0.5) - sv_thr) <= eps + sv_thr * T(1.2e-7);
            if (sv_near) {
              near = true;
            } else if (s1 * T(0.5) > sv_thr) {
              clear_fail = true;
            }
          }
        }
      }
    }
  }
  if (fp32 && !__any_sync(0xffffffffu, clear_fail)) {
    const uint32_t near_bits = __ballot_sync(0xffffffffu, has_bit && near);
    if (near_bits || e_near) listed = FlagBin(it, beta, near_bits, lane);
  }
  if (__any_sync(0xffffffffu, sv_fail)) {
    NoCandidate(it, beta, lane);
    return listed;
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
    k1 = RoundK1(n, beta, xs, L, B, it.psi);
  } else {
    const double xi1 = ldexp(2.0 * double(xs) + 1.0, -(L + 1));
    k1 = int64_t(round(double(n) * (double(beta) + xi1) / double(B)));
    const double xi0 = double(k1) / double(n) - (double(beta) + 0.5) / double(B);
    wf = WindowInFreq(it, xi0);
    if (fabs(wf) < it.win_thr) {
      NoCandidate(it, beta, lane);
      return listed;
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
    return listed;
  }
  // near-tie bins of the FP32 path: the rows that were not re-binned carry
  // the FP32 binning bound into the coefficient
  double err = 0.0;
  if (!fp32 && mode == kDecideExact) {
    float rm = 0.f, am = 0.f, msx = 0.f;
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        const float *r = it.row_max + size_t(t) * rows;
        const float *ms = it.row_ms + size_t(t) * rows;
        rm = fmaxf(rm, r[0]);
        msx = fmaxf(msx, ms[0]);
        // magnitudes in FP32 (an error bound needs no more)
        am = fmaxf(am, Abs32(u0[t]));
        if (has_bit) {
          rm = fmaxf(rm, fmaxf(r[2 * lane + 1], r[2 * lane + 2]));
          msx = fmaxf(msx, fmaxf(ms[2 * lane + 1], ms[2 * lane + 2]));
          am = fmaxf(am, fmaxf(Abs32(up[t]), Abs32(um[t])));
        }
      }
    }
    float e = it.eps_ms * sqrtf(msx) +
              it.eps_rel * (kEpsRowMax * rm + kEpsValue * am);
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
    return listed;
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
  return listed;
}

// The bin loop body of Iterate for one bin (warp-wide). T = float: the FP32
// path with near-tie detection, FP32 arithmetic only (GB300 runs FP64 at a
// small fraction of its FP32 rate): a surviving bin leaves a pending
// candidate (cand_valid = 2: k1 in cand_k0, the unscaled coefficient sum in
// cand_coef, its error bound in cand_err) that the merge finishes in FP64 on
// full warps. T = double: FP64 decisions to the end (the FP64 path, and the
// near-tie bins after their re-binning).
template <typename T, int TMAX, typename Src>
__device__ int DecideBin(const SigIter &it, int beta, const Src &src,
                          int mode) {
  using O = Ops<T>;
  using V = typename O::V;
  const int lane = threadIdx.x & 31;
  const int L = it.bits, TR = it.trials, rows = it.rows;
  const int B = it.bins;
  const bool has_bit = lane < L;
  const bool fp32 = sizeof(T) == 4;
  const int nm = it.bkt_count[beta];
  const int st = it.bkt_start[beta];
  int listed = -1;  // list position when this bin is listed as a near tie

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
  int pre_k1 = 0;  // k1 of the lane's mode (row factors below)
  if (lane < npre) {
    const int sl = it.bkt_list[st + lane];
    O::template terms<TMAX>(it, sl, pre_base);
    pre_k1 = it.mode_k1[sl];
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
  // FP32 error bound of this lane's values (see kEpsRms and friends): the
  // rows' rms terms (row 0 alone for the energy test, warp-uniform; with the
  // lane's two rows for its votes and the coefficient), the carried errors
  float eps_base = 0.f, eps_base0 = 0.f, rm0 = 0.f, rml = 0.f;
  if (fp32) {
    float ms0 = 0.f, msl = 0.f;
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        const float *rm = it.row_max + size_t(t) * rows;
        const float *ms = it.row_ms + size_t(t) * rows;
        rm0 = fmaxf(rm0, rm[0]);
        ms0 = fmaxf(ms0, ms[0]);
        if (has_bit) {
          rml = fmaxf(rml, fmaxf(rm[2 * lane + 1], rm[2 * lane + 2]));
          msl = fmaxf(msl, fmaxf(ms[2 * lane + 1], ms[2 * lane + 2]));
        }
      }
    }
    rml = fmaxf(rml, rm0);
    eps_base0 = it.eps_ms * sqrtf(ms0) + mode_err;
    eps_base = it.eps_ms * sqrtf(fmaxf(ms0, msl)) + mode_err;
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
      return listed;
    }
    if (fp32 ? it.bin_thr2_f > 0.f : it.bin_thr > 0) {
      T thr2;
      if (fp32) {
        thr2 = it.bin_thr2_f;
        const T eps0 = T(eps_base0 + it.eps_rel * (kEpsRowMax * rm0 +
                                                   kEpsValue * float(amax)));
        // |d e| <= 2 max|u0| eps + eps^2, plus the threshold's FP32 rounding
        e_near = fabs(e - thr2) <= T(2) * amax * eps0 + eps0 * eps0 +
                                       thr2 * T(1.2e-7);
      } else {
        thr2 = T(it.bin_thr * it.bin_thr);
      }
      if (e < thr2) {
        if (e_near) listed = FlagBin(it, beta, 0u, lane);
        NoCandidate(it, beta, lane);
        return listed;
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
  // four modes at a time: their row factors e^{2 pi i (B 2^s k1 mod n)/n}
  // (src/binner.cc:584-589) are evaluated side by side, then subtracted in
  // the bin's mode order
  for (int i0 = 0; i0 < nm; i0 += 4) {
    V fac[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u;
      if (i < nm) {
        const int64_t k1 = i < 32 ? __shfl_sync(0xffffffffu, pre_k1, i)
                                  : it.mode_k1[it.bkt_list[st + i]];
        if (has_bit) fac[u] = O::phase(it, off * k1);
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u;
      if (i < nm) {
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
          O::template terms<TMAX>(it, it.bkt_list[st + i], bs);
        }
        if (has_bit) {
#pragma unroll
          for (int t = 0; t < TMAX; ++t) {
            if (t < TR) {
              up[t] = vsub2(up[t], vmul2(bs[t], fac[u]));
              um[t] = vsub2(um[t], vmul2(bs[t], vconj2(fac[u])));
            }
          }
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
    return listed;
  }

  return DecideTail<T, TMAX>(it, beta, mode, u0, up, um, eps_base, rml, e_near,
                             listed);

}

}  // namespace

}  // namespace mpsft
