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
// Work decomposition: one CTA per (bins tile, row group, trial, signal);
// several lanes share a bin and split its f = p/B folds (t, t + kB, ...).
// Indices step exactly in uint32 (j += a*kB mod n with one conditional
// subtract), so no 64-bit division runs per sample. FP32: the phase is carried
// in fixed-point turns (exact reduction mod 1 by wrap-around) and converted
// only for sincospif; products in FP32; the per-lane sums and the lane tree
// use compensated (TwoSum) addition. FP64: per-sample double phase and
// sincospi, plain sums (the straightforward port).
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

// ---- FP32 fold of the row cluster (row 0 and pair groups 1..sc) --------
// For bin beta, the cluster's union is u = beta + k B for the span
// k = -h - Mc .. h + Mc (h = (folds - 1)/2, Mc = 2^(sc-1)): J = folds + 2 Mc
// samples y_u = x[a (q + u) + c] e^{2 pi i (b u / n - u / (2B))}. Row m B
// (m = 0, +-1, +-2, ..., +-Mc) folds
//   F_m[beta] = eps_m sum_{i < folds} y_{beta + (i - h + m) B} wt(beta + (i - h) B)
// (eps_m = -1 for m = +-1: the row's own phase -t/(2B) differs from -u/(2B)
// by m/2 turns), i.e. a J-sample correlation with the window. The mirror bin
// B - beta takes the samples at -u: y_{-u} = x[a (q - u) + c] conj(phase(u)),
// so one phase serves both (the reference's symmetry of V1/V4), and its
// window runs backwards.
//
// One warp per base bin beta <= (B - 1)/2: its lanes gather the span and the
// mirrored span into the warp's shared slice (J <= kMaxClusterSpan samples
// each), then lane r < 16 folds row r of beta and lane 16 + r row r of the
// mirror bin, the window weights broadcast from the lanes that loaded them.
// The cluster takes the CTAs of row groups 0..sc of the launch grid (their
// work would otherwise overlap), so every row of a signal is binned in the
// same launch and a sample's sector is read from DRAM once for all rows.
// The shared slices are small (12 KiB per CTA): random gathers need most of
// the L1 for their misses in flight (a 48 KiB tile per CTA made the binning
// 1.4x slower on GB300).
constexpr int kWarpsPerCta = 8;
constexpr int kSpanSlots = (kMaxClusterSpan + 31) / 32;  // span samples per lane
constexpr int kMirrorOff = kMaxClusterSpan + 8;  // padded: other shared banks

__device__ inline int ClusterRowOffset(int r) {
  // row r -> m: 0, then +2^s (r = 2s + 1), -2^s (r = 2s + 2)
  if (r == 0) return 0;
  return (r & 1) ? (1 << ((r - 1) >> 1)) : -(1 << ((r >> 1) - 1));
}

template <typename TX>
__device__ void FoldClusterWarp(const SigIter &it, int tr, int beta, int sc,
                                float2 *ys) {
  const int lane = threadIdx.x & 31;
  const int B = it.bins, f = it.folds;
  const int Mc = sc > 0 ? (1 << (sc - 1)) : 0;
  const int J = f + 2 * Mc;
  const int h = (f - 1) >> 1;
  const uint32_t n = uint32_t(it.n);
  const ModN mod{n, it.n_inv};
  const int64_t q = it.q[tr];
  const int64_t a = it.a, c = it.c;
  const uint64_t phs = it.phi_b - it.psi;  // b/n - 1/(2B) turns
  const bool mirror = beta != 0;
  const TX *__restrict__ x = reinterpret_cast<const TX *>(it.x);
  // gather: lane l takes span positions l, l + 32, ...; all loads first
  TX x1[kSpanSlots], x2[kSpanSlots];
  uint32_t p32[kSpanSlots];
#pragma unroll
  for (int s = 0; s < kSpanSlots; ++s) {
    const int j = lane + 32 * s;
    if (j < J) {
      const int64_t u = beta + int64_t(j - h - Mc) * B;
      x1[s] = __ldg(&x[mod(a * mod(q + u) + c)]);
      if (mirror) x2[s] = __ldg(&x[mod(a * mod(q - u) + c)]);
      p32[s] = uint32_t((phs * uint64_t(u) + (uint64_t(1) << 31)) >> 32);
    }
  }
  // window weights W[i] = wt(beta + (i - h) B), lane l holding i = l + 32 s
  float wreg[kSpanSlots];
#pragma unroll
  for (int s = 0; s < kSpanSlots; ++s) {
    const int i = lane + 32 * s;
    wreg[s] = 0.f;
    if (i < f) {
      const int64_t t = int64_t(beta) + int64_t(i - h) * B;
      wreg[s] = __ldg(&it.wt32[t < 0 ? -t : t]);
    }
  }
#pragma unroll
  for (int s = 0; s < kSpanSlots; ++s) {
    const int j = lane + 32 * s;
    if (j < J) {
      const float phi = float(int32_t(p32[s])) * 2.3283064365386963e-10f;
      float sn, cs;
      sincospif(2.0f * phi, &sn, &cs);
      const float2 v1 = to_f2(x1[s]);
      ys[j] = make_float2(v1.x * cs - v1.y * sn, v1.x * sn + v1.y * cs);
      if (mirror) {
        const float2 v2 = to_f2(x2[s]);
        ys[kMirrorOff + J - 1 - j] =
            make_float2(v2.x * cs + v2.y * sn, v2.y * cs - v2.x * sn);
      }
    }
  }
  __syncwarp();
  // fold: lane r < 16 row r of beta, lane 16 + r row r of B - beta
  const int sc2 = 1 + 2 * sc;
  const bool mir = lane >= 16;
  const int r = lane & 15;
  const bool live = r < sc2 && (!mir || mirror);
  const float2 *yb = ys + (mir ? kMirrorOff : 0) + Mc + (live ? ClusterRowOffset(r) : 0);
  CompF ar, ai;
  for (int i = 0; i < f; ++i) {
    // W[i] for the bin, W[f - 1 - i] for its mirror (uniform slot indices)
    const int i2 = f - 1 - i;
    float w1 = wreg[0], w2 = wreg[0];
#pragma unroll
    for (int s = 1; s < kSpanSlots; ++s) {
      if ((i >> 5) == s) w1 = wreg[s];
      if ((i2 >> 5) == s) w2 = wreg[s];
    }
    w1 = __shfl_sync(0xffffffffu, w1, i & 31);
    w2 = __shfl_sync(0xffffffffu, w2, i2 & 31);
    if (live) {
      const float w = mir ? w2 : w1;
      const float2 yv = yb[i];
      ar.add(yv.x * w);
      ai.add(yv.y * w);
    }
  }
  if (live) {
    const float e = (r == 1 || r == 2) ? -1.f : 1.f;
    float2 *fold = reinterpret_cast<float2 *>(it.fold);
    const int bin = mir ? B - beta : beta;
    fold[(size_t(tr) * it.rows + r) * it.bins_cap + bin] =
        make_float2(e * (ar.s + ar.c), e * (ai.s + ai.c));
  }
  __syncwarp();  // the slice is reused by the warp's next bin
}

// FP32 fold of the pair groups beyond the cluster: one CTA per (256/SPLIT
// bins, row group, trial, signal); SPLIT threads share a bin and take every
// SPLIT-th fold, BATCH folds of both rows in flight at a time. Setup without
// divisions: indices by Barrett reduction (or a mask), the phase
// m/n - t/(2B) as a 64-bit fixed-point product phi_b (t + off) - psi t
// (wrap-around = exact reduction mod 1, error < 2^-33 turns), rounded to
// 32-bit turns for sincospif. SPLIT, BATCH and CLUSTER (the row cluster on,
// or every group folded pairwise) are the launch shape the autotuner picks
// (FoldShapeOf); every shape computes the same sums up to FP32 rounding.
template <typename TX, int SPLIT, int BATCH, bool CLUSTER>
__global__ void __launch_bounds__(256, 4)
    k_bin_fold32(const SigIter *__restrict__ its, int gmax) {
  constexpr int kFoldSplit = SPLIT;
  constexpr int kFoldBatch = BATCH;
  constexpr int kFoldBins = 256 / SPLIT;  // bins per CTA
  PdlEnter(its, kTraceFold);
  const SigIter &it = its[blockIdx.z];
  if (!it.active || it.force_fp64) return;
  const int B = it.bins;
  const int g = blockIdx.y % gmax;
  const int tr = blockIdx.y / gmax;
  if (tr >= it.trials || g > it.bits) return;
  // the stash's header: whether this fold stashes its gathered samples (the
  // pairwise shapes on complex64 input do; the row cluster does not)
  constexpr bool kStash = !CLUSTER && sizeof(TX) == sizeof(float2);
  if (it.stash != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
    *reinterpret_cast<int32_t *>(it.stash) = kStash ? 1 : 0;
  }
  const int sc = CLUSTER ? ClusterGroups(it.folds, it.bits) : -1;
  if (g <= sc) {
    // the row cluster on the CTAs of groups 0..sc: a warp per base bin
    __shared__ float2 slices[kWarpsPerCta][kMirrorOff + kMaxClusterSpan];
    const int nb = (B + 1) >> 1;
    const int ctas = (sc + 1) * int(gridDim.x);
    const int w = threadIdx.x >> 5;
    for (int cta = g * int(gridDim.x) + int(blockIdx.x); cta * kWarpsPerCta < nb;
         cta += ctas) {
      const int beta = cta * kWarpsPerCta + w;
      if (beta < nb) FoldClusterWarp<TX>(it, tr, beta, sc, slices[w]);
    }
    return;
  }
  if (int(blockIdx.x) * kFoldBins >= B) return;

  const int lane = threadIdx.x & (kFoldSplit - 1);
  const int beta = blockIdx.x * kFoldBins + threadIdx.x / kFoldSplit;
  const bool valid = beta < B;
  const uint32_t n = uint32_t(it.n);
  const ModN mod{n, it.n_inv};
  const int64_t off = g == 0 ? 0 : (int64_t(B) << (g - 1));
  const bool pair = g > 0;
  // first t of this lane: t = beta mod B with |t| <= p2 (-p2 = (B + 1)/2 mod B
  // since p = f B with f odd), then every kFoldSplit-th fold
  int tm = beta - (B + 1) / 2;
  if (tm < 0) tm += B;
  int64_t t = -int64_t(it.p2) + tm + int64_t(lane) * B;
  const int f = it.folds;
  const int cnt = (valid && f > lane) ? (f - lane + kFoldSplit - 1) / kFoldSplit : 0;
  const int64_t q = it.q[tr];
  const int64_t a = it.a, c = it.c;
  uint32_t j1 = mod(a * mod(q + t + off) + c);
  uint32_t j2 = mod(a * mod(q - t - off) + c);
  const int64_t D = int64_t(kFoldSplit) * B;
  const uint32_t aD = mod(a * mod(D));
  uint64_t ph = it.phi_b * uint64_t(t + off) - it.psi * uint64_t(t);
  const uint64_t dph = (it.phi_b - it.psi) * uint64_t(D);

  const TX *__restrict__ x = reinterpret_cast<const TX *>(it.x);
  const float *__restrict__ wt = it.wt32;
  // stashed rows of this group (the + row, the - row) and their samples
  // at t = 0
  const int srows = kStash ? StashRows(it) : 0;
  const int rp = g == 0 ? 0 : 2 * g - 1, rm = 2 * g;
  TX *sp = nullptr, *sm = nullptr;
  if (rp < srows) {
    sp = reinterpret_cast<TX *>(it.stash + kStashHeader) +
         (size_t(tr) * srows + rp) * it.p + it.p2;
  }
  if (pair && rm < srows) {
    sm = reinterpret_cast<TX *>(it.stash + kStashHeader) +
         (size_t(tr) * srows + rm) * it.p + it.p2;
  }
  CompF r1, i1, r2, i2;
  for (int k0 = 0; k0 < cnt; k0 += kFoldBatch) {
    TX x1[kFoldBatch], x2[kFoldBatch];
    float w[kFoldBatch];
    uint32_t p32[kFoldBatch];
    const int64_t tb = t;  // t of the batch's first fold
#pragma unroll
    for (int u = 0; u < kFoldBatch; ++u) {
      if (k0 + u < cnt) {
        x1[u] = __ldg(&x[j1]);
        if (pair) x2[u] = __ldg(&x[j2]);
        w[u] = __ldg(&wt[t < 0 ? -t : t]);
        p32[u] = uint32_t((ph + (uint64_t(1) << 31)) >> 32);
        j1 = StepUp(j1, aD, n);
        j2 = StepDown(j2, aD, n);
        ph += dph;
        t += D;
      }
    }
#pragma unroll
    for (int u = 0; u < kFoldBatch; ++u) {
      if (k0 + u < cnt) {
        const float phi = float(int32_t(p32[u])) * 2.3283064365386963e-10f;
        float s, co;
        sincospif(2.0f * phi, &s, &co);
        const float wr = co * w[u], wi = s * w[u];
        const float2 v1 = to_f2(x1[u]);
        r1.add(v1.x * wr - v1.y * wi);
        i1.add(v1.x * wi + v1.y * wr);
        if (pair) {
          const float2 v2 = to_f2(x2[u]);
          r2.add(v2.x * wr + v2.y * wi);
          i2.add(v2.y * wr - v2.x * wi);
        }
        // the + row's sample at t, the - row's at -t
        const int64_t tu = tb + int64_t(u) * D;
        if (sp != nullptr) sp[tu] = x1[u];
        if (sm != nullptr) sm[-tu] = x2[u];
      }
    }
  }
#pragma unroll
  for (int o = 1; o < kFoldSplit; o <<= 1) {
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
  if (lane == 0 && valid) {
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
  PdlEnter();
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

// The FP32 fold's launch shapes (complex64 input; complex128 input uses
// shape 0): (SPLIT, BATCH, CLUSTER), shape 0 the default.
using FoldKernel = void (*)(const SigIter *, int);
const FoldKernel kFoldKernels[kFoldShapes] = {
    k_bin_fold32<float2, 4, 4, true>,  k_bin_fold32<float2, 2, 4, true>,
    k_bin_fold32<float2, 8, 4, true>,  k_bin_fold32<float2, 4, 8, true>,
    k_bin_fold32<float2, 2, 8, true>,  k_bin_fold32<float2, 8, 8, true>,
    k_bin_fold32<float2, 4, 4, false>, k_bin_fold32<float2, 2, 4, false>,
    k_bin_fold32<float2, 8, 4, false>, k_bin_fold32<float2, 4, 8, false>,
    k_bin_fold32<float2, 2, 8, false>, k_bin_fold32<float2, 8, 8, false>,
};

}  // namespace

FoldShape FoldShapeOf(int shape) {
  static const int8_t kSplit[kFoldShapes] = {4, 2, 8, 4, 2, 8, 4, 2, 8, 4, 2, 8};
  static const int8_t kBatch[kFoldShapes] = {4, 4, 4, 8, 8, 8, 4, 4, 4, 8, 8, 8};
  if (shape < 0 || shape >= kFoldShapes) shape = 0;
  FoldShape f;
  f.split = kSplit[shape];
  f.batch = kBatch[shape];
  f.cluster = shape < 6;
  f.bins_per_cta = 256 / f.split;
  return f;
}

void LaunchBinFold(const SigIter *d_its, int nsig, int max_bins, int max_bits,
                   int max_trials, bool x_c128, bool fp64, cudaStream_t s,
                   bool cond, int shape) {
  if (shape < 0 || shape >= kFoldShapes) shape = 0;
  const int gmax = max_bits + 1;
  dim3 grid((max_bins + 31) / 32, gmax * max_trials, nsig);
  if (fp64) {
    if (x_c128) {
      Launch(k_bin_fold64<double2>, grid, 256, 0, s, d_its, gmax, cond ? 1 : 0);
    } else {
      Launch(k_bin_fold64<float2>, grid, 256, 0, s, d_its, gmax, cond ? 1 : 0);
    }
  } else {
    const FoldShape sh = FoldShapeOf(x_c128 ? 0 : shape);
    dim3 grid32((max_bins + sh.bins_per_cta - 1) / sh.bins_per_cta,
                gmax * max_trials, nsig);
    if (x_c128) {
      Launch(k_bin_fold32<double2, 4, 4, true>, grid32, 256, 0, s, d_its, gmax);
    } else {
      Launch(kFoldKernels[shape], grid32, 256, 0, s, d_its, gmax);
    }
  }
}

}  // namespace mpsft

