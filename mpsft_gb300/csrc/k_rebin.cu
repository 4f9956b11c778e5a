// Re-binning of the near-tie bins listed by the FP32 decide pass, with
// FP64-class accuracy but on the FP32 pipes (this part has only about 1/64 of
// the FP32 rate in FP64 arithmetic).
//
// A listed bin beta of row r (offset tau_r = q + off) is evaluated directly,
// without the fold and the FFT:
//   U_r[beta] = sum_{t=-p2}^{p2} x[(a (tau_r + t) + c) mod n] wt(t) e^{2 pi i phi(t)},
//   phi(t) = (b (tau_r + t) mod n)/n - (2 beta + 1) t/(2B)
// (the fold, the size-B DFT and the row factor of BinInTime::Run in one sum,
// src/binner.cc:394-521). phi advances by the same Delta = b/n - (2 beta + 1)/(2B)
// (mod 1) per sample, so with s = e^{2 pi i Delta} a run of samples starting
// at t0 is
//   sum_{k} x_k w_k e^{2 pi i phi(t0 + k)} = sum_blocks A_blk sum_{k<64} x_k w_k s^k,
// A_blk = e^{2 pi i phi(t0)} s^{64 blk}. The inner sums run in float-float
// arithmetic (each value as an unevaluated sum hi + lo of two floats, about
// 2^-47 relative) against a per-bin table of s^k (k < 64) computed in FP64
// from exact integer phases; each block sum then enters an FP64 total through
// A_blk. The window comes from a float-float table of the FP64 window.
//
// The samples x[(a (tau_r + t) + c) mod n] come from the stash the FP32 fold
// wrote when it stashed the row (StashRows: every row when the fold gathers
// from few sectors, else row 0), read in order, and are gathered from x
// again otherwise (random accesses, at the random-gather rate).
//
// Work item = (signal, listed bin, trial, listed row, chunk of the support;
// RebinChunks(p) chunks),
// one warp each; the 32 lanes split the chunk into consecutive runs; lane sums
// are combined by a fixed shuffle tree and the chunk partials are added in
// chunk order by whichever warp finishes a row's last chunk (so the result
// does not depend on the scheduling).
#include "common.cuh"
#include "launch.h"
#include "rebin.cuh"

namespace mpsft {

namespace {

// x*y + u*v in float-float: exact products of the high parts (FMA), two-sum
// of those, the cross terms in the low word, then renormalisation.
__device__ __forceinline__ FF DotFF(FF x, FF y, FF u, FF v) {
  const float p1 = __fmul_rn(x.hi, y.hi);
  const float e1 = fmaf(x.hi, y.hi, -p1);
  const float p2 = __fmul_rn(u.hi, v.hi);
  const float e2 = fmaf(u.hi, v.hi, -p2);
  const float s = __fadd_rn(p1, p2);
  const float bb = __fsub_rn(s, p1);
  float lo = __fadd_rn(__fsub_rn(p1, __fsub_rn(s, bb)), __fsub_rn(p2, bb));
  lo = __fadd_rn(lo, __fadd_rn(e1, e2));
  lo = fmaf(x.hi, y.lo, lo);
  lo = fmaf(x.lo, y.hi, lo);
  lo = fmaf(u.hi, v.lo, lo);
  lo = fmaf(u.lo, v.hi, lo);
  const float h = __fadd_rn(s, lo);
  return {h, __fsub_rn(lo, __fsub_rn(h, s))};
}

// acc += t (two-sum of the high words, renormalised)
__device__ __forceinline__ void AccFF(FF &acc, FF t) {
  const float s = __fadd_rn(acc.hi, t.hi);
  const float bb = __fsub_rn(s, acc.hi);
  float lo = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(t.hi, bb));
  lo = __fadd_rn(lo, __fadd_rn(acc.lo, t.lo));
  const float h = __fadd_rn(s, lo);
  acc.lo = __fsub_rn(lo, __fsub_rn(h, s));
  acc.hi = h;
}

__device__ __forceinline__ FF Neg(FF a) { return {-a.hi, -a.lo}; }

// x * w with x an input sample and w the float-float window: complex64
// samples are exact floats (exact product of the high word by FMA); complex128
// samples are multiplied in FP64 first.
__device__ __forceinline__ void SampleTimesWindow(float2 v, float2 w, FF *re,
                                                  FF *im) {
  float p = __fmul_rn(v.x, w.x);
  re->hi = p;
  re->lo = fmaf(v.x, w.y, fmaf(v.x, w.x, -p));
  p = __fmul_rn(v.y, w.x);
  im->hi = p;
  im->lo = fmaf(v.y, w.y, fmaf(v.y, w.x, -p));
}
__device__ __forceinline__ void SampleTimesWindow(double2 v, float2 w, FF *re,
                                                  FF *im) {
  const double wd = double(w.x) + double(w.y);
  *re = FFOf(v.x * wd);
  *im = FFOf(v.y * wd);
}

// The samples t0 <= t < t1 of a work item summed against the bin's phase
// steps (s^k in pw, s^64 in S, e^{2 pi i phi(t0)} = (ar, ai)) into (tr, ti).
// FROM_STASH: the samples read in order from the fold's stash (src[t]);
// else gathered, x[j] with j stepping by a mod n. The two are separate loops,
// so that each keeps its eight loads in flight together.
template <typename TX, bool FROM_STASH>
__device__ __forceinline__ void SumRun(const TX *__restrict__ src, uint32_t j,
                                       uint32_t astep, uint32_t nn,
                                       const float2 *__restrict__ wff,
                                       const float4 *pw, int64_t t0, int64_t t1,
                                       double2 S, double ar, double ai, double *tr,
                                       double *ti) {
  for (int64_t tb = t0; tb < t1; tb += kPowLen) {
    const int len = int(min(int64_t(kPowLen), t1 - tb));
    FF sr{0.f, 0.f}, si{0.f, 0.f};
    for (int kb = 0; kb < len; kb += 8) {
      TX v[8];
      float2 wv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (kb + u < len) {
          const int64_t tt = tb + kb + u;
          if (FROM_STASH) {
            v[u] = __ldg(&src[tt]);
          } else {
            v[u] = __ldg(&src[j]);
            j += astep;
            if (j >= nn) j -= nn;
          }
          wv[u] = __ldg(&wff[tt < 0 ? -tt : tt]);
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (kb + u < len) {
          FF xr, xi;
          SampleTimesWindow(v[u], wv[u], &xr, &xi);
          const float4 p = pw[kb + u];
          const FF pr{p.x, p.z}, pi{p.y, p.w};
          // (xr + i xi)(pr + i pi)
          AccFF(sr, DotFF(xr, pr, Neg(xi), pi));
          AccFF(si, DotFF(xr, pi, xi, pr));
        }
      }
    }
    const double br = double(sr.hi) + double(sr.lo);
    const double bi = double(si.hi) + double(si.lo);
    *tr += ar * br - ai * bi;
    *ti += ar * bi + ai * br;
    const double nar = ar * S.x - ai * S.y;
    ai = ar * S.y + ai * S.x;
    ar = nar;
  }
}

// The preparation of the direct evaluation of every bin (mpsft_bin_in_time,
// FP64_DIRECT): one warp per listed bin. A solve's FP32 decide kernel
// prepares its listed bins itself when it lists them.
__global__ void __launch_bounds__(256) k_rebin_prep(const SigIter *__restrict__ its) {
  PdlEnter();
  const SigIter &it = its[blockIdx.y];
  if (!it.active || it.force_fp64) return;
  const int nf = *(volatile int32_t *)&it.flags[2];
  if (nf > it.esc_cap) return;
  const int e = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (e >= nf) return;
  PrepListedBin(it, e, it.esc_list[e], threadIdx.x & 31);
}

template <typename TX>
__global__ void __launch_bounds__(256, 2)
    k_rebin_ff(const SigIter *__restrict__ its, int nsig) {
  PdlEnter(its, kTraceRebin);
  __shared__ int64_t items_end[kRebinMaxSignals];
  __shared__ float4 pw_s[8][kPowLen];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // the signals' work item counts and their inclusive prefix sums, by warp 0
  // (32 signals per step, a shuffle scan each)
  if (warp == 0) {
    int64_t carry = 0;
    for (int s0 = 0; s0 < nsig; s0 += 32) {
      const int s = s0 + lane;
      int64_t items = 0;
      if (s < nsig) {
        const SigIter &q = its[s];
        if (q.active && !q.force_fp64) {
          const int nf = *(volatile int32_t *)&q.flags[2];
          if (nf <= q.esc_cap) items = int64_t(nf) * q.trials * q.rows * RebinChunks(q.p);
        }
      }
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t v = __shfl_up_sync(0xffffffffu, items, o);
        if (lane >= o) items += v;
      }
      if (s < nsig) items_end[s] = carry + items;
      carry += __shfl_sync(0xffffffffu, items, 31);
    }
  }
  __syncthreads();
  float4 *pw = pw_s[warp];
  const int64_t total = items_end[nsig - 1];
  for (int64_t w = int64_t(blockIdx.x) * 8 + warp; w < total;
       w += int64_t(gridDim.x) * 8) {
    int sig = 0;
    while (w >= items_end[sig]) ++sig;
    // (a signal's items: at most kMaxListed * kMaxTrials * rows * chunks,
    // far below 2^32, so the decode divides in 32 bits)
    uint32_t local = uint32_t(w - (sig > 0 ? items_end[sig - 1] : 0));
    const SigIter &it = its[sig];
    const int nch = RebinChunks(it.p);
    const int c = int(local % uint32_t(nch));
    local /= uint32_t(nch);
    const int r = int(local % uint32_t(it.rows));
    local /= uint32_t(it.rows);
    const int t = int(local % uint32_t(it.trials));
    const int e = int(local / uint32_t(it.trials));
    // row not listed (a null mask lists every row)
    if (r > 0 && it.esc_mask != nullptr &&
        !((it.esc_mask[e] >> ((r - 1) >> 1)) & 1u)) {
      continue;
    }
    const int beta = it.esc_list[e];
    const int64_t n = it.n;
    const int64_t B = it.bins;
    const ModN mod{uint32_t(n), it.n_inv};
    int64_t off = 0;
    if (r > 0) {
      const int s = (r - 1) / 2;
      off = (r & 1) ? (B << s) : -(B << s);
    }
    const int64_t tau = int64_t(it.q[t]) + off;
    const int64_t chunk = (int64_t(it.p) + nch - 1) / nch;
    const int64_t c0 = -int64_t(it.p2) + c * chunk;
    const int64_t c1 = min(c0 + chunk, int64_t(it.p2) + 1);
    const int64_t per = (chunk + 31) / 32;
    const int64_t t0 = c0 + lane * per;
    const int64_t t1 = min(t0 + per, c1);
    // the bin's phase-step powers s^k (k < 64) into shared memory and s^64
    // (StepPowers): from the per-bin tables its preparation filled, else
    // evaluated here
    const int64_t g = 2 * int64_t(beta) + 1;
    const uint32_t bm = mod(it.b);
    float4 p0, p1;
    double2 S;
    if (it.esc_pow != nullptr) {
      p0 = it.esc_pow[size_t(e) * kPowLen + lane];
      p1 = it.esc_pow[size_t(e) * kPowLen + lane + 32];
      S = it.esc_step[e];
    } else {
      StepPowers(it, beta, lane, &p0, &p1, &S);
    }
    __syncwarp();
    pw[lane] = p0;
    pw[lane + 32] = p1;
    __syncwarp();
    double tr = 0.0, ti = 0.0;
    // the row's samples from the fold's stash when it wrote them (read in
    // order), else gathered from x
    const TX *__restrict__ sx = nullptr;
    if (it.stash != nullptr && __ldcg(reinterpret_cast<const int32_t *>(it.stash)) == 1) {
      const int srows = StashRows(it);
      if (r < srows) {
        sx = reinterpret_cast<const TX *>(it.stash + kStashHeader) +
             (size_t(t) * srows + r) * it.p + it.p2;
      }
    }
    if (t0 < t1) {
      const int64_t twoB = 2 * B;
      const int64_t u0 = mod(tau + t0);
      uint32_t j = mod(int64_t(it.a) * u0 + it.c);
      const uint32_t astep = mod(it.a);
      const uint32_t nn = uint32_t(n);
      const int64_t m0 = mod(int64_t(bm) * u0);
      const int64_t r0 = PosMod(g * t0, twoB);
      const double2 a0 = StepPhase(it, m0, r0);
      // (only complex64 input has a stash)
      if (sizeof(TX) == sizeof(float2) && sx != nullptr) {
        SumRun<TX, true>(sx, 0u, 0u, 0u, it.wtff, pw, t0, t1, S, a0.x, a0.y, &tr, &ti);
      } else {
        SumRun<TX, false>(reinterpret_cast<const TX *>(it.x), j, astep, nn, it.wtff, pw,
                          t0, t1, S, a0.x, a0.y, &tr, &ti);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      tr += __shfl_xor_sync(0xffffffffu, tr, o);
      ti += __shfl_xor_sync(0xffffffffu, ti, o);
    }
    // the warp that completes a (trial, row) adds its chunk partials in
    // chunk order (the result does not depend on which warp that is)
    const size_t etr = (size_t(e) * it.trials + t) * it.rows + r;
    int last = 0;
    if (lane == 0) {
      it.esc_part[etr * kRebinChunks + c] = make_double2(tr, ti);
      __threadfence();
      last = atomicAdd(&it.esc_cnt[etr], 1) == nch - 1;
    }
    if (__shfl_sync(0xffffffffu, last, 0) && lane == 0) {
      __threadfence();
      double2 s = __ldcg(&it.esc_part[etr * kRebinChunks]);
      for (int cc = 1; cc < nch; ++cc) {
        const double2 p = __ldcg(&it.esc_part[etr * kRebinChunks + cc]);
        s.x += p.x;
        s.y += p.y;
      }
      it.esc_sum[etr] = s;
    }
  }
}

}  // namespace

void LaunchRebin(const SigIter *d_its, int nsig, int max_listed, bool x_c128,
                 bool prepare, cudaStream_t s) {
  // optionally the listed bins' preparation (a solve's decide kernel does it
  // when it lists them), then a persistent grid whose warps stride over the
  // work items; batches are cut into groups of at most kRebinMaxSignals
  if (prepare) {
    dim3 pgrid((max_listed + 7) / 8, nsig);
    Launch(k_rebin_prep, pgrid, 256, 0, s, d_its);
  }
  const int blocks = 152 * 2;  // two resident blocks per SM (124 registers)
  for (int s0 = 0; s0 < nsig; s0 += kRebinMaxSignals) {
    const int cnt = nsig - s0 < kRebinMaxSignals ? nsig - s0 : kRebinMaxSignals;
    if (x_c128) {
      Launch(k_rebin_ff<double2>, blocks, 256, 0, s, d_its + s0, cnt);
    } else {
      Launch(k_rebin_ff<float2>, blocks, 256, 0, s, d_its + s0, cnt);
    }
  }
}

bool RebinKernelsLaunchable() {
  int a = 0, b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_rebin_ff<float2>, 256, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_rebin_ff<double2>, 256, 0);
  return a > 0 && b > 0;
}

}  // namespace mpsft
