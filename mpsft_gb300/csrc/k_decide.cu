// Mode bucketing, frequency-domain subtraction of found modes, per-bin
// identification and coefficient estimation, and the mode-table merge.
//
// Reference: BinInFreqV1::Run (src/binner.cc:565-591), the bin loop of
// Iterate (src/iterate.cc:113-175), IdentifyFreq (src/iterate.cc:44-76) and
// MatPencil (src/freqid.cc:27-48). All of it runs in FP64.
//
// One warp per (bin, signal): lane s holds rows 2s+1 and 2s+2 (bit s) of
// every trial, all lanes hold row 0. A bin's modes are taken in increasing
// k0, so the subtraction order does not depend on the table layout and the
// result is bit-reproducible.
#include "common.cuh"
#include "launch.h"

namespace mpsft {

namespace {

// ---------------------------------------------------------------- bucket
// Counting sort of the table's slots by the bin of their mode under the
// current permutation: bin = ((a k0 + b) mod n) * bins / n.
__global__ void __launch_bounds__(1024) k_bucket(const SigIter *__restrict__ its) {
  extern __shared__ int32_t cnt[];  // bins entries
  __shared__ int32_t warp_tot[32];
  const SigIter &it = its[blockIdx.x];
  if (!it.active) return;
  const int B = it.bins, cap = it.tab_cap;
  const int64_t n = it.n;
  for (int i = threadIdx.x; i < B; i += blockDim.x) cnt[i] = 0;
  __syncthreads();
  for (int s = threadIdx.x; s < cap; s += blockDim.x) {
    const int32_t key = it.tab_key[s];
    if (key == kEmptyKey) continue;
    const int64_t k1 = PosMod(int64_t(it.a) * key + it.b, n);
    atomicAdd(&cnt[int(k1 * B / n)], 1);
  }
  __syncthreads();
  // Exclusive scan: each thread owns a contiguous chunk of bins.
  const int chunk = (B + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * chunk;
  const int hi = min(lo + chunk, B);
  int local = 0;
  for (int i = lo; i < hi; ++i) local += cnt[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = lane < int(blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += v;
    }
    warp_tot[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  int run = incl - local + (warp > 0 ? warp_tot[warp - 1] : 0);
  for (int i = lo; i < hi; ++i) {
    const int c = cnt[i];
    it.bkt_count[i] = c;
    it.bkt_start[i] = run;
    run += c;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < B; i += blockDim.x) cnt[i] = 0;
  __syncthreads();
  for (int s = threadIdx.x; s < cap; s += blockDim.x) {
    const int32_t key = it.tab_key[s];
    if (key == kEmptyKey) continue;
    const int64_t k1 = PosMod(int64_t(it.a) * key + it.b, n);
    const int bin = int(k1 * B / n);
    const int pos = it.bkt_start[bin] + atomicAdd(&cnt[bin], 1);
    it.bkt_list[pos] = s;
  }
}

__device__ inline double2 ShflXor(double2 v, int o) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, o),
                      __shfl_xor_sync(0xffffffffu, v.y, o));
}

// Loads the bin's rows, subtracts the bin's modes (BinInFreqV1), and, unless
// subtract_only, runs the decisions and writes the candidate.
template <int TMAX>
__device__ void DecideBin(const SigIter &it, int beta, bool subtract_only) {
  const int lane = threadIdx.x & 31;
  const int L = it.bits, T = it.trials, rows = it.rows;
  const int64_t n = it.n;
  const int B = it.bins;
  const bool has_bit = lane < L;
  const size_t cap = size_t(it.bins_cap);
  double2 u0[TMAX], up[TMAX], um[TMAX];
#pragma unroll
  for (int t = 0; t < TMAX; ++t) {
    if (t < T) {
      const double2 *base = it.ubuf + size_t(t) * rows * cap;
      u0[t] = base[beta];
      if (has_bit) {
        up[t] = base[(2 * lane + 1) * cap + beta];
        um[t] = base[(2 * lane + 2) * cap + beta];
      } else {
        up[t] = um[t] = make_double2(0, 0);
      }
    }
  }
  const int64_t off = has_bit ? (int64_t(B) << lane) : 0;

  // ---- subtraction of the modes found so far, in increasing k0
  const int nm = it.bkt_count[beta];
  const int st = it.bkt_start[beta];
  int32_t last = INT32_MIN;
  bool have_last = false;
  for (int i = 0; i < nm; ++i) {
    int32_t best = INT32_MAX;
    int best_slot = -1;
    for (int j = 0; j < nm; ++j) {
      const int sl = it.bkt_list[st + j];
      const int32_t key = it.tab_key[sl];
      if ((!have_last || key > last) && (best_slot < 0 || key < best)) {
        best = key;
        best_slot = sl;
      }
    }
    last = best;
    have_last = true;
    const int32_t k0 = best;
    const double2 coef = it.tab_coef[best_slot];
    const int64_t k1 = PosMod(int64_t(it.a) * k0 + it.b, n);
    const double xi = (double(beta) + 0.5) / double(B) - double(k1) / double(n);
    const double wf = WindowInFreq(it, xi);
    const double2 wc = cscale(coef, wf);
    double2 fac = make_double2(1, 0);
    if (has_bit) fac = UnitPhase64(off * k1, n);
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < T) {
        const int64_t ph = int64_t(it.q[t]) * k1 + int64_t(it.c) * k0;
        const double2 bs = cmul(wc, UnitPhase64(ph, n));
        u0[t] = csub(u0[t], bs);
        if (has_bit) {
          up[t] = csub(up[t], cmul(bs, fac));
          um[t] = csub(um[t], cmul(bs, cconj(fac)));
        }
      }
    }
  }
  if (subtract_only) {
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < T) {
        double2 *base = it.ubuf + size_t(t) * rows * cap;
        if (lane == 0) base[beta] = u0[t];
        if (has_bit) {
          base[(2 * lane + 1) * cap + beta] = up[t];
          base[(2 * lane + 2) * cap + beta] = um[t];
        }
      }
    }
    return;
  }

  // ---- non-finite input is reported instead of being voted on
  bool finite = true;
#pragma unroll
  for (int t = 0; t < TMAX; ++t) {
    if (t < T) {
      finite = finite && isfinite(u0[t].x) && isfinite(u0[t].y) &&
               isfinite(up[t].x) && isfinite(up[t].y) && isfinite(um[t].x) &&
               isfinite(um[t].y);
    }
  }
  if (__any_sync(0xffffffffu, !finite)) {
    if (lane == 0) {
      atomicOr(&it.flags[1], kStatusNonFinite);
      it.cand_valid[beta] = 0;
    }
    return;
  }

  // ---- energy threshold (src/iterate.cc:114-124)
  double e = 0;
#pragma unroll
  for (int t = 0; t < TMAX; ++t) {
    if (t < T) e += u0[t].x * u0[t].x + u0[t].y * u0[t].y;
  }
  e /= T;
  if (it.bin_thr > 0 && e < it.bin_thr * it.bin_thr) {
    if (lane == 0) it.cand_valid[beta] = 0;
    return;
  }

  // ---- IdentifyFreq: per-bit majority of the pencil votes, sv rejection
  int count = 0;
  bool sv_fail = false;
  if (has_bit) {
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < T) {
        double s0, s1;
        if (Pencil(u0[t], up[t], um[t], &s0, &s1)) ++count;
        if (it.sv_thr > 0 && s1 * 0.5 > it.sv_thr) sv_fail = true;
      }
    }
  }
  if (__any_sync(0xffffffffu, sv_fail)) {
    if (lane == 0) it.cand_valid[beta] = 0;
    return;
  }
  const uint32_t mask = __ballot_sync(0xffffffffu, has_bit && count > T / 2);
  // bit 0 is the most significant digit of xi
  const uint32_t xs = L > 0 ? (__brev(mask) >> (32 - L)) : 0u;
  const double xi1 = ldexp(2.0 * double(xs) + 1.0, -(L + 1));
  const int32_t k1 =
      int32_t(round(double(n) * (double(beta) + xi1) / double(B)));
  const double xi0 = double(k1) / double(n) - (double(beta) + 0.5) / double(B);
  const double wf = WindowInFreq(it, xi0);
  if (fabs(wf) < it.win_thr) {
    if (lane == 0) it.cand_valid[beta] = 0;
    return;
  }

  // ---- coefficient (src/iterate.cc:146-171)
  double2 acc = make_double2(0, 0);
  double2 fac2 = make_double2(1, 0);
  if (has_bit) fac2 = UnitPhase64(-off * k1, n);
#pragma unroll
  for (int t = 0; t < TMAX; ++t) {
    if (t < T) {
      const double2 fac = UnitPhase64(-int64_t(it.q[t]) * k1, n);
      if (lane == 0) acc = cadd(acc, cmul(u0[t], fac));
      if (has_bit) {
        acc = cadd(acc, cmul(up[t], cmul(fac, fac2)));
        acc = cadd(acc, cmul(um[t], cmul(fac, cconj(fac2))));
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc = cadd(acc, ShflXor(acc, o));
  if (lane == 0) {
    double2 coef = cscale(acc, 1.0 / double(T * (1 + 2 * L)));
    const int32_t k0 =
        int32_t(PosMod(int64_t(it.a_inv) * (int64_t(k1) - it.b), n));
    coef = cmul(coef, UnitPhase64(-int64_t(it.c) * k0, n));
    coef = make_double2(coef.x / wf, coef.y / wf);
    it.cand_k0[beta] = k0;
    it.cand_coef[beta] = coef;
    it.cand_valid[beta] = 1;
    it.flags[0] = 1;
  }
}

template <int TMAX>
__global__ void __launch_bounds__(256)
    k_decide(const SigIter *__restrict__ its, int subtract_only) {
  const SigIter &it = its[blockIdx.y];
  if (!it.active) return;
  const int beta = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (beta >= it.bins) return;
  DecideBin<TMAX>(it, beta, subtract_only != 0);
}

// ---------------------------------------------------------------- merge
__device__ void InsertMode(const SigIter &it, int32_t k0, double2 coef) {
  const int cap = it.tab_cap;
  uint32_t slot = KeySlot(k0, cap);
  for (int probe = 0; probe < cap; ++probe) {
    const int32_t prev = atomicCAS(&it.tab_key[slot], kEmptyKey, k0);
    if (prev == kEmptyKey) {
      atomicAdd(it.tab_count, 1);
    }
    if (prev == kEmptyKey || prev == k0) {
      atomicAdd(&it.tab_coef[slot].x, coef.x);
      atomicAdd(&it.tab_coef[slot].y, coef.y);
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
  InsertMode(it, it.cand_k0[beta], it.cand_coef[beta]);
}

__global__ void k_table_insert(const SigIter *__restrict__ it,
                               const int32_t *__restrict__ k0,
                               const double2 *__restrict__ coef, int64_t m) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= m) return;
  InsertMode(*it, k0[i], coef[i]);
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

template <int TMAX>
void LaunchDecideT(const SigIter *d_its, int nsig, int max_bins, int sub,
                   cudaStream_t s) {
  dim3 grid((max_bins + 7) / 8, nsig);
  k_decide<TMAX><<<grid, 256, 0, s>>>(d_its, sub);
}

}  // namespace

void LaunchBucket(const SigIter *d_its, int nsig, int max_bins, int max_cap,
                  cudaStream_t s) {
  (void)max_cap;
  k_bucket<<<nsig, 1024, size_t(max_bins) * sizeof(int32_t), s>>>(d_its);
}

// The trial count selects the register footprint of the decide kernel.
void LaunchDecide(const SigIter *d_its, int nsig, int max_bins, int max_trials,
                  bool subtract_only, cudaStream_t s) {
  const int sub = subtract_only ? 1 : 0;
  if (max_trials <= 1) {
    LaunchDecideT<1>(d_its, nsig, max_bins, sub, s);
  } else if (max_trials <= 5) {
    LaunchDecideT<5>(d_its, nsig, max_bins, sub, s);
  } else {
    LaunchDecideT<kMaxTrials>(d_its, nsig, max_bins, sub, s);
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
