// Found-mode preparation and bucketing, frequency-domain subtraction of found
// modes, per-bin identification and coefficient estimation, and the merge of
// the new modes into the table.
//
// Reference: BinInFreqV1::Run (src/binner.cc:565-591), the bin loop of
// Iterate (src/iterate.cc:113-175), IdentifyFreq (src/iterate.cc:44-76) and
// MatPencil (src/freqid.cc:27-48).
//
// k_mode_prep (threads striding over the occupied slots) evaluates, once per
// mode and iteration, what BinInFreq needs from a mode: k1 = (a k0 + b) mod n,
// its bin,
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
#include "decide.cuh"
#include "launch.h"

namespace mpsft {

namespace {

// ---------------------------------------------------------------- prep
// Per occupied slot (the table's insertion list): k1 = (a k0 + b)
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

// One occupied slot s of k_mode_prep.
__device__ void ModePrepSlot(const SigIter &it, int s, int cond) {
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

__global__ void k_mode_prep(const SigIter *__restrict__ its, int cond) {
  PdlEnter(its, kTraceModePrep);
  const SigIter &it = its[blockIdx.y];
  if (!it.active) return;
  if (cond && !RedoFP64(it)) return;
  // a few blocks per signal striding over the occupied slots (a grid over
  // the whole table would flood the SMs with empty blocks at the start of
  // every iteration, ahead of the other streams' kernels)
  const int count = *it.tab_count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += gridDim.x * blockDim.x) {
    ModePrepSlot(it, it.occ_list[i], cond);
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

// Sorts the occupied slots by (bin, k0): a counting sort by bin (per-bin
// counts, their exclusive scan, then each slot's key k0 << 20 | slot placed
// in its bin's run), then each bin's run sorted by k0 by one thread
// (insertion sort; a run holds the few modes of one bin). The subtraction
// later walks each bin's modes in increasing k0, an order that does not
// depend on the table layout. Thread 0 also evaluates this iteration's FP32
// error scale eps. Shared memory: the keys (half the table, BucketKeys),
// then the bins' counts and fill positions.
__global__ void __launch_bounds__(1024) k_bucket(const SigIter *__restrict__ its,
                                                 int max_bins, int prep) {
  PdlEnter(its, kTraceBucket);
  extern __shared__ unsigned long long keys[];
  const SigIter &it = its[blockIdx.x];
  if (!it.active) return;
  const int B = it.bins;
  const int occ = *it.tab_count;
  if (prep) {
    // the mode preparation of k_mode_prep for this signal's slots first
    // (one kernel fewer at the start of an iteration)
    for (int i = threadIdx.x; i < occ; i += blockDim.x) {
      ModePrepSlot(it, it.occ_list[i], 0);
    }
    __syncthreads();  // their bins are visible to the whole block
  }
  int *cnt = reinterpret_cast<int *>(keys + BucketKeys(it.tab_cap));
  int *fill = cnt + max_bins;
  // shared keys were sized for half the table (BucketKeys); more occupied
  // slots end the solve with a capacity status instead of overflowing
  if (occ > BucketKeys(it.tab_cap)) {
    if (threadIdx.x == 0) atomicOr(&it.flags[1], kStatusCapacity);
    return;
  }
  for (int b = threadIdx.x; b < B; b += blockDim.x) cnt[b] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < occ; i += blockDim.x) {
    atomicAdd(&cnt[it.mode_bin[it.occ_list[i]]], 1);
  }
  __syncthreads();
  // exclusive scan of the counts: each thread a contiguous chunk, then the
  // chunk totals by warp shuffles and one pass over the warps' totals
  __shared__ int warp_tot[32];
  const int per = (B + blockDim.x - 1) / blockDim.x;
  const int b0 = threadIdx.x * per;
  int local = 0;
  for (int b = b0; b < b0 + per && b < B; ++b) local += cnt[b];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) {
      const int t = warp_tot[w];
      warp_tot[w] = acc;
      acc += t;
    }
  }
  __syncthreads();
  int run = warp_tot[warp] + incl - local;
  for (int b = b0; b < b0 + per && b < B; ++b) {
    fill[b] = run;
    it.bkt_start[b] = run;
    it.bkt_count[b] = cnt[b];
    run += cnt[b];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < occ; i += blockDim.x) {
    const int sl = it.occ_list[i];
    const int pos = atomicAdd(&fill[it.mode_bin[sl]], 1);
    keys[pos] = (static_cast<unsigned long long>(uint32_t(it.tab_key[sl])) << 20) |
                static_cast<unsigned long long>(sl);
  }
  __syncthreads();
  // each bin's run in increasing k0 (keys are distinct: one slot per k0): a
  // key's place in its run is the number of smaller keys in the run, every
  // key ranked by its own thread (runs are a bin's few modes)
  for (int i = threadIdx.x; i < occ; i += blockDim.x) {
    const unsigned long long k = keys[i];
    // the run holding position i: the bin whose [start, fill) contains it
    const int bin = it.mode_bin[int(k & 0xFFFFFu)];
    const int st = fill[bin] - cnt[bin], en = fill[bin];
    int rank = 0;
    for (int j = st; j < en; ++j) rank += keys[j] < k ? 1 : 0;
    it.bkt_list[st + rank] = int32_t(k & 0xFFFFFu);
  }
}

// One warp per bin. cond: only signals whose iteration is redone in FP64
// (more near-tie bins than their list holds) take part.
template <typename T, int TMAX>
__global__ void __launch_bounds__(256, (sizeof(T) == 4 && TMAX == 1) ? 6 : 1)
    k_decide(const SigIter *__restrict__ its, int mode, int cond, int mark) {
  PdlEnter(its, kTraceDecide);
  const SigIter &it = its[blockIdx.y];
  if (!it.active) return;
  if (cond ? !RedoFP64(it) : it.force_fp64) return;
  const int beta = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (beta >= it.bins) return;
  int e;
  if constexpr (sizeof(T) == sizeof(float)) {
    e = DecideBin<T, TMAX>(it, beta, FromBins32{it, beta}, mode);
  } else {
    e = DecideBin<T, TMAX>(it, beta, FromBins{it, beta}, mode);
  }
  // a listed near tie: with mark, the bin's candidate is held back from the
  // merge (cand_valid + kCandListed) until its FP64 decision; its
  // re-binning's arrival counters cleared and (solves and iterations) its
  // phase-step powers evaluated, once for all the re-binning's work items
  if (e >= 0) {
    if (mark && (threadIdx.x & 31) == 0) it.cand_valid[beta] += kCandListed;
    if (it.esc_pow != nullptr) {
      PrepListedBin(it, e, beta, threadIdx.x & 31);
    } else {
      ClearListedBin(it, e, threadIdx.x & 31);
    }
  }
}

// The listed near-tie bins of the FP32 pass, decided in FP64 on their
// re-binned rows. kListedBlocks blocks per signal take every
// kListedBlocks-th listed bin (k_listed_terms) or group of 8 listed bins
// (k_decide_listed).
constexpr int kListedBlocks = 8;

__device__ void MergeBin(const SigIter &it, int beta);

// FP64 mode subtraction of the listed bins, beside their re-binning: one
// block of W warps per listed bin. The bin's found modes get their FP64
// row-0 terms (ModeTerms64: two FP64 erf each, long on this part; a thread
// per mode), then their sum over the bin in every row: row 0 takes the terms
// themselves, the rows 2s+1, 2s+2 of bit s the terms times the row factor
// e^{+-2 pi i (B 2^s k1 mod n)/n} (src/binner.cc:584-589), lane s of every
// warp. Warp w takes the groups of G consecutive modes w, w + W, ..., loads
// their terms and row-factor table entries together and keeps per-lane
// partial sums (a long chain of FP64 operations per mode; GB300 has few FP64
// pipes, with long latencies); the partials meet in shared memory in warp
// order, into esc_msub. Signals whose list overflowed are redone whole or
// marked unresolved (k_decide_listed).
template <int TMAX, int W, int G>
__global__ void __launch_bounds__(32 * W) k_listed_terms(const SigIter *__restrict__ its) {
  PdlEnter(its, kTraceListedTerms);
  __shared__ double2 s_p0[W][TMAX];
  __shared__ double2 s_pp[W][32][TMAX];
  __shared__ double2 s_pm[W][32][TMAX];
  const SigIter &it = its[blockIdx.y];
  if (!it.active || it.force_fp64 || it.esc_mask == nullptr) return;
  const int nf = *(volatile int32_t *)&it.flags[2];
  if (nf > it.esc_cap) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int TR = it.trials;
  const bool has_bit = lane < it.bits;
  const int64_t off = has_bit ? (int64_t(it.bins) << lane) : 0;
  const ModN mod{uint32_t(it.n), it.n_inv};
  const uint32_t lo_mask = (1u << it.ph_k) - 1u;
  for (int e = blockIdx.x; e < nf; e += kListedBlocks) {
    const int beta = it.esc_list[e];
    const int nm = it.bkt_count[beta], st = it.bkt_start[beta];
    for (int i = threadIdx.x; i < nm; i += blockDim.x) {
      const int sl = it.bkt_list[st + i];
      ModeTerms64(it, sl, it.mode_k1[sl], it.mode_bin[sl]);
    }
    __syncthreads();  // the block's terms are visible to the whole block
    double2 p0[TMAX], pp[TMAX], pm[TMAX];
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      p0[t] = pp[t] = pm[t] = make_double2(0.0, 0.0);
    }
    for (int i0 = warp * G; i0 < nm; i0 += G * W) {
      // G modes: slots (past the end: the group's first, not accumulated),
      // then their terms, k1 and row-factor table entries, all loads issued
      // before any is used
      int sl[G];
#pragma unroll
      for (int u = 0; u < G; ++u) sl[u] = it.bkt_list[st + min(i0 + u, nm - 1)];
      int64_t k1[G];
      double2 bs[G][TMAX];
#pragma unroll
      for (int u = 0; u < G; ++u) {
        k1[u] = it.mode_k1[sl[u]];
#pragma unroll
        for (int t = 0; t < TMAX; ++t) {
          if (t < TR) bs[u][t] = it.mode_base[size_t(sl[u]) * TR + t];
        }
      }
      double2 h[G], l[G];
#pragma unroll
      for (int u = 0; u < G; ++u) {
        const uint32_t r = mod(off * k1[u]);
        h[u] = it.ph_hi[r >> it.ph_k];
        l[u] = it.ph_lo[r & lo_mask];
      }
#pragma unroll
      for (int u = 0; u < G; ++u) {
        if (i0 + u < nm) {
          const double2 fac = cmul(h[u], l[u]);
#pragma unroll
          for (int t = 0; t < TMAX; ++t) {
            if (t < TR) {
              p0[t] = cadd(p0[t], bs[u][t]);
              pp[t] = cadd(pp[t], cmul(bs[u][t], fac));
              pm[t] = cadd(pm[t], cmul(bs[u][t], cconj(fac)));
            }
          }
        }
      }
    }
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        if (lane == 0) s_p0[warp][t] = p0[t];
        s_pp[warp][lane][t] = pp[t];
        s_pm[warp][lane][t] = pm[t];
      }
    }
    __syncthreads();
    if (warp == 0) {
      double2 *out = it.esc_msub + size_t(e) * TR * it.rows;
#pragma unroll
      for (int t = 0; t < TMAX; ++t) {
        if (t < TR) {
          if (lane == 0) {
            double2 sum = s_p0[0][t];
#pragma unroll
            for (int w = 1; w < W; ++w) sum = cadd(sum, s_p0[w][t]);
            out[size_t(t) * it.rows] = sum;
          }
          if (has_bit) {
            double2 sp = s_pp[0][lane][t], sm = s_pm[0][lane][t];
#pragma unroll
            for (int w = 1; w < W; ++w) {
              sp = cadd(sp, s_pp[w][lane][t]);
              sm = cadd(sm, s_pm[w][lane][t]);
            }
            out[size_t(t) * it.rows + 2 * lane + 1] = sp;
            out[size_t(t) * it.rows + 2 * lane + 2] = sm;
          }
        }
      }
    }
    __syncthreads();  // the partials are rewritten for the next listed bin
  }
}

// FP64 decisions of the listed near-tie bins: one warp per listed bin (lane s
// holds bit s), on the re-binned rows (FromRebin) minus the bin's found modes
// (esc_msub): energy threshold, then DecideTail, and the bin's candidate into
// the table. Signals whose list overflowed are redone whole instead (redo),
// or marked unresolved, their held-back bins keeping their FP32 candidates.
template <int TMAX>
__global__ void __launch_bounds__(256)
    k_decide_listed(const SigIter *__restrict__ its, int redo, int merge) {
  PdlEnter(its, kTraceDecideListed);
  const SigIter &it = its[blockIdx.y];
  if (!it.active) return;
  if (it.force_fp64) return;
  const int nf = *(volatile int32_t *)&it.flags[2];
  if (nf > it.esc_cap) {
    if (!redo && blockIdx.x == 0 && threadIdx.x == 0) {
      atomicOr(&it.flags[1], kStatusUnresolved);
    }
    if (merge && threadIdx.x == 0) {
      for (int e = blockIdx.x; e < it.esc_cap; e += kListedBlocks) {
        const int beta = it.esc_list[e];
        it.cand_valid[beta] -= kCandListed;
        MergeBin(it, beta);
      }
    }
    return;
  }
  const int lane = threadIdx.x & 31;
  const int TR = it.trials;
  const bool has_bit = lane < it.bits;
  for (int e = blockIdx.x * 8 + (threadIdx.x >> 5); e < nf; e += kListedBlocks * 8) {
    const int beta = it.esc_list[e];
    const FromRebin src{it, e, beta, it.esc_mask[e]};
    const double2 *ms = it.esc_msub + size_t(e) * TR * it.rows;
    double2 u0[TMAX], up[TMAX], um[TMAX];
    double en = 0.0;
#pragma unroll
    for (int t = 0; t < TMAX; ++t) {
      if (t < TR) {
        u0[t] = csub(src.get(t, 0), __ldcg(&ms[size_t(t) * it.rows]));
        en += u0[t].x * u0[t].x + u0[t].y * u0[t].y;
        if (has_bit) {
          up[t] = csub(src.get(t, 2 * lane + 1),
                       __ldcg(&ms[size_t(t) * it.rows + 2 * lane + 1]));
          um[t] = csub(src.get(t, 2 * lane + 2),
                       __ldcg(&ms[size_t(t) * it.rows + 2 * lane + 2]));
        } else {
          up[t] = um[t] = make_double2(0.0, 0.0);
        }
      }
    }
    en /= double(TR);
    // energy threshold on row 0 (src/iterate.cc:114-124)
    bool go = true;
    if (!isfinite(en)) {
      if (lane == 0) {
        atomicOr(&it.flags[1], kStatusNonFinite);
        it.cand_valid[beta] = 0;
      }
      go = false;
    } else if (it.bin_thr > 0 && en < it.bin_thr * it.bin_thr) {
      NoCandidate(it, beta, lane);
      go = false;
    }
    if (go) {
      DecideTail<double, TMAX>(it, beta, kDecideExact, u0, up, um, 0.f, 0.f, false,
                               -1);
    }
    // the bin's candidate (written by lane 0 above) into the table
    if (merge && lane == 0) MergeBin(it, beta);
  }
}

// ---------------------------------------------------------------- merge
// Candidate of bin beta -> table. A pending FP32 candidate is finished here
// in FP64 (src/iterate.cc:139-171): the window response at
// xi0 = k1/n - (beta + 1/2)/B and its threshold, the average over the
// T (1 + 2L) values, k0 = a^-1 (k1 - b) mod n, the factor e^{-2 pi i c k0/n}
// and the division by the window response.
__device__ void MergeBin(const SigIter &it, int beta) {
  const int v = it.cand_valid[beta];
  if (!v) return;
  int32_t k0 = it.cand_k0[beta];
  double2 coef = it.cand_coef[beta];
  double err = it.cand_err[beta];
  const ModN mod{uint32_t(it.n), it.n_inv};
  // k1 of the candidate (pending: cand_k0 holds it), and whether it lies in
  // this bin's range
  const int64_t k1 = v == 2 ? int64_t(k0) : int64_t(mod(int64_t(it.a) * k0 + it.b));
  const bool own = int64_t(mod.quot(k1 * int64_t(it.bins))) == beta;
  if (v == 2) {
    const int64_t n = it.n;
    const int B = it.bins;
    // xi0 = k1/n - (beta + 1/2)/B from its exact integer numerator
    // (|num| < 2^53) and 1/(2nB); one FP64 division per candidate (each is a
    // long sequence on this part's FP64 pipes)
    const int64_t num = 2 * int64_t(B) * k1 - (2 * int64_t(beta) + 1) * n;
    const double wf = WindowInFreq(it, double(num) * it.xi_scale);
    if (fabs(wf) < it.win_thr) {
      it.cand_valid[beta] = 0;
      return;
    }
    const double m = double(it.trials * (1 + 2 * it.bits));
    const double scale = 1.0 / (m * wf);  // the average and the window
    k0 = int32_t(mod(int64_t(it.a_inv) * mod(k1 - it.b)));
    coef = cmul(coef, Phase64(it, -int64_t(it.c) * k0));
    coef = make_double2(coef.x * scale, coef.y * scale);
    err = err * fabs(m * scale);
    it.cand_k0[beta] = k0;
    it.cand_coef[beta] = coef;
    it.cand_err[beta] = err;
    it.cand_valid[beta] = 1;
  }
  it.flags[0] = 1;
  if (!own) {
    const int j = atomicAdd(&it.flags[4], 1);
    if (j < kSpillCap) {
      it.spill_beta[j] = beta;
      it.spill_k0[j] = k0;
      it.spill_coef[j] = coef;
      it.spill_err[j] = err;
      return;
    }
    // (a full spill list: added at once, the order of these few additions
    // then follows the blocks)
  }
  InsertMode(it, k0, coef, err);
}

// The spilled candidates of every signal (InsertSpills), after the merges of
// an iteration that no stop-rule kernel follows.
__global__ void k_insert_spills(const SigIter *__restrict__ its, int nsig) {
  PdlEnter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsig) return;
  const SigIter &it = its[i];
  if (it.active && it.flags[4] > 0) InsertSpills(it);
}

// Candidates -> table, one thread per bin; bins held back for their FP64
// near-tie decision (cand_valid >= kCandListed) are merged by that decision.
__global__ void k_merge(const SigIter *__restrict__ its) {
  PdlEnter(its, kTraceMerge);
  const SigIter &it = its[blockIdx.y];
  if (!it.active) return;
  const int beta = blockIdx.x * blockDim.x + threadIdx.x;
  if (beta >= it.bins) return;
  if (it.cand_valid[beta] >= kCandListed) return;
  MergeBin(it, beta);
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

// The occupied entries of every table into one packed staging area, signal
// s at [o_s, o_s + count_s) with o_s the sum of the counts before it (each
// block adds them up itself), sorted by k0 (one block per signal, bitonic
// sort of (k0, slot) in shared memory: ranking every key by counting the
// smaller ones, O(count^2), took 16x longer at the tables of 64 config-2
// solves); a table with more entries than the sort holds (only after a
// capacity status) is written in insertion order and sorted[s] = 0.
__global__ void __launch_bounds__(1024)
    k_export_tables(const SigIter *__restrict__ its, int nsig, int32_t *keys,
                    double2 *coefs, int32_t *counts, int32_t *sorted) {
  extern __shared__ unsigned long long sk[];
  __shared__ long long s_base;
  const SigIter &it = its[blockIdx.x];
  const int cnt = *it.tab_count;
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  {
    long long part = 0;
    for (int j = threadIdx.x; j < int(blockIdx.x); j += blockDim.x) {
      part += *its[j].tab_count;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0 && part != 0) {
      atomicAdd(reinterpret_cast<unsigned long long *>(&s_base),
                static_cast<unsigned long long>(part));
    }
  }
  __syncthreads();
  const size_t base = size_t(s_base);
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
                   int cond, int mark, cudaStream_t s) {
  dim3 grid((max_bins + 7) / 8, nsig);
  Launch(k_decide<T, TMAX>, grid, 256, 0, s, d_its, mode, cond, mark);
}

template <typename T>
void LaunchDecideP(const SigIter *d_its, int nsig, int max_bins, int max_trials,
                   int mode, int cond, int mark, cudaStream_t s) {
  if (max_trials <= 1) {
    LaunchDecideT<T, 1>(d_its, nsig, max_bins, mode, cond, mark, s);
  } else if (max_trials <= 5) {
    LaunchDecideT<T, 5>(d_its, nsig, max_bins, mode, cond, mark, s);
  } else {
    LaunchDecideT<T, kMaxTrials>(d_its, nsig, max_bins, mode, cond, mark, s);
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
  k_export_tables<<<nsig, 1024, sm, s>>>(d_its, nsig, keys, coefs, counts, sorted);
}

void LaunchModePrep(const SigIter *d_its, int nsig, int max_cap, cudaStream_t s,
                    bool cond) {
  // the occupied count is only known on the device: up to 8 blocks per
  // signal stride over it (a table holds at most max_cap / 2 entries)
  dim3 grid(std::min(8, std::max(1, max_cap / 2 / 256)), nsig);
  Launch(k_mode_prep, grid, 256, 0, s, d_its, cond ? 1 : 0);
}

// Shared memory of k_bucket: the keys, then two ints per bin.
inline size_t BucketSmem(int max_cap, int max_bins) {
  return size_t(BucketKeys(max_cap)) * sizeof(unsigned long long) +
         2 * sizeof(int) * size_t(max_bins);
}

void LaunchBucket(const SigIter *d_its, int nsig, int max_bins, int max_cap,
                  cudaStream_t s, bool prep) {
  const size_t sm = BucketSmem(max_cap, max_bins);
  cudaFuncSetAttribute(k_bucket, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(sm));
  Launch(k_bucket, nsig, 1024, sm, s, d_its, max_bins, prep ? 1 : 0);
}

void LaunchDecide(const SigIter *d_its, int nsig, int max_bins, int max_trials,
                  bool fp32, bool subtract_only, cudaStream_t s, bool cond,
                  bool mark_listed) {
  const int mode = subtract_only ? kSubtractOnly : kDecide;
  if (fp32) {
    LaunchDecideP<float>(d_its, nsig, max_bins, max_trials, mode, 0,
                         mark_listed ? 1 : 0, s);
  } else {
    LaunchDecideP<double>(d_its, nsig, max_bins, max_trials, mode, cond ? 1 : 0,
                          0, s);
  }
}

void LaunchDecideListed(const SigIter *d_its, int nsig, int max_trials,
                        bool redo, bool merge, cudaStream_t s) {
  dim3 grid(kListedBlocks, nsig);
  const int r = redo ? 1 : 0, mg = merge ? 1 : 0;
  if (max_trials <= 1) {
    Launch(k_decide_listed<1>, grid, 256, 0, s, d_its, r, mg);
  } else if (max_trials <= 5) {
    Launch(k_decide_listed<5>, grid, 256, 0, s, d_its, r, mg);
  } else {
    Launch(k_decide_listed<kMaxTrials>, grid, 256, 0, s, d_its, r, mg);
  }
}

void LaunchListedTerms(const SigIter *d_its, int nsig, int max_trials, cudaStream_t s) {
  dim3 grid(kListedBlocks, nsig);
  if (max_trials <= 1) {
    Launch(k_listed_terms<1, 8, 4>, grid, 32 * 8, 0, s, d_its);
  } else if (max_trials <= 5) {
    Launch(k_listed_terms<5, 4, 2>, grid, 32 * 4, 0, s, d_its);
  } else {
    Launch(k_listed_terms<kMaxTrials, 2, 1>, grid, 32 * 2, 0, s, d_its);
  }
}

void LaunchMerge(const SigIter *d_its, int nsig, int max_bins,
                 cudaStream_t s) {
  dim3 grid((max_bins + 255) / 256, nsig);
  Launch(k_merge, grid, 256, 0, s, d_its);
}

void LaunchInsertSpills(const SigIter *d_its, int nsig, cudaStream_t s) {
  Launch(k_insert_spills, (nsig + 127) / 128, 128, 0, s, d_its, nsig);
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
  int a = 0, b = 0, c = 0;
  const size_t smb = size_t(BucketKeys(kMaxTableCap)) * sizeof(unsigned long long);
  const size_t smk = BucketSmem(kMaxTableCap, kMaxFFT / 2);
  cudaFuncSetAttribute(k_bucket, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(smk));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_bucket, 1024, smk);
  int e = 0;
  cudaFuncSetAttribute(k_export_tables, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(smb));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e, k_export_tables, 1024, smb);
  a = a < e ? a : e;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_decide<double, kMaxTrials>, 256, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_decide<float, kMaxTrials>, 256, 0);
  int l = 0, l1 = 0, l5 = 0, d = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&l, k_listed_terms<kMaxTrials, 2, 1>, 64, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&l1, k_listed_terms<1, 8, 4>, 256, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&l5, k_listed_terms<5, 4, 2>, 128, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d, k_decide_listed<kMaxTrials>, 256, 0);
  l = (l1 > 0 && l5 > 0 && d > 0) ? l : 0;
  return a > 0 && b > 0 && c > 0 && l > 0;
}

}  // namespace mpsft
