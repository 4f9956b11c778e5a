// Size-B forward DFT of every folded row (FFTPlan::Run of size B,
// src/base.cc:86-97, called at src/binner.cc:428 and 509-510), by Bluestein's
// chirp-z method over the shared-memory radix-2 FFT (any odd B, including
// large primes), followed by the row factor e^{2 pi i (b q mod n)/n} that the
// fold left out. Output: complex128 bins in ubuf.
//
// One CTA per (row, trial, signal). FP32 path: the convolution runs in FP32
// (M <= 16384 points, 128 KB of shared memory); FP64 path: in FP64
// (M <= 8192). In solves and iterations the FP32 path writes complex64 bins
// (ubuf32) and keeps the FP64 pipes out of the epilogue (GB300 issues FP64
// at a small fraction of its FP32 rate, with long latencies): the row factor
// is applied as a float-float value, and each product is formed with exact
// FMA products and a two-sum, then rounded once to FP32.
#include <algorithm>

#include "fft.cuh"
#include "launch.h"

namespace mpsft {

namespace {

__device__ inline const float2 *ChirpOf(const SigIter &it, float2 *) { return it.chirp32; }
__device__ inline const double2 *ChirpOf(const SigIter &it, double2 *) { return it.chirp64; }
__device__ inline const float2 *ChatOf(const SigIter &it, float2 *) { return it.chat32; }
__device__ inline const double2 *ChatOf(const SigIter &it, double2 *) { return it.chat64; }

// y * (bh + bl) rounded to FP32 (bh + bl: a unit phase as float-float):
// the high products exactly (FMA residuals), a two-sum of the pair, then the
// residuals and the low-word products, one final rounding.
__device__ __forceinline__ float DotRound(float x0, float y0, float x1, float y1,
                                          float l0, float l1) {
  // x0 y0 + x1 y1 + (x0 l0 + x1 l1)
  const float p0 = __fmul_rn(x0, y0), e0 = fmaf(x0, y0, -p0);
  const float p1 = __fmul_rn(x1, y1), e1 = fmaf(x1, y1, -p1);
  const float s = __fadd_rn(p0, p1);
  const float bb = __fsub_rn(s, p0);
  const float es = __fadd_rn(__fsub_rn(p0, __fsub_rn(s, bb)), __fsub_rn(p1, bb));
  const float lo = __fadd_rn(__fadd_rn(es, __fadd_rn(e0, e1)),
                             fmaf(x0, l0, __fmul_rn(x1, l1)));
  return __fadd_rn(s, lo);
}
__device__ __forceinline__ float2 MulPhaseFF(float2 y, float2 bh, float2 bl) {
  return make_float2(DotRound(y.x, bh.x, -y.y, bh.y, bl.x, bl.y),
                     DotRound(y.x, bh.y, y.y, bh.x, bl.y, bl.x));
}

// cond: only signals whose iteration is redone in FP64 take part. Also
// records the largest |U| of each row (used by the FP32 near-tie bound).
//
// Rows per block: small transforms share a block, RowsPerBlock(M) rows side by
// side (M/8 threads each for the radix-8 passes), so that late iterations
// with few bins do not launch a block per tiny row.
constexpr int kRowFftThreads = 512;
constexpr int kRowsMax = 64;
__device__ __forceinline__ int RowsPerBlock(int M) {
  const int r = kRowFftThreads * 8 / M;
  return r < 1 ? 1 : (r > kRowsMax ? kRowsMax : r);
}

template <typename V>
__global__ void __launch_bounds__(kRowFftThreads)
    k_row_fft(const SigIter *__restrict__ its, int max_trials,
              const V *__restrict__ tw, int cond, int rpb_cap) {
  PdlEnter(its, kTraceRowFft);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned row_max_bits[kRowsMax];
  const SigIter &it = its[blockIdx.z];
  if (!it.active) return;
  if (cond ? !RedoFP64(it) : it.force_fp64) return;
  const int tr = blockIdx.y;
  const int B = it.bins, M = it.fft_m;
  const int rpb = min(RowsPerBlock(M), rpb_cap);
  const int row0 = blockIdx.x * rpb;
  if (row0 >= it.rows || tr >= it.trials) return;
  const int nth = kRowFftThreads / rpb;  // threads per row
  const int lr = threadIdx.x / nth, tid = threadIdx.x % nth;
  const int row = row0 + lr;
  const bool live = lr < rpb && row < it.rows;
  V *a = reinterpret_cast<V *>(smem_raw) + size_t(lr) * PadLen(M);
  const V *__restrict__ chirp = ChirpOf(it, (V *)nullptr);
  const V *__restrict__ chat = ChatOf(it, (V *)nullptr);
  if (threadIdx.x < kRowsMax) row_max_bits[threadIdx.x] = 0u;
  // the trial's row factor as float-float for the complex64 epilogue (read
  // after the transforms' barriers)
  __shared__ float2 bq_ff[2];
  const bool out32 = sizeof(V) == sizeof(float2) && it.ubuf32 != nullptr;
  if (out32 && threadIdx.x == 0) {
    const double br = it.bq_re[tr], bi = it.bq_im[tr];
    const float hr = __double2float_rn(br), hi = __double2float_rn(bi);
    bq_ff[0] = make_float2(hr, hi);
    bq_ff[1] = make_float2(__double2float_rn(br - double(hr)),
                           __double2float_rn(bi - double(hi)));
  }
  // element loops: up to 8 elements per thread with their loads issued
  // together (a thread covers M / nth elements)
  if (live) {
    const V *__restrict__ src = reinterpret_cast<const V *>(it.fold) +
                                (size_t(tr) * it.rows + row) * it.bins_cap;
    for (int j0 = tid; j0 < M; j0 += 8 * nth) {
      V v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = j0 + u * nth;
        if (j < M) {
          v[u] = j < B ? vmul(src[j], __ldg(&chirp[j]))
                       : vmake2(0.0, 0.0, (V *)nullptr);
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = j0 + u * nth;
        if (j < M) a[Pad(j)] = v[u];
      }
    }
  }
  __syncthreads();
  // forward DIF (bit-reversed out), product with chat (stored bit-reversed),
  // inverse DIT (natural out); rows past the last run the barriers only
  BlockFFTDif(a, live ? M : 0, it.fft_log2m, tw, false, tid, nth);
  if (live) {
    for (int j0 = tid; j0 < M; j0 += 8 * nth) {
      V w[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = j0 + u * nth;
        if (j < M) w[u] = __ldg(&chat[j]);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = j0 + u * nth;
        if (j < M) a[Pad(j)] = vmul(a[Pad(j)], w[u]);
      }
    }
  }
  __syncthreads();
  BlockFFTDit(a, live ? M : 0, it.fft_log2m, tw, true, tid, nth);
  float ss = 0.f;  // this thread's share of the row's sum of |U|^2
  float mx = 0.f;  // and of its largest |U|
  if (live && out32) {
    // FP32 bins: exact power-of-two scale, float-float row factor
    const float inv_mf = 1.0f / float(M);
    const float2 bh = bq_ff[0], bl = bq_ff[1];
    float2 *dst = it.ubuf32 + (size_t(tr) * it.rows + row) * it.bins_cap;
    for (int k0 = tid; k0 < B; k0 += 8 * nth) {
      V w[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = k0 + u * nth;
        if (k < B) w[u] = __ldg(&chirp[k]);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = k0 + u * nth;
        if (k < B) {
          const V z = vmul(a[Pad(k)], w[u]);
          const float2 y = make_float2(float(z.x) * inv_mf, float(z.y) * inv_mf);
          dst[k] = MulPhaseFF(y, bh, bl);
          const float y2 = y.x * y.x + y.y * y.y;
          ss += y2;
          mx = fmaxf(mx, sqrtf(y2));
        }
      }
    }
  } else if (live) {
    const double inv_m = 1.0 / double(M);
    const double2 bq = make_double2(it.bq_re[tr], it.bq_im[tr]);
    double2 *dst = it.ubuf + (size_t(tr) * it.rows + row) * it.bins_cap;
    for (int k0 = tid; k0 < B; k0 += 8 * nth) {
      V w[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = k0 + u * nth;
        if (k < B) w[u] = __ldg(&chirp[k]);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = k0 + u * nth;
        if (k < B) {
          const double2 y = cscale(to_d2(vmul(a[Pad(k)], w[u])), inv_m);
          dst[k] = cmul(bq, y);
          const double y2 = y.x * y.x + y.y * y.y;
          ss += float(y2);
          mx = fmaxf(mx, float(sqrt(y2)));
        }
      }
    }
  }
  // the row's sum of |U|^2 in a fixed order: a shuffle tree over segments of
  // min(nth, 32) threads (a row's threads are consecutive, nth a power of
  // two), then the row's segments in order
  __shared__ float seg_ss[kRowFftThreads / 8];
  const int seg = nth < 32 ? nth : 32;
  for (int o = seg >> 1; o > 0; o >>= 1) {
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & (seg - 1)) == 0) {
    seg_ss[threadIdx.x / seg] = ss;
    // non-negative floats order like their bit patterns
    if (live) atomicMax(&row_max_bits[lr], __float_as_uint(mx));
  }
  __syncthreads();  // (rows past the last only reach the barriers)
  if (live && tid == 0 && it.row_max != nullptr) {
    it.row_max[tr * it.rows + row] = __uint_as_float(row_max_bits[lr]);
    const int nseg = nth / seg;
    float t = 0.f;
    for (int j = 0; j < nseg; ++j) t += seg_ss[lr * nseg + j];
    it.row_ms[tr * it.rows + row] = t / float(B);
  }
}

// Small bins (Bluestein size M <= kDirectMaxM, bins <= 63): the DFT as a
// direct sum X[k] = sum_j F[j] e^{-2 pi i j k / B}, two warps per row and one
// output per lane, with the unit roots of the bins grid in shared memory;
// then the same epilogue as the Bluestein kernel. Each sum runs as four
// interleaved FMA chains over j = u mod 4 (each with its own root index
// j k mod B), added pairwise at the end: a short dependency chain per term,
// and an FP32 error below that of the Bluestein transform it replaces (two
// 128-point transforms at B = 51).
constexpr int kDirectMaxM = 128;
constexpr int kDirectMaxBins = kDirectMaxM / 2;
constexpr int kDirectRowsPerBlock = 4;  // two warps per row

__global__ void __launch_bounds__(64 * kDirectRowsPerBlock)
    k_row_dft_small(const SigIter *__restrict__ its, int cond) {
  PdlEnter(its, kTraceRowFft);
  __shared__ float2 roots[kDirectMaxBins];
  __shared__ float2 rows[kDirectRowsPerBlock][kDirectMaxBins];
  __shared__ float wmax[2 * kDirectRowsPerBlock];
  __shared__ float wss[2 * kDirectRowsPerBlock];
  const SigIter &it = its[blockIdx.z];
  if (!it.active) return;
  if (cond ? !RedoFP64(it) : it.force_fp64) return;
  const int tr = blockIdx.y;
  const int B = it.bins;
  if (tr >= it.trials) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lr = warp >> 1;
  const int row = blockIdx.x * kDirectRowsPerBlock + lr;
  const bool live = row < it.rows;
  for (int r = threadIdx.x; r < B; r += blockDim.x) {
    float sn, cs;
    sincospif(-2.0f * float(r) / float(B), &sn, &cs);
    roots[r] = make_float2(cs, sn);
  }
  if (live) {
    const float2 *__restrict__ src = reinterpret_cast<const float2 *>(it.fold) +
                                     (size_t(tr) * it.rows + row) * it.bins_cap;
    for (int j = (warp & 1) * 32 + lane; j < B; j += 64) rows[lr][j] = src[j];
  }
  __syncthreads();
  const int k = (warp & 1) * 32 + lane;
  float mx = 0.f, ss = 0.f;
  if (live && k < B) {
    const float2 *f = rows[lr];
    float xr[4] = {0.f, 0.f, 0.f, 0.f}, xi[4] = {0.f, 0.f, 0.f, 0.f};
    int id[4];
    id[0] = 0;
    id[1] = k;
    id[2] = (2 * k) % B;
    id[3] = (3 * k) % B;
    const int step = (4 * k) % B;
    int j = 0;
    for (; j + 4 <= B; j += 4) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float2 v = f[j + u], w = roots[id[u]];
        xr[u] = fmaf(v.x, w.x, xr[u]);
        xr[u] = fmaf(-v.y, w.y, xr[u]);
        xi[u] = fmaf(v.x, w.y, xi[u]);
        xi[u] = fmaf(v.y, w.x, xi[u]);
        id[u] += step;
        if (id[u] >= B) id[u] -= B;
      }
    }
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      if (j + u < B) {
        const float2 v = f[j + u], w = roots[id[u]];
        xr[u] = fmaf(v.x, w.x, xr[u]);
        xr[u] = fmaf(-v.y, w.y, xr[u]);
        xi[u] = fmaf(v.x, w.y, xi[u]);
        xi[u] = fmaf(v.y, w.x, xi[u]);
      }
    }
    const float2 y = make_float2((xr[0] + xr[1]) + (xr[2] + xr[3]),
                                 (xi[0] + xi[1]) + (xi[2] + xi[3]));
    const size_t o = (size_t(tr) * it.rows + row) * it.bins_cap + k;
    if (it.ubuf32 != nullptr) {
      const double br = it.bq_re[tr], bi = it.bq_im[tr];
      const float2 bh = make_float2(__double2float_rn(br), __double2float_rn(bi));
      const float2 bl = make_float2(__double2float_rn(br - double(bh.x)),
                                    __double2float_rn(bi - double(bh.y)));
      it.ubuf32[o] = MulPhaseFF(y, bh, bl);
    } else {
      const double2 bq = make_double2(it.bq_re[tr], it.bq_im[tr]);
      it.ubuf[o] = cmul(bq, make_double2(y.x, y.y));
    }
    ss = y.x * y.x + y.y * y.y;
    mx = sqrtf(ss);
  }
  // the row's largest magnitude and mean |U|^2: each warp's (a fixed shuffle
  // tree), then the row's pair of warps
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
  }
  if (lane == 0) {
    wmax[warp] = mx;
    wss[warp] = ss;
  }
  __syncthreads();
  if (live && (warp & 1) == 0 && lane == 0 && it.row_max != nullptr) {
    it.row_max[tr * it.rows + row] = fmaxf(wmax[warp], wmax[warp + 1]);
    it.row_ms[tr * it.rows + row] = (wss[warp] + wss[warp + 1]) / float(B);
  }
}

}  // namespace

// Shared memory of a block: one padded row of the largest transform, or the
// rows of smaller ones side by side (at most 4096 + 256 + 64 slots).
inline size_t RowFftSlots(int max_m) {
  const size_t one = size_t(PadLen(max_m));
  const size_t packed = size_t(kRowFftThreads) * 8 + kRowFftThreads / 2 + kRowsMax;
  return one > packed ? one : packed;
}

void LaunchRowFFT(const SigIter *d_its, int nsig, int max_rows,
                  int max_trials, int max_m, bool fp64, const float2 *tw32,
                  const double2 *tw64, cudaStream_t s, bool cond) {
  // rows per block: as many as the transform size allows, but no fewer
  // blocks than about two per SM (so that a single signal, or the FP64
  // pipes, still spread over the GPU); every transform of the launch has at
  // most max_m points, so at least rpb rows per block
  if (!fp64 && max_m <= kDirectMaxM) {
    dim3 g((max_rows + kDirectRowsPerBlock - 1) / kDirectRowsPerBlock, max_trials,
           nsig);
    Launch(k_row_dft_small, g, 64 * kDirectRowsPerBlock, 0, s, d_its, cond ? 1 : 0);
    return;
  }
  // (a power of two, so that a row's threads are whole shuffle segments)
  int rpb_cap = 1;
  while (int64_t(rpb_cap) * 2 <= int64_t(max_rows) * max_trials * nsig / (2 * 152)) {
    rpb_cap *= 2;
  }
  const int rpb = std::max(
      1, std::min({kRowsMax, kRowFftThreads * 8 / std::max(1, max_m), rpb_cap}));
  dim3 grid((max_rows + rpb - 1) / rpb, max_trials, nsig);
  if (fp64) {
    const size_t sm = RowFftSlots(max_m) * sizeof(double2);
    cudaFuncSetAttribute(k_row_fft<double2>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    Launch(k_row_fft<double2>, grid, kRowFftThreads, sm, s, d_its, max_trials, tw64,
                                                        cond ? 1 : 0, rpb_cap);
  } else {
    const size_t sm = RowFftSlots(max_m) * sizeof(float2);
    cudaFuncSetAttribute(k_row_fft<float2>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    Launch(k_row_fft<float2>, grid, kRowFftThreads, sm, s, d_its, max_trials, tw32,
                                                       cond ? 1 : 0, rpb_cap);
  }
}

bool FftKernelsLaunchable() {
  int n1 = 0, n2 = 0;
  const size_t sm32 = RowFftSlots(kMaxFFT) * sizeof(float2);
  const size_t sm64 = RowFftSlots(kMaxFFT64) * sizeof(double2);
  cudaFuncSetAttribute(k_row_fft<float2>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm32));
  cudaFuncSetAttribute(k_row_fft<double2>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm64));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_row_fft<float2>, 512, sm32);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n2, k_row_fft<double2>, 512, sm64);
  return n1 > 0 && n2 > 0;
}

}  // namespace mpsft
