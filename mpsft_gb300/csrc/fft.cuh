// Shared-memory FFTs used by the Bluestein size-B transform.
#pragma once

#include "common.cuh"

namespace mpsft {

template <typename V> struct Real;
template <> struct Real<float2> { using T = float; };
template <> struct Real<double2> { using T = double; };

__device__ inline float2 vadd(float2 a, float2 b) {
  return make_float2(a.x + b.x, a.y + b.y);
}
__device__ inline float2 vsub(float2 a, float2 b) {
  return make_float2(a.x - b.x, a.y - b.y);
}
__device__ inline double2 vadd(double2 a, double2 b) { return cadd(a, b); }
__device__ inline double2 vsub(double2 a, double2 b) { return csub(a, b); }
__device__ inline float2 vmul(float2 a, float2 b) { return cmulf(a, b); }
__device__ inline double2 vmul(double2 a, double2 b) { return cmul(a, b); }
__device__ inline float2 vconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ inline double2 vconj(double2 a) { return cconj(a); }
__device__ inline float2 vmake(double re, double im) {
  return make_float2(float(re), float(im));
}
__device__ inline double2 vmake2(double re, double im, double2 *) {
  return make_double2(re, im);
}
__device__ inline float2 vmake2(double re, double im, float2 *) {
  return make_float2(float(re), float(im));
}
__device__ inline double2 to_d2(float2 a) { return make_double2(a.x, a.y); }
__device__ inline double2 to_d2(double2 a) { return a; }

// Shared-memory layout of the transforms: element i at Pad(i), one empty
// slot after every 16 elements. Half a warp's 8-byte accesses then fall on
// 16 distinct bank pairs in every pass (runs of 16 consecutive elements for
// spans h >= 16; for smaller spans the groups' strided elements shift by one
// slot per 16), and on 8 distinct pairs with 16-byte elements. An array of m
// elements occupies PadLen(m) slots.
__device__ __forceinline__ int Pad(int i) { return i + (i >> 4); }
__host__ __device__ inline int PadLen(int m) { return m + (m >> 4) + 1; }

// W_N^e = e^{-2 pi i e / N}, N = 2^log2n, e < N / 2 (conjugated for the
// inverse), from the size-N block of the twiddle table (TwiddleAt): the
// consecutive e of a warp's lanes read consecutive entries.
template <typename V>
__device__ __forceinline__ V Twiddle(const V *__restrict__ tw, int log2n, int e,
                                     bool inverse) {
  V w = __ldg(&tw[TwiddleBase(log2n) + e]);
  if (inverse) w.y = -w.y;
  return w;
}

// Twiddles of a fused pass (up to three radix-2 stages, spans 4h, 2h, h):
// stage S's butterfly m (m < S) takes W_{2Sh}^{k + m h}. Four are read from
// the table, W_{8h}^k, W_{8h}^{k + h}, W_{4h}^k and W_{2h}^k; the others are
// these times W_{2S}^{S/2} = -i (+i for the inverse), an exact rotation, so
// every twiddle is a table value.
template <typename V>
__device__ __forceinline__ V RotMinusI(V w, bool inverse) {
  V r;
  r.x = inverse ? -w.y : w.y;
  r.y = inverse ? w.x : -w.x;
  return r;
}
template <typename V>
__device__ __forceinline__ void PassTwiddles(const V *__restrict__ tw, int lh, int k,
                                             int R, bool inverse, V *wb) {
  if (R >= 8) {
    wb[0] = Twiddle(tw, lh + 3, k, inverse);
    wb[1] = Twiddle(tw, lh + 3, k + (1 << lh), inverse);
  }
  if (R >= 4) wb[2] = Twiddle(tw, lh + 2, k, inverse);
  wb[3] = Twiddle(tw, lh + 1, k, inverse);
}
template <typename V>
__device__ __forceinline__ V TwStage(const V *wb, int S, int m, bool inverse) {
  if (S == 4) return m < 2 ? wb[m] : RotMinusI(wb[m - 2], inverse);
  if (S == 2) return m == 0 ? wb[2] : RotMinusI(wb[2], inverse);
  return wb[3];
}

// In-place radix-2 FFTs of a[0..m) (padded layout) in shared memory (m = 2^log2m <=
// kMaxFFT), unnormalised, with up to three radix-2 stages fused per pass: a
// thread loads R = 2^r elements spaced h apart, runs the r stages in
// registers and stores them back, so a pass costs one barrier.
//   BlockFFTDif: decimation in frequency, natural order in, bit-reversed out.
//   BlockFFTDit: decimation in time, bit-reversed in, natural order out.
// A DIF forward transform, a pointwise product in bit-reversed order and a
// DIT inverse transform make a circular convolution without any reordering.
// Threads tid = 0 .. nth-1 share the transform (several transforms of the
// same size can run side by side in one block); every thread of the block
// must call them (each pass ends with a block barrier).
template <typename V, int R>
__device__ __forceinline__ void DifPass(V *a, int m, int lh, const V *tw,
                                        bool inverse, int tid, int nth) {
  const int groups = m / R;
  const int h = 1 << lh;
  for (int g = tid; g < groups; g += nth) {
    const int k = g & (h - 1);
    const int base = ((g >> lh) << lh) * R + k;
    V x[R];
    V wb[4];  // the pass's table twiddles (loads issued with the data)
    PassTwiddles(tw, lh, k, R, inverse, wb);
#pragma unroll
    for (int j = 0; j < R; ++j) x[j] = a[Pad(base + j * h)];
    // stages of span S h, S = R/2 .. 1: pairs (j, j + S), twiddle
    // W_{2Sh}^{k + (j mod S) h} on the difference
#pragma unroll
    for (int S = R / 2; S >= 1; S >>= 1) {
#pragma unroll
      for (int j = 0; j < R; ++j) {
        if ((j & S) == 0) {
          const V u = x[j], v = x[j + S];
          x[j] = vadd(u, v);
          x[j + S] = vmul(vsub(u, v), TwStage(wb, S, j & (S - 1), inverse));
        }
      }
    }
#pragma unroll
    for (int j = 0; j < R; ++j) a[Pad(base + j * h)] = x[j];
  }
  __syncthreads();
}

template <typename V, int R>
__device__ __forceinline__ void DitPass(V *a, int m, int lh, const V *tw,
                                        bool inverse, int tid, int nth) {
  const int groups = m / R;
  const int h = 1 << lh;
  for (int g = tid; g < groups; g += nth) {
    const int k = g & (h - 1);
    const int base = ((g >> lh) << lh) * R + k;
    V x[R];
    V wb[4];
    PassTwiddles(tw, lh, k, R, inverse, wb);
#pragma unroll
    for (int j = 0; j < R; ++j) x[j] = a[Pad(base + j * h)];
    // stages of span S h, S = 1 .. R/2: twiddle W_{2Sh}^{k + (j mod S) h}
    // on the upper input
#pragma unroll
    for (int S = 1; S < R; S <<= 1) {
#pragma unroll
      for (int j = 0; j < R; ++j) {
        if ((j & S) == 0) {
          const V u = x[j];
          const V v = vmul(x[j + S], TwStage(wb, S, j & (S - 1), inverse));
          x[j] = vadd(u, v);
          x[j + S] = vsub(u, v);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < R; ++j) a[Pad(base + j * h)] = x[j];
  }
  __syncthreads();
}

template <typename V>
__device__ void BlockFFTDif(V *a, int m, int log2m, const V *__restrict__ tw,
                            bool inverse, int tid, int nth) {
  // spans m/2, m/4, ..., 1 in passes of up to three stages
  int left = log2m;
  while (left > 0) {
    const int r = left >= 3 ? 3 : left;
    const int lh = left - r;  // log2 of the smallest span of this pass
    if (r == 3) {
      DifPass<V, 8>(a, m, lh, tw, inverse, tid, nth);
    } else if (r == 2) {
      DifPass<V, 4>(a, m, lh, tw, inverse, tid, nth);
    } else {
      DifPass<V, 2>(a, m, lh, tw, inverse, tid, nth);
    }
    left -= r;
  }
}

template <typename V>
__device__ void BlockFFTDit(V *a, int m, int log2m, const V *__restrict__ tw,
                            bool inverse, int tid, int nth) {
  // spans 1, 2, ..., m/2 in passes of up to three stages
  int done = 0;
  while (done < log2m) {
    const int r = log2m - done >= 3 ? 3 : log2m - done;
    // (done: log2 of the smallest span of this pass)
    if (r == 3) {
      DitPass<V, 8>(a, m, done, tw, inverse, tid, nth);
    } else if (r == 2) {
      DitPass<V, 4>(a, m, done, tw, inverse, tid, nth);
    } else {
      DitPass<V, 2>(a, m, done, tw, inverse, tid, nth);
    }
    done += r;
  }
}

}  // namespace mpsft
