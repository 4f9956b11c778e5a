// Shared-memory radix-2 FFT used by the Bluestein size-B transform.
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

// In-place FFT of a[0..m) in shared memory (m = 2^log2m <= kMaxFFT), natural
// order in and out, unnormalised. tw[e] = e^{-2 pi i e / kMaxFFT} for
// e < kMaxFFT / 2 (global, read through the read-only cache). inverse selects
// the conjugate twiddles. Every thread of the block must call it.
template <typename V>
__device__ void BlockFFT(V *a, int m, int log2m, const V *__restrict__ tw,
                         bool inverse) {
  if (log2m == 0) return;  // a 1-point transform is the identity
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    const int j = int(__brev(uint32_t(i)) >> (32 - log2m));
    if (j > i) {
      const V t = a[i];
      a[i] = a[j];
      a[j] = t;
    }
  }
  __syncthreads();
  for (int s = 0; s < log2m; ++s) {
    const int h = 1 << s;
    const int stride = kMaxFFT >> (s + 1);
    for (int bf = threadIdx.x; bf < (m >> 1); bf += blockDim.x) {
      const int j = bf & (h - 1);
      const int i0 = ((bf >> s) << (s + 1)) + j;
      const int i1 = i0 + h;
      V w = __ldg(&tw[j * stride]);
      if (inverse) w.y = -w.y;
      const V u = a[i0];
      const V v = vmul(a[i1], w);
      a[i0] = vadd(u, v);
      a[i1] = vsub(u, v);
    }
    __syncthreads();
  }
}

}  // namespace mpsft
