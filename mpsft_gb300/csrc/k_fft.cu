// Size-B forward DFT of every folded row (FFTPlan::Run of size B,
// src/base.cc:86-97, called at src/binner.cc:428 and 509-510), by Bluestein's
// chirp-z method over the shared-memory radix-2 FFT (any odd B, including
// large primes), followed by the row factor e^{2 pi i (b q mod n)/n} that the
// fold left out. Output: complex128 bins in ubuf.
//
// One CTA per (row, trial, signal). FP32 path: the convolution runs in FP32
// (M <= 16384 points, 128 KB of shared memory); FP64 path: in FP64
// (M <= 8192).
#include "fft.cuh"
#include "launch.h"

namespace mpsft {

namespace {

template <typename V>
__global__ void __launch_bounds__(512)
    k_row_fft(const SigIter *__restrict__ its, int max_trials,
              const V *__restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *a = reinterpret_cast<V *>(smem_raw);
  const SigIter &it = its[blockIdx.z];
  if (!it.active) return;
  const int row = blockIdx.x;
  const int tr = blockIdx.y;
  if (row >= it.rows || tr >= it.trials) return;
  const int B = it.bins, M = it.fft_m;
  const V *__restrict__ chirp = reinterpret_cast<const V *>(it.chirp);
  const V *__restrict__ chat = reinterpret_cast<const V *>(it.chat);
  const V *__restrict__ src = reinterpret_cast<const V *>(it.fold) +
                              (size_t(tr) * it.rows + row) * it.bins_cap;
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    a[j] = j < B ? vmul(src[j], __ldg(&chirp[j]))
                 : vmake2(0.0, 0.0, (V *)nullptr);
  }
  __syncthreads();
  BlockFFT(a, M, it.fft_log2m, tw, false);
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    a[j] = vmul(a[j], __ldg(&chat[j]));
  }
  __syncthreads();
  BlockFFT(a, M, it.fft_log2m, tw, true);
  const double inv_m = 1.0 / double(M);
  const double2 bq = make_double2(it.bq_re[tr], it.bq_im[tr]);
  double2 *dst = it.ubuf + (size_t(tr) * it.rows + row) * it.bins_cap;
  for (int k = threadIdx.x; k < B; k += blockDim.x) {
    const double2 y = cscale(to_d2(vmul(a[k], __ldg(&chirp[k]))), inv_m);
    dst[k] = cmul(bq, y);
  }
}

}  // namespace

void LaunchRowFFT(const SigIter *d_its, int nsig, int max_rows,
                  int max_trials, int max_m, bool fp64, const float2 *tw32,
                  const double2 *tw64, cudaStream_t s) {
  dim3 grid(max_rows, max_trials, nsig);
  if (fp64) {
    const size_t sm = size_t(max_m) * sizeof(double2);
    cudaFuncSetAttribute(k_row_fft<double2>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    k_row_fft<double2><<<grid, 512, sm, s>>>(d_its, max_trials, tw64);
  } else {
    const size_t sm = size_t(max_m) * sizeof(float2);
    cudaFuncSetAttribute(k_row_fft<float2>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    k_row_fft<float2><<<grid, 512, sm, s>>>(d_its, max_trials, tw32);
  }
}

}  // namespace mpsft
