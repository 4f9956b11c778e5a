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

__device__ inline const float2 *ChirpOf(const SigIter &it, float2 *) { return it.chirp32; }
__device__ inline const double2 *ChirpOf(const SigIter &it, double2 *) { return it.chirp64; }
__device__ inline const float2 *ChatOf(const SigIter &it, float2 *) { return it.chat32; }
__device__ inline const double2 *ChatOf(const SigIter &it, double2 *) { return it.chat64; }

// cond: only signals whose iteration is redone in FP64 take part. Also
// records the largest |U| of each row (used by the FP32 near-tie bound).
template <typename V>
__global__ void __launch_bounds__(512)
    k_row_fft(const SigIter *__restrict__ its, int max_trials,
              const V *__restrict__ tw, int cond) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float red[16];
  V *a = reinterpret_cast<V *>(smem_raw);
  const SigIter &it = its[blockIdx.z];
  if (!it.active) return;
  if (cond ? !RedoFP64(it) : it.force_fp64) return;
  const int row = blockIdx.x;
  const int tr = blockIdx.y;
  if (row >= it.rows || tr >= it.trials) return;
  const int B = it.bins, M = it.fft_m;
  const V *__restrict__ chirp = ChirpOf(it, (V *)nullptr);
  const V *__restrict__ chat = ChatOf(it, (V *)nullptr);
  const V *__restrict__ src = reinterpret_cast<const V *>(it.fold) +
                              (size_t(tr) * it.rows + row) * it.bins_cap;
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    a[Pad(j)] = j < B ? vmul(src[j], __ldg(&chirp[j]))
                      : vmake2(0.0, 0.0, (V *)nullptr);
  }
  __syncthreads();
  // forward DIF (bit-reversed out), product with chat (stored bit-reversed),
  // inverse DIT (natural out)
  BlockFFTDif(a, M, it.fft_log2m, tw, false);
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    a[Pad(j)] = vmul(a[Pad(j)], __ldg(&chat[j]));
  }
  __syncthreads();
  BlockFFTDit(a, M, it.fft_log2m, tw, true);
  const double inv_m = 1.0 / double(M);
  const double2 bq = make_double2(it.bq_re[tr], it.bq_im[tr]);
  double2 *dst = it.ubuf + (size_t(tr) * it.rows + row) * it.bins_cap;
  float mx = 0.f;
  for (int k = threadIdx.x; k < B; k += blockDim.x) {
    const double2 y = cscale(to_d2(vmul(a[Pad(k)], __ldg(&chirp[k]))), inv_m);
    dst[k] = cmul(bq, y);
    mx = fmaxf(mx, float(sqrt(y.x * y.x + y.y * y.y)));
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0 && it.row_max != nullptr) {
    for (int w = 1; w < int(blockDim.x >> 5); ++w) mx = fmaxf(mx, red[w]);
    it.row_max[tr * it.rows + row] = mx;
  }
}

}  // namespace

void LaunchRowFFT(const SigIter *d_its, int nsig, int max_rows,
                  int max_trials, int max_m, bool fp64, const float2 *tw32,
                  const double2 *tw64, cudaStream_t s, bool cond) {
  dim3 grid(max_rows, max_trials, nsig);
  if (fp64) {
    const size_t sm = size_t(PadLen(max_m)) * sizeof(double2);
    cudaFuncSetAttribute(k_row_fft<double2>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    k_row_fft<double2><<<grid, 512, sm, s>>>(d_its, max_trials, tw64,
                                             cond ? 1 : 0);
  } else {
    const size_t sm = size_t(PadLen(max_m)) * sizeof(float2);
    cudaFuncSetAttribute(k_row_fft<float2>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    k_row_fft<float2><<<grid, 512, sm, s>>>(d_its, max_trials, tw32,
                                            cond ? 1 : 0);
  }
}

bool FftKernelsLaunchable() {
  int n1 = 0, n2 = 0;
  const size_t sm32 = size_t(PadLen(kMaxFFT)) * sizeof(float2);
  const size_t sm64 = size_t(PadLen(kMaxFFT64)) * sizeof(double2);
  cudaFuncSetAttribute(k_row_fft<float2>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm32));
  cudaFuncSetAttribute(k_row_fft<double2>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm64));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_row_fft<float2>, 512, sm32);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n2, k_row_fft<double2>, 512, sm64);
  return n1 > 0 && n2 > 0;
}

}  // namespace mpsft
