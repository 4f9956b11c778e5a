// Window tables, FFT twiddles and Bluestein chirp tables.
//
// Window (src/window.cc:28-75): wt(t) = w * sinc(pi t w) * exp(-2 (pi t sigma_f)^2)
// with w = 1/(2 bins); wt(0) = w. The window is even, so only |t| in
// [0, p2] is stored. Computed in FP64 and also rounded to FP32.
//
// Bluestein (chirp-z) form of the size-B DFT X[k] = sum_j y[j] e^{-2 pi i jk/B}:
//   X[k] = chirp[k] * sum_j (y[j] chirp[j]) * conj(chirp[k - j]),
//   chirp[j] = e^{-pi i j^2 / B} with j^2 reduced mod 2B exactly,
// a circular convolution of length M = 2^ceil(log2(2B - 1)) done with the
// shared-memory FFT; chat = FFT_M of the conjugate chirp sequence, stored in
// bit-reversed order.
#include "fft.cuh"
#include "launch.h"

namespace mpsft {

namespace {

__global__ void k_twiddles(float2 *tw32, double2 *tw64) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kTwiddleEntries) return;
  TwiddleAt(e, tw32, tw64);
}

// sin(x)/x with the reference's Taylor guard (src/sincos.cc:69-88).
__device__ double SincPi(double x) {
  const double t0 = 2.220446049250313080847e-16;  // DBL_EPSILON
  const double t2 = 1.4901161193847656e-08;       // sqrt(t0)
  const double tn = 1.220703125e-04;              // sqrt(t2)
  if (x < 0) x = -x;
  if (x >= tn) return sin(x) / x;
  double r = 1.0;
  if (x >= t0) {
    const double x2 = x * x;
    r -= x2 / 6.0;
    if (x >= t2) r += (x2 * x2) / 120.0;
  }
  return r;
}

// FP64 window (the reference's evaluation order) into wt64 and, when
// present, the float-float copy wtff; with_fp32 also rounds it into wt32.
__global__ void k_window64(const SigIter *__restrict__ its, int with_fp32) {
  PdlEnter(its, kTraceWindow64);
  const SigIter &it = its[blockIdx.y];
  if (!it.active || it.tables_valid) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > it.p2) return;
  double v;
  if (i == 0) {
    v = it.width;
  } else {
    const double t = double(i);
    const double u = __dmul_rn(__dmul_rn(t, M_PI), it.sigma_f);
    v = __dmul_rn(__dmul_rn(it.width, SincPi(__dmul_rn(__dmul_rn(t, M_PI),
                                                       it.width))),
                  exp(__dmul_rn(__dmul_rn(-2.0, u), u)));
  }
  it.wt64[i] = v;
  if (with_fp32) it.wt32[i] = float(v);
  if (it.wtff != nullptr) {
    const float h = __double2float_rn(v);
    it.wtff[i] = make_float2(h, __double2float_rn(v - double(h)));
  }
}

// The same window evaluated in FP32 for the FP32 binning (a few ulp; the
// FP64 tables are built beside it, off the binning's critical path).
__global__ void k_window32(const SigIter *__restrict__ its) {
  PdlEnter(its, kTraceWindow32);
  const SigIter &it = its[blockIdx.y];
  if (!it.active || it.tables_valid || it.force_fp64) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > it.p2) return;
  const float w = float(it.width);
  float v = w;
  if (i > 0) {
    const float t = float(i);
    const float y = t * w;  // sinc argument in units of pi
    const float u = t * float(M_PI * it.sigma_f);
    v = w * (sinpif(y) / (float(M_PI) * y)) * expf(-2.f * u * u);
  }
  it.wt32[i] = v;
}

// ph_lo[l] = e^{2 pi i l / n} for l < 2^ph_k and ph_hi[h] = e^{2 pi i h 2^ph_k / n}
// for h <= (n - 1) >> ph_k, from exact integer phases.
__global__ void k_phase_tables(const SigIter *__restrict__ its) {
  const SigIter &it = its[blockIdx.y];
  if (!it.ph_build) return;  // (tables shared with another signal, or cached)
  const int64_t n = it.n;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  double s, c;
  if (i < (int64_t(1) << it.ph_k)) {
    sincospi(2.0 * (double(i) / double(n)), &s, &c);
    it.ph_lo[i] = make_double2(c, s);
  }
  if (i <= ((n - 1) >> it.ph_k)) {
    sincospi(2.0 * (double(i << it.ph_k) / double(n)), &s, &c);
    it.ph_hi[i] = make_double2(c, s);
  }
}

__device__ inline float2 *ChirpOf(const SigIter &it, float2 *) { return it.chirp32; }
__device__ inline double2 *ChirpOf(const SigIter &it, double2 *) { return it.chirp64; }
__device__ inline float2 *ChatOf(const SigIter &it, float2 *) { return it.chat32; }
__device__ inline double2 *ChatOf(const SigIter &it, double2 *) { return it.chat64; }

// cond: only signals with more near-tie bins than their list holds (whose
// iteration is redone in FP64) take part.
template <typename V>
__global__ void __launch_bounds__(512)
    k_bluestein_setup(const SigIter *__restrict__ its, const V *__restrict__ tw,
                      int cond) {
  PdlEnter(its, kTraceBluestein);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *a = reinterpret_cast<V *>(smem_raw);
  const SigIter &it = its[blockIdx.x];
  if (!it.active) return;
  if (cond ? !RedoFP64(it) : (it.force_fp64 || it.tables_valid)) return;
  const int B = it.bins, M = it.fft_m;
  V *chirp = ChirpOf(it, (V *)nullptr);
  V *chat = ChatOf(it, (V *)nullptr);
  const int64_t twoB = 2 * int64_t(B);
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    a[Pad(j)] = vmake2(0.0, 0.0, (V *)nullptr);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < B; j += blockDim.x) {
    const int64_t j2 = (int64_t(j) * j) % twoB;
    double s, c;
    sincospi(-double(j2) / double(B), &s, &c);
    chirp[j] = vmake2(c, s, (V *)nullptr);
    const V cc = vmake2(c, -s, (V *)nullptr);  // conj(chirp[j])
    a[Pad(j)] = cc;
    if (j > 0) a[Pad(M - j)] = cc;
  }
  // FP32 tables: the bins-grid unit roots of the near-tie phase steps
  if (!cond && sizeof(V) == sizeof(float2) && it.r2b64 != nullptr) {
    for (int r = threadIdx.x; r < twoB; r += blockDim.x) {
      double s, c;
      sincospi(-double(r) / double(B), &s, &c);
      it.r2b64[r] = make_double2(c, s);
    }
  }
  __syncthreads();
  // chat in bit-reversed order (the row transforms' forward output order)
  BlockFFTDif(a, M, it.fft_log2m, tw, false, int(threadIdx.x), int(blockDim.x));
  for (int j = threadIdx.x; j < M; j += blockDim.x) chat[j] = a[Pad(j)];
}

}  // namespace

void LaunchTwiddles(float2 *tw32, double2 *tw64, cudaStream_t s) {
  const int n = kTwiddleEntries;
  k_twiddles<<<(n + 255) / 256, 256, 0, s>>>(tw32, tw64);
}

void LaunchPhaseTables(const SigIter *d_its, int nsig, int64_t entries,
                       cudaStream_t s) {
  dim3 grid(unsigned((entries + 255) / 256), nsig);
  k_phase_tables<<<grid, 256, 0, s>>>(d_its);
}

void LaunchWindow(const SigIter *d_its, int nsig, int max_p2, cudaStream_t s) {
  dim3 grid((max_p2 + 1 + 255) / 256, nsig);
  Launch(k_window64, grid, 256, 0, s, d_its, 1);
}

void LaunchWindow64(const SigIter *d_its, int nsig, int max_p2, cudaStream_t s) {
  dim3 grid((max_p2 + 1 + 255) / 256, nsig);
  Launch(k_window64, grid, 256, 0, s, d_its, 0);
}

void LaunchWindow32(const SigIter *d_its, int nsig, int max_p2, cudaStream_t s) {
  dim3 grid((max_p2 + 1 + 255) / 256, nsig);
  Launch(k_window32, grid, 256, 0, s, d_its);
}

void LaunchBluesteinSetup(const SigIter *d_its, int nsig, int max_m, bool fp64,
                          const float2 *tw32, const double2 *tw64,
                          cudaStream_t s, bool cond) {
  if (fp64) {
    const size_t sm = size_t(PadLen(max_m)) * sizeof(double2);
    cudaFuncSetAttribute(k_bluestein_setup<double2>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    Launch(k_bluestein_setup<double2>, nsig, 512, sm, s, d_its, tw64, cond ? 1 : 0);
  } else {
    const size_t sm = size_t(PadLen(max_m)) * sizeof(float2);
    cudaFuncSetAttribute(k_bluestein_setup<float2>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    Launch(k_bluestein_setup<float2>, nsig, 512, sm, s, d_its, tw32, cond ? 1 : 0);
  }
}

}  // namespace mpsft

namespace mpsft {

namespace {

// Deterministic mean |x|^2: block b of signal s sums a fixed share in a
// fixed tree order, then one block adds the partials in order. per_block = 0:
// every sample (grid stride); otherwise block b sums the per_block samples
// from n b / kEnergyBlocks on (an estimate from kEnergyBlocks evenly spread
// runs).
template <typename TX>
__global__ void k_energy_partial(const void *const *__restrict__ xs,
                                 const int64_t *__restrict__ ns,
                                 double *__restrict__ energy, int per_block) {
  __shared__ double red[256];
  const int sig = blockIdx.y;
  const TX *x = reinterpret_cast<const TX *>(xs[sig]);
  const int64_t n = ns[sig];
  // per-thread sums in FP32 (a few thousand terms), combined in FP64
  float acc = 0.f;
  const int64_t run = per_block > 0 ? min(int64_t(per_block), n / kEnergyBlocks) : 0;
  if (run > 0) {
    const int64_t start = n * blockIdx.x / kEnergyBlocks;
    for (int64_t i = threadIdx.x; i < run; i += blockDim.x) {
      const TX v = x[start + i];
      const float re = float(v.x), im = float(v.y);
      acc = fmaf(re, re, fmaf(im, im, acc));
    }
  } else {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += int64_t(gridDim.x) * blockDim.x) {
      const TX v = x[i];
      const float re = float(v.x), im = float(v.y);
      acc = fmaf(re, re, fmaf(im, im, acc));
    }
  }
  red[threadIdx.x] = double(acc);
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) energy[size_t(sig) * kEnergyStride + 1 + blockIdx.x] = red[0];
}

__global__ void k_energy_final(const int64_t *__restrict__ ns,
                               double *__restrict__ energy, int per_block) {
  __shared__ double red[kEnergyBlocks];
  const int sig = blockIdx.x;
  double *e = energy + size_t(sig) * kEnergyStride;
  red[threadIdx.x] = e[1 + threadIdx.x];
  __syncthreads();
  for (int o = kEnergyBlocks / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  const int64_t n = ns[sig];
  const int64_t run = per_block > 0 ? min(int64_t(per_block), n / kEnergyBlocks) : 0;
  if (threadIdx.x == 0) e[0] = red[0] / double(run > 0 ? run * kEnergyBlocks : n);
}

// The estimate alone (per_block > 0): one block per signal, thread t taking
// sample t of every run, then the block's fixed tree; a signal shorter than
// kEnergyBlocks runs of per_block samples is summed whole.
template <typename TX>
__global__ void __launch_bounds__(256)
    k_energy_sample(const void *const *__restrict__ xs, const int64_t *__restrict__ ns,
                    double *__restrict__ energy, int per_block) {
  __shared__ double red[256];
  const int sig = blockIdx.x;
  const TX *x = reinterpret_cast<const TX *>(xs[sig]);
  const int64_t n = ns[sig];
  const int64_t run = min(int64_t(per_block), n / kEnergyBlocks);
  float acc = 0.f;
  if (run > 0) {
    for (int r = 0; r < kEnergyBlocks; ++r) {
      const int64_t start = n * r / kEnergyBlocks;
      for (int64_t i = threadIdx.x; i < run; i += blockDim.x) {
        const TX v = x[start + i];
        const float re = float(v.x), im = float(v.y);
        acc = fmaf(re, re, fmaf(im, im, acc));
      }
    }
  } else {
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      const TX v = x[i];
      const float re = float(v.x), im = float(v.y);
      acc = fmaf(re, re, fmaf(im, im, acc));
    }
  }
  red[threadIdx.x] = double(acc);
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    energy[size_t(sig) * kEnergyStride] = red[0] / double(run > 0 ? run * kEnergyBlocks : n);
  }
}

}  // namespace

void LaunchEnergy(const void *const *x, const int64_t *n, int nsig, bool c128,
                  double *energy, cudaStream_t s, int per_block) {
  if (per_block > 0) {
    if (c128) {
      k_energy_sample<double2><<<nsig, 256, 0, s>>>(x, n, energy, per_block);
    } else {
      k_energy_sample<float2><<<nsig, 256, 0, s>>>(x, n, energy, per_block);
    }
    return;
  }
  dim3 grid(kEnergyBlocks, nsig);
  if (c128) {
    k_energy_partial<double2><<<grid, 256, 0, s>>>(x, n, energy, 0);
  } else {
    k_energy_partial<float2><<<grid, 256, 0, s>>>(x, n, energy, 0);
  }
  k_energy_final<<<nsig, kEnergyBlocks, 0, s>>>(n, energy, 0);
}

bool WindowKernelsLaunchable() {
  int n1 = 0, n2 = 0;
  const size_t sm32 = size_t(PadLen(kMaxFFT)) * sizeof(float2);
  const size_t sm64 = size_t(PadLen(kMaxFFT64)) * sizeof(double2);
  cudaFuncSetAttribute(k_bluestein_setup<float2>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm32));
  cudaFuncSetAttribute(k_bluestein_setup<double2>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm64));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_bluestein_setup<float2>, 512, sm32);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n2, k_bluestein_setup<double2>, 512, sm64);
  return n1 > 0 && n2 > 0;
}

}  // namespace mpsft
