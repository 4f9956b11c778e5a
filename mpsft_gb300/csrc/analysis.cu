// Test data and result analysis of the recovery loop, on the device (the
// reference does both on the host, around Demo1::Run):
//   mpsft_generate_mode_map  GenerateModeMap (src/gen.cc:27-39), host;
//   mpsft_signal_generate    Demo1's constructor (src/demo1.cc:27-34) with
//                            GenerateXhatAlt's distribution (src/gen.cc:77-89);
//   mpsft_signal_spectrum    xhat = FFT(x) / n in FP64;
//   mpsft_post_analyze       Demo1::PostAnalyze (src/demo1.cc:61-112).
// The dense size-n transforms are cuFFT Z2Z. cuFFT is opened at the first
// call that needs it, so the rest of the library does not depend on it.
#include <cufft.h>
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_set>
#include <vector>

#include "internal.h"

namespace {

using mpsft::CtxFail;

#define ACUDA(ctx, call)                                                        \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      return CtxFail(ctx, MPSFT_ERR_CUDA,                                       \
                     std::string(#call) + ": " + cudaGetErrorString(e_));       \
    }                                                                           \
  } while (0)

constexpr int kThreads = 256;
constexpr int kBlocks = 152 * 4;  // grid-stride kernels: 4 blocks per SM

// ------------------------------------------------------------------ cuFFT
struct CufftApi {
  decltype(&cufftCreate) create = nullptr;
  decltype(&cufftMakePlanMany64) make_plan = nullptr;
  decltype(&cufftSetStream) set_stream = nullptr;
  decltype(&cufftExecZ2Z) exec_z2z = nullptr;
  decltype(&cufftDestroy) destroy = nullptr;
  bool ok = false;
};

const CufftApi &Cufft() {
  static const CufftApi api = [] {
    CufftApi a;
    std::vector<std::string> names = {"libcufft.so.12", "libcufft.so"};
    const char *home = std::getenv("CUDA_HOME");
    names.push_back(std::string(home ? home : "/usr/local/cuda") +
                    "/lib64/libcufft.so.12");
    void *h = nullptr;
    for (const std::string &name : names) {
      h = dlopen(name.c_str(), RTLD_NOW | RTLD_LOCAL);
      if (h) break;
    }
    if (!h) return a;
    a.create = reinterpret_cast<decltype(a.create)>(dlsym(h, "cufftCreate"));
    a.make_plan =
        reinterpret_cast<decltype(a.make_plan)>(dlsym(h, "cufftMakePlanMany64"));
    a.set_stream = reinterpret_cast<decltype(a.set_stream)>(dlsym(h, "cufftSetStream"));
    a.exec_z2z = reinterpret_cast<decltype(a.exec_z2z)>(dlsym(h, "cufftExecZ2Z"));
    a.destroy = reinterpret_cast<decltype(a.destroy)>(dlsym(h, "cufftDestroy"));
    a.ok = a.create && a.make_plan && a.set_stream && a.exec_z2z && a.destroy;
    return a;
  }();
  return api;
}

// An in-place size-n Z2Z transform on ctx's stream (plan destroyed with the
// object; the caller synchronises the stream first).
class DenseFft {
 public:
  ~DenseFft() {
    if (made_) Cufft().destroy(plan_);
  }
  int Exec(mpsft_ctx *ctx, int64_t n, double2 *data, int direction) {
    const CufftApi &f = Cufft();
    if (!f.ok) {
      return CtxFail(ctx, MPSFT_ERR_CUDA, "cuFFT (libcufft.so.12) could not be opened");
    }
    if (!made_) {
      if (f.create(&plan_) != CUFFT_SUCCESS) {
        return CtxFail(ctx, MPSFT_ERR_CUDA, "cufftCreate failed");
      }
      made_ = true;
      long long dims[1] = {static_cast<long long>(n)};
      size_t work = 0;
      if (f.make_plan(plan_, 1, dims, nullptr, 1, n, nullptr, 1, n, CUFFT_Z2Z, 1,
                      &work) != CUFFT_SUCCESS) {
        return CtxFail(ctx, MPSFT_ERR_NOMEM, "cuFFT plan of size n failed");
      }
      if (f.set_stream(plan_, ctx->stream) != CUFFT_SUCCESS) {
        return CtxFail(ctx, MPSFT_ERR_CUDA, "cufftSetStream failed");
      }
    }
    cufftDoubleComplex *p = reinterpret_cast<cufftDoubleComplex *>(data);
    if (f.exec_z2z(plan_, p, p, direction) != CUFFT_SUCCESS) {
      return CtxFail(ctx, MPSFT_ERR_CUDA, "cufftExecZ2Z failed");
    }
    return MPSFT_OK;
  }

 private:
  cufftHandle plan_ = 0;
  bool made_ = false;
};

// Device buffers freed on the context's stream when the call returns.
class Scratch {
 public:
  explicit Scratch(mpsft_ctx *ctx) : ctx_(ctx) {}
  ~Scratch() {
    for (void *p : ptrs_) cudaFreeAsync(p, ctx_->stream);
  }
  template <class T>
  int Take(size_t count, T **out) {
    void *p = nullptr;
    if (cudaMallocAsync(&p, std::max<size_t>(count, 1) * sizeof(T), ctx_->stream) !=
        cudaSuccess) {
      cudaGetLastError();
      return CtxFail(ctx_, MPSFT_ERR_NOMEM, "device scratch allocation failed");
    }
    ptrs_.push_back(p);
    *out = static_cast<T *>(p);
    return MPSFT_OK;
  }

 private:
  mpsft_ctx *ctx_;
  std::vector<void *> ptrs_;
};

// ---------------------------------------------------------------- kernels
// SplitMix64 (Steele, Lea and Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014): output i of the sequence started at seed is the
// mix of seed + (i + 1) * golden gamma, so any output is computed directly.
constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ull;

__device__ __forceinline__ double UniformOpen0(uint64_t seed, uint64_t i) {
  uint64_t z = seed + (i + 1) * kGamma;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return double((z >> 11) + 1) * 0x1p-53;  // (0, 1]
}

__global__ void k_scatter_modes(const int32_t *__restrict__ k,
                                const double2 *__restrict__ c, int64_t count,
                                double2 *__restrict__ xh) {
  for (int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; j < count;
       j += int64_t(gridDim.x) * blockDim.x) {
    xh[k[j]] = c[j];
  }
}

__device__ __forceinline__ void Store(float2 *p, double2 v) {
  *p = make_float2(float(v.x), float(v.y));
}
__device__ __forceinline__ void Store(double2 *p, double2 v) { *p = v; }

// out[t] = modes[t] + noise_t; the noise pair from outputs 2t, 2t+1 by the
// Box-Muller transform, scaled to variance sigma^2 / 2 per component.
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_add_noise(const double2 *__restrict__ modes, T *__restrict__ out, int64_t n,
                double sigma, uint64_t seed) {
  const double h = sigma * 0.70710678118654752440;
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
       t += int64_t(gridDim.x) * blockDim.x) {
    double2 v = modes[t];
    if (sigma > 0.0) {
      const double u1 = UniformOpen0(seed, 2 * uint64_t(t));
      const double u2 = UniformOpen0(seed, 2 * uint64_t(t) + 1);
      const double r = sqrt(-2.0 * log(u1));
      double s, c;
      sincospi(2.0 * u2, &s, &c);
      v.x += h * (r * c);
      v.y += h * (r * s);
    }
    Store(out + t, v);
  }
}

template <class T>
__global__ void __launch_bounds__(kThreads)
    k_widen(const T *__restrict__ x, double2 *__restrict__ y, int64_t n) {
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
       t += int64_t(gridDim.x) * blockDim.x) {
    const T v = x[t];
    y[t] = make_double2(double(v.x), double(v.y));
  }
}

__global__ void __launch_bounds__(kThreads)
    k_divide(double2 *__restrict__ y, int64_t n) {
  const double dn = double(n);
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
       t += int64_t(gridDim.x) * blockDim.x) {
    y[t] = make_double2(y[t].x / dn, y[t].y / dn);
  }
}

__global__ void k_mark(const int32_t *__restrict__ k, int64_t count,
                       uint32_t *__restrict__ bits) {
  for (int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; j < count;
       j += int64_t(gridDim.x) * blockDim.x) {
    atomicOr(&bits[k[j] >> 5], 1u << (k[j] & 31));
  }
}

// Sum, sum of squares and maximum of v over a block (fixed order), written
// by thread 0 to out[0..3).
__device__ void BlockReduce3(double s1, double s2, double mx, double *out) {
  __shared__ double sh[3][kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sh[0][w] = s1;
    sh[1][w] = s2;
    sh[2][w] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0, m = 0.0;
    for (int i = 0; i < kThreads / 32; ++i) {
      a += sh[0][i];
      b += sh[1][i];
      m = fmax(m, sh[2][i]);
    }
    out[0] = a;
    out[1] = b;
    out[2] = m;
  }
}

// |xhat_i| at every frequency without a found mode (the found spectrum is 0
// there): per-block sum, sum of squares and maximum.
__global__ void __launch_bounds__(kThreads)
    k_unfound_err(const double2 *__restrict__ xh, const uint32_t *__restrict__ bits,
                  int64_t n, double *__restrict__ partial) {
  double s1 = 0.0, s2 = 0.0, mx = 0.0;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    if ((bits[i >> 5] >> (i & 31)) & 1u) continue;
    const double e = hypot(xh[i].x, xh[i].y);
    s1 += e;
    s2 += e * e;
    mx = fmax(mx, e);
  }
  BlockReduce3(s1, s2, mx, partial + 3 * blockIdx.x);
}

// One block: for every found mode e = |c - xhat_k|, split into hits (k in
// the sorted true positions) and misses. out: {hit sum, hit sum of squares,
// miss sum, miss sum of squares, found sum, found sum of squares, found max};
// counts: {hits, misses}.
__global__ void __launch_bounds__(kThreads)
    k_found_err(const double2 *__restrict__ xh, const int32_t *__restrict__ fk,
                const double2 *__restrict__ fc, int64_t count,
                const int32_t *__restrict__ tk, int64_t tcount, double *out,
                int32_t *counts) {
  double h1 = 0.0, h2 = 0.0, m1 = 0.0, m2 = 0.0, mx = 0.0;
  int32_t hits = 0;
  for (int64_t j = threadIdx.x; j < count; j += blockDim.x) {
    const int32_t k = fk[j];
    const double e = hypot(fc[j].x - xh[k].x, fc[j].y - xh[k].y);
    int64_t lo = 0, hi = tcount;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (tk[mid] < k) lo = mid + 1; else hi = mid;
    }
    if (lo < tcount && tk[lo] == k) {
      h1 += e;
      h2 += e * e;
      ++hits;
    } else {
      m1 += e;
      m2 += e * e;
    }
    mx = fmax(mx, e);
  }
  __shared__ double sh[3];
  BlockReduce3(h1, h2, 0.0, sh);
  __syncthreads();
  if (threadIdx.x == 0) {
    out[0] = sh[0];
    out[1] = sh[1];
  }
  __syncthreads();
  BlockReduce3(m1, m2, mx, sh);
  __syncthreads();
  if (threadIdx.x == 0) {
    out[2] = sh[0];
    out[3] = sh[1];
    out[6] = sh[2];
  }
  __shared__ int32_t hsum;
  if (threadIdx.x == 0) hsum = 0;
  __syncthreads();
  atomicAdd(&hsum, hits);
  __syncthreads();
  if (threadIdx.x == 0) {
    counts[0] = hsum;
    counts[1] = int32_t(count) - hsum;
  }
}

unsigned GridFor(int64_t n) {
  return unsigned(std::max<int64_t>(1, std::min<int64_t>(kBlocks, (n + kThreads - 1) / kThreads)));
}

// xhat = FFT(x) / n of sig into y (n values, device).
int Spectrum(mpsft_ctx *ctx, const mpsft_signal *sig, double2 *y) {
  const int64_t n = sig->n;
  if (sig->dtype == MPSFT_C128) {
    ACUDA(ctx, cudaMemcpyAsync(y, sig->d_x, size_t(n) * sizeof(double2),
                               cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    k_widen<float2><<<GridFor(n), kThreads, 0, ctx->stream>>>(
        static_cast<const float2 *>(sig->d_x), y, n);
    ACUDA(ctx, cudaGetLastError());
  }
  DenseFft fft;
  int rc = fft.Exec(ctx, n, y, CUFFT_FORWARD);
  if (rc) return rc;
  k_divide<<<GridFor(n), kThreads, 0, ctx->stream>>>(y, n);
  ACUDA(ctx, cudaGetLastError());
  // the plan's work area must outlive the transform
  ACUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MPSFT_OK;
}

// Sorted copy of positions; MPSFT_ERR_INVALID unless all lie in [0, n) and
// (when distinct) none repeats.
int SortedPositions(mpsft_ctx *ctx, const int32_t *k, int64_t count, int64_t n,
                    bool distinct, std::vector<int32_t> *out) {
  out->assign(k, k + count);
  std::sort(out->begin(), out->end());
  if (count > 0 && (out->front() < 0 || out->back() >= n)) {
    return CtxFail(ctx, MPSFT_ERR_INVALID, "positions must lie in [0, n)");
  }
  if (distinct && std::adjacent_find(out->begin(), out->end()) != out->end()) {
    return CtxFail(ctx, MPSFT_ERR_INVALID, "positions must be distinct");
  }
  return MPSFT_OK;
}

}  // namespace

extern "C" {

int mpsft_generate_mode_map(mpsft_rng *rng, int32_t n, int32_t count,
                            int32_t *out_k, double *out_c) {
  if (!rng || n <= 0 || count < 0 || count > n || (count > 0 && (!out_k || !out_c))) {
    return MPSFT_ERR_INVALID;
  }
  // the reference writes Cplex(RandomNormal(), RandomNormal()); its g++
  // build evaluates the two arguments right to left, so the imaginary part
  // takes the first draw
  std::unordered_set<int32_t> seen;
  int32_t m = 0;
  while (m < count) {
    const int32_t idx = rng->Draw() % n;  // Draw() >= 0: UnsafePosMod
    if (!seen.insert(idx).second) continue;
    const double im = rng->Normal();
    const double re = rng->Normal();
    std::complex<double> c(re, im);
    c /= std::abs(c);
    out_k[m] = idx;
    out_c[2 * m] = c.real();
    out_c[2 * m + 1] = c.imag();
    ++m;
  }
  return MPSFT_OK;
}

int mpsft_signal_generate(mpsft_ctx *ctx, int64_t n, const int32_t *k,
                          const double *coef, int64_t count, double sigma,
                          uint64_t seed, int dtype, mpsft_signal **out) {
  if (!ctx || !out || count < 0 || (count > 0 && (!k || !coef))) {
    return CtxFail(ctx, MPSFT_ERR_INVALID, "null argument");
  }
  if (dtype != MPSFT_C64 && dtype != MPSFT_C128) {
    return CtxFail(ctx, MPSFT_ERR_INVALID, "dtype must be MPSFT_C64 or MPSFT_C128");
  }
  if (!(sigma >= 0.0) || !std::isfinite(sigma)) {
    return CtxFail(ctx, MPSFT_ERR_INVALID, "sigma must be finite and >= 0");
  }
  int rc = mpsft::CtxCheckN(ctx, n);
  if (rc) return rc;
  std::vector<int32_t> sorted;
  rc = SortedPositions(ctx, k, count, n, true, &sorted);
  if (rc) return rc;
  ACUDA(ctx, cudaSetDevice(ctx->device));
  const size_t elem = dtype == MPSFT_C64 ? 8 : 16;
  void *dx = nullptr;
  if (cudaMalloc(&dx, size_t(n) * elem) != cudaSuccess) {
    cudaGetLastError();
    return CtxFail(ctx, MPSFT_ERR_NOMEM, "device allocation of the signal failed");
  }
  rc = [&]() -> int {
    Scratch scratch(ctx);
    DenseFft fft;
    double2 *xm = nullptr;
    int r = scratch.Take(size_t(n), &xm);
    if (r) return r;
    ACUDA(ctx, cudaMemsetAsync(xm, 0, size_t(n) * sizeof(double2), ctx->stream));
    if (count > 0) {
      int32_t *dk = nullptr;
      double2 *dc = nullptr;
      r = scratch.Take(size_t(count), &dk);
      if (r == MPSFT_OK) r = scratch.Take(size_t(count), &dc);
      if (r) return r;
      ACUDA(ctx, cudaMemcpyAsync(dk, k, sizeof(int32_t) * count,
                                 cudaMemcpyHostToDevice, ctx->stream));
      ACUDA(ctx, cudaMemcpyAsync(dc, coef, sizeof(double2) * count,
                                 cudaMemcpyHostToDevice, ctx->stream));
      k_scatter_modes<<<GridFor(count), kThreads, 0, ctx->stream>>>(dk, dc, count, xm);
      ACUDA(ctx, cudaGetLastError());
      // x_t = sum_k xh_k e^{+2 pi i k t / n}: the unnormalised backward FFT
      r = fft.Exec(ctx, n, xm, CUFFT_INVERSE);
      if (r) {
        cudaStreamSynchronize(ctx->stream);
        return r;
      }
    }
    if (dtype == MPSFT_C64) {
      k_add_noise<float2><<<GridFor(n), kThreads, 0, ctx->stream>>>(
          xm, static_cast<float2 *>(dx), n, sigma, seed);
    } else {
      k_add_noise<double2><<<GridFor(n), kThreads, 0, ctx->stream>>>(
          xm, static_cast<double2 *>(dx), n, sigma, seed);
    }
    ACUDA(ctx, cudaGetLastError());
    ACUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MPSFT_OK;
  }();
  if (rc == MPSFT_OK) {
    const cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = CtxFail(ctx, MPSFT_ERR_CUDA, cudaGetErrorString(e));
  }
  if (rc) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(dx);
    return rc;
  }
  mpsft_signal *s = new mpsft_signal;
  s->ctx = ctx;
  s->d_x = dx;
  s->n = n;
  s->dtype = dtype;
  s->owned = true;
  *out = s;
  return MPSFT_OK;
}

int mpsft_signal_spectrum(mpsft_ctx *ctx, const mpsft_signal *sig, double *out) {
  if (!ctx || !sig || !out) return CtxFail(ctx, MPSFT_ERR_INVALID, "null argument");
  if (sig->ctx != ctx) {
    return CtxFail(ctx, MPSFT_ERR_INVALID, "signal belongs to another context");
  }
  ACUDA(ctx, cudaSetDevice(ctx->device));
  Scratch scratch(ctx);
  double2 *y = nullptr;
  int rc = scratch.Take(size_t(sig->n), &y);
  if (rc) return rc;
  rc = Spectrum(ctx, sig, y);
  if (rc) return rc;
  ACUDA(ctx, cudaMemcpyAsync(out, y, size_t(sig->n) * sizeof(double2),
                             cudaMemcpyDefault, ctx->stream));
  ACUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MPSFT_OK;
}

int mpsft_post_analyze(mpsft_ctx *ctx, const mpsft_signal *sig,
                       const int32_t *true_k, int64_t true_count,
                       const int32_t *found_k, const double *found_c,
                       int64_t found_count, mpsft_analysis *out) {
  if (!ctx || !sig || !out || true_count < 0 || found_count < 0 ||
      (true_count > 0 && !true_k) || (found_count > 0 && (!found_k || !found_c))) {
    return CtxFail(ctx, MPSFT_ERR_INVALID, "null argument");
  }
  if (sig->ctx != ctx) {
    return CtxFail(ctx, MPSFT_ERR_INVALID, "signal belongs to another context");
  }
  const int64_t n = sig->n;
  std::vector<int32_t> tk, fk_sorted;
  int rc = SortedPositions(ctx, true_k, true_count, n, false, &tk);
  if (rc == MPSFT_OK) rc = SortedPositions(ctx, found_k, found_count, n, true, &fk_sorted);
  if (rc) return rc;
  ACUDA(ctx, cudaSetDevice(ctx->device));
  Scratch scratch(ctx);
  double2 *xh = nullptr, *dfc = nullptr;
  int32_t *dfk = nullptr, *dtk = nullptr, *dcounts = nullptr;
  uint32_t *bits = nullptr;
  double *partial = nullptr;
  const int64_t words = (n + 31) / 32;
  const unsigned grid = GridFor(n);
  rc = scratch.Take(size_t(n), &xh);
  if (rc == MPSFT_OK) rc = scratch.Take(size_t(words), &bits);
  if (rc == MPSFT_OK) rc = scratch.Take(size_t(found_count), &dfk);
  if (rc == MPSFT_OK) rc = scratch.Take(size_t(found_count), &dfc);
  if (rc == MPSFT_OK) rc = scratch.Take(size_t(tk.size()), &dtk);
  if (rc == MPSFT_OK) rc = scratch.Take(size_t(3) * grid + 8, &partial);
  if (rc == MPSFT_OK) rc = scratch.Take(size_t(2), &dcounts);
  if (rc) return rc;
  rc = Spectrum(ctx, sig, xh);
  if (rc) return rc;
  ACUDA(ctx, cudaMemsetAsync(bits, 0, size_t(words) * 4, ctx->stream));
  if (found_count > 0) {
    ACUDA(ctx, cudaMemcpyAsync(dfk, found_k, sizeof(int32_t) * found_count,
                               cudaMemcpyHostToDevice, ctx->stream));
    ACUDA(ctx, cudaMemcpyAsync(dfc, found_c, sizeof(double2) * found_count,
                               cudaMemcpyHostToDevice, ctx->stream));
    k_mark<<<GridFor(found_count), kThreads, 0, ctx->stream>>>(dfk, found_count, bits);
    ACUDA(ctx, cudaGetLastError());
  }
  if (!tk.empty()) {
    ACUDA(ctx, cudaMemcpyAsync(dtk, tk.data(), sizeof(int32_t) * tk.size(),
                               cudaMemcpyHostToDevice, ctx->stream));
  }
  k_unfound_err<<<grid, kThreads, 0, ctx->stream>>>(xh, bits, n, partial);
  ACUDA(ctx, cudaGetLastError());
  k_found_err<<<1, kThreads, 0, ctx->stream>>>(xh, dfk, dfc, found_count, dtk,
                                              int64_t(tk.size()), partial + 3 * grid,
                                              dcounts);
  ACUDA(ctx, cudaGetLastError());
  std::vector<double> hp(3 * grid + 8);
  int32_t counts[2] = {0, 0};
  ACUDA(ctx, cudaMemcpyAsync(hp.data(), partial, sizeof(double) * hp.size(),
                             cudaMemcpyDeviceToHost, ctx->stream));
  ACUDA(ctx, cudaMemcpyAsync(counts, dcounts, sizeof(counts), cudaMemcpyDeviceToHost,
                             ctx->stream));
  ACUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double s1 = 0.0, s2 = 0.0, mx = 0.0;
  for (unsigned b = 0; b < grid; ++b) {
    s1 += hp[3 * b];
    s2 += hp[3 * b + 1];
    mx = std::max(mx, hp[3 * b + 2]);
  }
  const double *f = hp.data() + 3 * grid;
  std::memset(out, 0, sizeof(*out));
  out->hit = counts[0];
  out->miss = counts[1];
  // the reference divides by the counts as they are (0 / 0 is NaN)
  out->hit_l1 = f[0] / double(counts[0]);
  out->hit_l2 = std::sqrt(f[1] / double(counts[0]));
  out->miss_l1 = f[2] / double(counts[1]);
  out->miss_l2 = std::sqrt(f[3] / double(counts[1]));
  out->l1 = (s1 + f[0] + f[2]) / double(n);
  out->l2 = std::sqrt((s2 + f[1] + f[3]) / double(n));
  out->max_err = std::max(mx, f[6]);
  return MPSFT_OK;
}

}  // extern "C"
