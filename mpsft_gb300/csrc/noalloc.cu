// mpsft_bin_in_time_noalloc: the binning of mpsft_bin_in_time for callers that
// cannot allocate device memory (for example code that runs inside a
// caller-managed memory pool, or a plugin host that forbids cudaMalloc after
// start-up because allocation can block or fragment the pool).
//
// All scratch lives in one file-scope __device__ array of a fixed size
// (kNoAllocScratchBytes, 2.5 MiB), which every GPU that loads this
// library holds until the process exits. The caller passes the input samples
// and the output bin matrix as device pointers and a stream; nothing here calls
// cudaMalloc, cudaFree or any allocating library routine.
//
// Host code cannot use the array's name as a device address (it names a host
// stand-in), so the first call on each device, with that device current,
// resolves the address with cudaGetSymbolAddress and fills the FFT twiddle
// table in the array; that first call synchronises its stream and should come
// before any stream capture. All calls share the array and leave their data in
// it: calls that overlap on the GPU (two streams, or two threads) race.
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/mpsft.h"
#include "launch.h"

namespace {

using namespace mpsft;

constexpr int32_t kNaMaxBins = 2047;   // Bluestein size M <= 4096
constexpr int32_t kNaMaxBits = 20;     // rows <= 41
constexpr int32_t kNaMaxRows = 1 + 2 * kNaMaxBits;
constexpr int32_t kNaMaxM = 4096;
constexpr int64_t kNaMaxP2 =
    (int64_t(kFoldLanes) * kMaxFoldsPerLane * kNaMaxBins - 1) / 2;

constexpr size_t Align256(size_t v) { return (v + 255) & ~size_t(255); }
constexpr size_t kOffIter = 0;
constexpr size_t kOffTw32 = kOffIter + Align256(sizeof(SigIter));
constexpr size_t kOffTw64 = kOffTw32 + Align256(sizeof(float2) * kMaxFFT / 2);
constexpr size_t kOffWt32 = kOffTw64 + Align256(sizeof(double2) * kMaxFFT / 2);
constexpr size_t kOffWt64 = kOffWt32 + Align256(sizeof(float) * (kNaMaxP2 + 1));
constexpr size_t kOffFold = kOffWt64 + Align256(sizeof(double) * (kNaMaxP2 + 1));
constexpr size_t kOffChirp =
    kOffFold + Align256(sizeof(double2) * size_t(kNaMaxRows) * kNaMaxBins);
constexpr size_t kOffChat = kOffChirp + Align256(sizeof(double2) * kNaMaxBins);
constexpr size_t kNoAllocScratchBytes =
    kOffChat + Align256(sizeof(double2) * kNaMaxM);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char *g_scratch_addr[kMaxDevices] = {};

// Resolves the scratch address on the current device and fills the twiddles
// (once per device).
int ScratchForCurrentDevice(cudaStream_t stream, unsigned char **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return MPSFT_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (g_scratch_addr[dev] == nullptr) {
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess ||
        ptr == nullptr) {
      cudaGetLastError();
      return MPSFT_ERR_CUDA;
    }
    unsigned char *base = static_cast<unsigned char *>(ptr);
    LaunchTwiddles(reinterpret_cast<float2 *>(base + kOffTw32),
                   reinterpret_cast<double2 *>(base + kOffTw64), stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess ||
        cudaGetLastError() != cudaSuccess) {
      return MPSFT_ERR_CUDA;
    }
    g_scratch_addr[dev] = base;
  }
  *out = g_scratch_addr[dev];
  return MPSFT_OK;
}

}  // namespace

extern "C" int mpsft_bin_in_time_noalloc(const void *x_device, int64_t n,
                                         int dtype, int32_t bins, int32_t bits,
                                         double delta, int32_t a, int32_t b,
                                         int32_t c, int32_t q, int precision,
                                         double *out_device, void *stream) {
  if (!x_device || !out_device) return MPSFT_ERR_INVALID;
  if (dtype != MPSFT_C64 && dtype != MPSFT_C128) return MPSFT_ERR_INVALID;
  if (precision != MPSFT_PREC_FP32 && precision != MPSFT_PREC_FP64) {
    return MPSFT_ERR_INVALID;
  }
  if (n < 3 || n > INT32_MAX) return MPSFT_ERR_INVALID;
  if (bins <= 0 || bins % 2 == 0 || bits < 0) return MPSFT_ERR_INVALID;
  if (!(delta > 0 && delta < 1)) return MPSFT_ERR_INVALID;
  if (bins > kNaMaxBins || bits > kNaMaxBits) return MPSFT_ERR_CAPACITY;
  if ((int64_t(bins) << (bits > 0 ? bits - 1 : 0)) > INT32_MAX) {
    return MPSFT_ERR_INVALID;
  }

  // Window scalars in the reference's operation order (src/window.cc:28-51).
  const double width = 1.0 / (2.0 * bins);
  const double sq = std::sqrt(-std::log(delta));
  const double sigma_f = 0.5 / (bins * 2.0 * M_SQRT2 * sq);
  const double sigma_t = 1.0 / ((2.0 * M_PI) * sigma_f);
  const double tmp = 2.0 * M_SQRT2 * sigma_t * sq + 1;
  int32_t folds = int32_t(std::ceil(tmp / double(bins)));
  if (folds % 2 == 0) ++folds;
  if (folds > kFoldLanes * kMaxFoldsPerLane) return MPSFT_ERR_CAPACITY;
  const int32_t p = folds * bins;
  int log2m = 0;
  while ((1 << log2m) < 2 * bins - 1) ++log2m;

  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  unsigned char *base = nullptr;
  const int rc = ScratchForCurrentDevice(st, &base);
  if (rc != MPSFT_OK) return rc;

  const bool fp64 = precision == MPSFT_PREC_FP64;
  SigIter it;
  std::memset(&it, 0, sizeof(it));
  it.x = x_device;
  it.n = int32_t(n);
  it.bins = bins;
  it.bits = bits;
  it.rows = 1 + 2 * bits;
  it.p = p;
  it.p2 = (p - 1) / 2;
  it.folds = folds;
  it.a = a;
  it.b = b;
  it.c = c;
  it.trials = 1;
  it.active = 1;
  it.q[0] = q;
  const int64_t m = (int64_t(b) * q) % n;
  const double f = double(m) / double(n) * (2.0 * M_PI);
  it.bq_re[0] = std::cos(f);
  it.bq_im[0] = std::sin(f);
  it.width = width;
  it.sigma_f = sigma_f;
  it.erf_d = M_SQRT2 * M_PI * sigma_t;
  it.fft_log2m = log2m;
  it.fft_m = 1 << log2m;
  SetFixedPoint(&it);
  it.wt32 = reinterpret_cast<float *>(base + kOffWt32);
  it.wt64 = reinterpret_cast<double *>(base + kOffWt64);
  it.fold = base + kOffFold;
  it.ubuf = reinterpret_cast<double2 *>(out_device);
  it.bins_cap = bins;
  // one region serves the FP32 or the FP64 tables (a call uses one kind)
  it.chirp32 = reinterpret_cast<float2 *>(base + kOffChirp);
  it.chat32 = reinterpret_cast<float2 *>(base + kOffChat);
  it.chirp64 = reinterpret_cast<double2 *>(base + kOffChirp);
  it.chat64 = reinterpret_cast<double2 *>(base + kOffChat);

  SigIter *d_it = reinterpret_cast<SigIter *>(base + kOffIter);
  if (cudaMemcpyAsync(d_it, &it, sizeof(it), cudaMemcpyHostToDevice, st) !=
      cudaSuccess) {
    cudaGetLastError();
    return MPSFT_ERR_CUDA;
  }
  const float2 *tw32 = reinterpret_cast<const float2 *>(base + kOffTw32);
  const double2 *tw64 = reinterpret_cast<const double2 *>(base + kOffTw64);
  if (fp64) {
    LaunchWindow(d_it, 1, it.p2, st);
  } else {
    LaunchWindow32(d_it, 1, it.p2, st);
  }
  LaunchBluesteinSetup(d_it, 1, it.fft_m, fp64, tw32, tw64, st);
  LaunchBinFold(d_it, 1, bins, bits, 1, dtype == MPSFT_C128, fp64, st);
  LaunchRowFFT(d_it, 1, it.rows, 1, it.fft_m, fp64, tw32, tw64, st);
  if (cudaGetLastError() != cudaSuccess) return MPSFT_ERR_CUDA;
  return MPSFT_OK;
}
