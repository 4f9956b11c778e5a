// mpsft_bin_in_time_noalloc: the binning of mpsft_bin_in_time for callers that
// cannot allocate device memory (for example code that runs inside a
// caller-managed memory pool, or a plugin host that forbids cudaMalloc after
// start-up because allocation can block or fragment the pool).
//
// All scratch lives in one file-scope __device__ array of a fixed size
// (kNoAllocScratchBytes, 2.5 MiB), which every GPU that loads this
// library holds until the process exits. The caller passes the input samples
// and the output bin matrix as device pointers and a stream; nothing here calls
// cudaMalloc, cudaFree or any allocating library routine, and nothing is
// copied from host memory: the call's descriptor travels as a kernel
// argument.
//
// Host code cannot use the array's name as a device address (it names a host
// stand-in), so every call, with the caller's device current, resolves the
// address with cudaGetSymbolAddress (a lookup, no allocation; a context reset
// reloads the module, possibly elsewhere). The FFT twiddle table inside the
// array is filled on the device by the first call after the module is loaded:
// a word in the array records that it is in place, and a reloaded module
// starts with that word clear. All calls share the array and leave their data
// in it: calls that overlap on the GPU (two streams, or two threads) race.
#include <cstring>

#include "../../include/mpsft.h"
#include "internal.h"
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
constexpr size_t kOffReady = 0;
constexpr size_t kOffIter = kOffReady + 256;
constexpr size_t kOffTw32 = kOffIter + Align256(sizeof(SigIter));
constexpr size_t kOffTw64 = kOffTw32 + Align256(sizeof(float2) * kTwiddleEntries);
constexpr size_t kOffWt32 = kOffTw64 + Align256(sizeof(double2) * kTwiddleEntries);
constexpr size_t kOffWt64 = kOffWt32 + Align256(sizeof(float) * (kNaMaxP2 + 1));
constexpr size_t kOffFold = kOffWt64 + Align256(sizeof(double) * (kNaMaxP2 + 1));
constexpr size_t kOffChirp =
    kOffFold + Align256(sizeof(double2) * size_t(kNaMaxRows) * kNaMaxBins);
constexpr size_t kOffChat = kOffChirp + Align256(sizeof(double2) * kNaMaxBins);
constexpr size_t kNoAllocScratchBytes =
    kOffChat + Align256(sizeof(double2) * kNaMaxM);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// value of the ready word once the twiddles are in the array
constexpr uint32_t kTwiddlesReady = 0x54574431u;

// Stores the call's descriptor (a kernel argument, so nothing is copied from
// host memory) and, when the ready word is clear, fills the twiddle table and
// then sets the word. One block: every thread has finished its share of the
// table before the word is set, and later kernels of the call, ordered after
// this one on the stream, see the whole table.
__global__ void __launch_bounds__(1024)
    k_noalloc_setup(SigIter it, SigIter *dst, float2 *tw32, double2 *tw64,
                    uint32_t *ready) {
  if (threadIdx.x == 0) *dst = it;
  if (*(volatile uint32_t *)ready == kTwiddlesReady) return;
  for (int e = threadIdx.x; e < kTwiddleEntries; e += blockDim.x) {
    TwiddleAt(e, tw32, tw64);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) *(volatile uint32_t *)ready = kTwiddlesReady;
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

  // the same lengths as mpsft_bin_in_time (the permutation needs an
  // invertible a: prime or power-of-two n)
  if (!SupportedN(n)) return MPSFT_ERR_UNSUPPORTED_N;
  const WinParams w = MakeWindow(bins, delta);
  if (w.folds > kFoldLanes * kMaxFoldsPerLane) return MPSFT_ERR_CAPACITY;

  void *ptr = nullptr;
  if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess ||
      ptr == nullptr) {
    cudaGetLastError();
    return MPSFT_ERR_CUDA;
  }
  unsigned char *base = static_cast<unsigned char *>(ptr);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

  // the descriptor mpsft_bin_in_time builds, over the caller's buffers and
  // the array
  const bool fp64 = precision == MPSFT_PREC_FP64;
  mpsft_signal sig;
  sig.d_x = const_cast<void *>(x_device);
  sig.n = n;
  sig.dtype = dtype;
  const Transform tf{a, b, c, InverseMod(a, n)};
  SigIter it;
  std::memset(&it, 0, sizeof(it));
  FillIter(&it, &sig, bins, bits, delta, tf, &q, 1);
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
  float2 *tw32 = reinterpret_cast<float2 *>(base + kOffTw32);
  double2 *tw64 = reinterpret_cast<double2 *>(base + kOffTw64);
  k_noalloc_setup<<<1, 1024, 0, st>>>(it, d_it, tw32, tw64,
                                      reinterpret_cast<uint32_t *>(base + kOffReady));
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
