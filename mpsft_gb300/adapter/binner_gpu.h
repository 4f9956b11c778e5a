// Drop-in GPU binners for the reference's own code (jiaweichiu/mpsft).
//
// BinInTimeGPU and BinInFreqGPU are BinInTime / BinInFreq implementations
// (src/binner.h:30-41, src/binner.h:123-133) that run on a GB300 through the
// mpsft-gb300 C ABI (include/mpsft.h). With the factory patch beside this file
// (binner_factory.patch) applied to src/binner.cc, IterateOptions'
// bin_in_time_type = kBinInTimeGPU and bin_in_freq_type = kBinInFreqGPU
// (src/iterate.h:57-58) make the reference's own Iterate bin on the GPU, with
// no other change. IterateGPU has Iterate's signature (src/iterate.h:65) and
// runs the whole iteration (binning, subtraction, identification, estimation)
// on the GPU, drawing the transform and the q's from the reference's global
// RNG in Iterate's order.
//
// Compile this file with the reference's headers on the include path and
// link libmpsft_gb300.so. It is not part of the library: it needs the
// reference's classes.
#pragma once

#include <cstdint>
#include <vector>

#include "base.h"
#include "binner.h"
#include "integer.h"
#include "iterate.h"
#include "window.h"

#include "mpsft.h"

namespace mps {

// Factory type numbers of the GPU binners (BinInTime::Create and
// BinInFreq::Create, src/binner.cc:58-76, src/binner.cc:526-535).
constexpr int kBinInTimeGPU = 5;
constexpr int kBinInFreqGPU = 2;

// The library's context and a device copy of the signal, one per host thread
// (a context is used by one thread at a time, as the reference's binners
// are), kept across binner objects and Iterate calls: Iterate builds new
// binners on every call (src/iterate.cc:93-96), and a context per binner
// would pay for its creation and its work buffers every time.
class GpuSession {
 public:
  // The calling thread's session; the context is created on first use on
  // device MPSFT_DEVICE (default 0).
  static GpuSession &ForThisThread();

  mpsft_ctx *ctx();
  // The device copy of x, refreshed from x on every call (x is host memory
  // the caller may have changed since the last call).
  const mpsft_signal *Upload(const CplexArray &x);

  // Precision of the GPU binning: MPSFT_PREC_FP64 (default; the reference
  // computes in FP64) or MPSFT_PREC_FP32.
  int precision() const { return precision_; }
  void set_precision(int p) { precision_ = p; }

  ~GpuSession();

 private:
  GpuSession() = default;
  mpsft_ctx *ctx_ = nullptr;
  mpsft_signal *sig_ = nullptr;
  int64_t sig_n_ = 0;
  int precision_ = MPSFT_PREC_FP64;
};

// BinInTime::Run on the GPU, windowed by the binner's own Window table
// (Window::wt(), src/window.h:32), so that the window is the reference's bit
// for bit whatever delta built it.
class BinInTimeGPU : public BinInTime {
 public:
  BinInTimeGPU(const Window &win, int32_t bits);
  void Run(const CplexArray &x, const Transform &tf, int32_t q,
           CplexMatrix *out) override;

 private:
  std::vector<double> rows_;  // host staging: (1 + 2 bits) x bins complex
};

// BinInFreq::Run on the GPU: each mode's window response is the binner's own
// Window::SampleInFreq (src/window.cc:77-81), evaluated here per mode; the
// per-row subtraction runs on the device.
class BinInFreqGPU : public BinInFreq {
 public:
  BinInFreqGPU(const Window &win, int32_t bits);
  void Run(const ModeMap &mm, const Transform &tf, int32_t q,
           CplexMatrix *out) override;

 private:
  std::vector<double> rows_;
  std::vector<int32_t> k0_;
  std::vector<double> coef_, wf_;
};

// Iterate (src/iterate.cc:80-176) with every step on the GPU. Draws
// Transform(n) and then one q per trial from the global RNG, as Iterate does
// (src/iterate.cc:92-104), so the RNG ends where Iterate would leave it.
bool IterateGPU(const CplexArray &x, const IterateOptions &opt, ModeMap *mm);

}  // namespace mps
