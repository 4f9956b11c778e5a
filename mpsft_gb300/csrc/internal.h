// Definitions of the C ABI's opaque types, shared by the library's host
// translation units (engine.cu: solves and bins; analysis.cu: signal
// generation, dense spectra, result analysis).
#pragma once

#include <cuda_runtime.h>

#include <condition_variable>
#include <cstdint>
#include <functional>
#include <memory>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mpsft.h"
#include "common.cuh"

// A few host threads that run the parts of a call's host work that are
// independent per signal (the solve graph's draw tables) beside the calling
// thread. Run(n, fn) calls fn(0) .. fn(n - 1), each once, on the workers and
// the caller, and returns when all are done.
class HostPool {
 public:
  explicit HostPool(int workers) {
    for (int w = 0; w < workers; ++w) threads_.emplace_back([this] { Work(); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lock(mu_);
      stop_ = true;
    }
    wake_.notify_all();
    for (std::thread &t : threads_) t.join();
  }
  void Run(int n, const std::function<void(int)> &fn) {
    {
      std::lock_guard<std::mutex> lock(mu_);
      fn_ = &fn;
      n_ = n;
      next_ = 0;
      left_ = n;
      ++gen_;
    }
    wake_.notify_all();
    Drain();
    std::unique_lock<std::mutex> lock(mu_);
    done_.wait(lock, [this] { return left_ == 0; });
    fn_ = nullptr;
  }

 private:
  void Drain() {
    for (;;) {
      int i;
      const std::function<void(int)> *fn;
      {
        std::lock_guard<std::mutex> lock(mu_);
        if (fn_ == nullptr || next_ >= n_) return;
        i = next_++;
        fn = fn_;
      }
      (*fn)(i);
      std::lock_guard<std::mutex> lock(mu_);
      if (--left_ == 0) done_.notify_all();
    }
  }
  void Work() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lock(mu_);
        wake_.wait(lock, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
      }
      Drain();
    }
  }
  std::vector<std::thread> threads_;
  std::mutex mu_;
  std::condition_variable wake_, done_;
  const std::function<void(int)> *fn_ = nullptr;
  int n_ = 0, next_ = 0, left_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

struct mpsft_ctx {
  int device = 0;
  std::unique_ptr<HostPool> pool;  // made at the first large batched solve
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  // second stream, at the highest priority, for the kernels of an iteration
  // that do not depend on the gather/fold (tables, mode preparation and
  // bucketing): their few blocks go ahead of the fold's many, so that the
  // FFT and the decisions do not wait for them
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaEvent_t ev_blue = nullptr;  // Bluestein tables (the row FFT waits for them)
  // third stream, at the lowest priority, for the FP64 window tables (only
  // the near-tie re-binning and the FP64 kernels use them): FP64
  // transcendentals, slow on this part, that fill SMs the fold leaves idle
  cudaStream_t side64 = nullptr;
  cudaEvent_t ev_join64 = nullptr;
  cudaEvent_t ev_fork_l = nullptr, ev_join_l = nullptr;  // listed-bin terms
  cudaEvent_t ev_join_m = nullptr;  // merge of the bins not listed
  // fourth stream, at the lowest priority: in the fixed-bins phase, the plan
  // and gather/fold of the next iteration while the current one decides
  cudaStream_t pre = nullptr;
  cudaEvent_t ev_plan_p = nullptr, ev_join_p = nullptr;
  cudaEvent_t ev_loop0 = nullptr, ev_loop1 = nullptr;  // timing of the loop
  // stream the solve graph is captured on, and the last instantiated graph
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<int64_t> graph_key;
  // device solve state and draw tables of the current call (in the arena)
  mpsft::SolveCtl *d_solve_ctl = nullptr;
  int32_t *d_draws = nullptr;
  double *d_draw_bq = nullptr;
  int64_t graph_body_kernels = 0;
  bool graph_unavailable = false;
  std::string err;
  bool profiling = false;
  float2 *tw32 = nullptr;
  double2 *tw64 = nullptr;
  // grow-only device arena reused across calls
  unsigned char *arena = nullptr;
  size_t arena_size = 0;
  // pinned host staging for per-iteration control words
  int32_t *h_ctl = nullptr;
  size_t h_ctl_n = 0;
  // pinned staging of exported mode tables
  unsigned char *h_stage = nullptr;  // pinned: a call's results
  size_t res_est = 0;  // table entries the last solve call exported
  // pinned, device-mapped staging of a solve's small uploads (copied by a
  // kernel, see Upload), its device address and the bump offset
  unsigned char *h_up = nullptr, *d_up = nullptr;
  size_t h_up_n = 0, up_off = 0;
  int64_t up_launches = 0;  // copy kernels Upload launched in this call
  size_t h_stage_n = 0;
  std::vector<cudaEvent_t> events;
  // binning launches of the last call made with profiling on
  std::vector<mpsft_bin_launch> bin_launches;
  // launch shapes of the FP32 fold chosen by the autotuner, per key (bins,
  // signal length and batch size classes: ceil(log2); complex128 input);
  // force_shape >= 0 overrides the table (tuning runs, tests)
  struct TuneEntry {
    int32_t bins_log2, n_log2, nsig_log2, c128, shape;
    float us;
  };
  std::vector<TuneEntry> tuning;
  // device clock at the end of every iteration body of the last solve graph
  // (mpsft_ctx_set_timeline)
  bool timeline_on = false;
  std::vector<unsigned long long> timeline;  // (kernel id, clock) pairs
  unsigned long long *trace = nullptr;       // the current solve's buffer
  uint32_t *trace_count = nullptr;
  int32_t force_shape = -1;
  int64_t tuning_version = 0;
  // table cache of FP32 solves: window tables (FP32, FP64, float-float) and
  // FP32 Bluestein tables per odd number of bins for one window delta, built
  // on first use and kept, like FFT plans (win_dev: block offsets, valid and
  // claim words, then the pool)
  unsigned char *win_dev = nullptr;
  // FP64 unit-phase tables (ph_lo, then ph_hi) of one signal length, kept
  // for the next calls of that length
  double2 *ph_cache = nullptr;
  int64_t ph_cache_n = 0;
  size_t win_bytes = 0;
  double win_delta = 0.0;
  int32_t win_bmin = 0, win_bmax = 0;
};

struct mpsft_signal {
  mpsft_ctx *ctx = nullptr;
  void *d_x = nullptr;
  int64_t n = 0;
  int dtype = MPSFT_C64;
  bool owned = false;
};

// The reference's global RNG state (src/base.cc:32-56) made explicit: one
// engine shared by its integer and normal distributions.
struct mpsft_rng {
  std::mt19937 eng;
  std::uniform_int_distribution<int32_t> uid;
  std::normal_distribution<double> nd;
  // integer draws that a batched solve took from a copy of this generator
  // and that it has not taken itself yet: taken before its next draw (a
  // reseed drops them)
  int64_t pending = 0;
  // a reseed is applied to the engine at its next use (seeding fills the
  // engine's whole state): a batched solve's working copies then seed
  // themselves on the host threads that fill the draw tables, side by side
  bool seed_pending = false;
  int32_t seed_value = 0;
  void CatchUp() {
    if (seed_pending) {
      eng.seed(seed_value);
      seed_pending = false;
    }
    for (; pending > 0; --pending) uid(eng);
  }
  int32_t Draw() {
    CatchUp();
    return uid(eng);
  }
  double Normal() {
    CatchUp();
    return nd(eng);
  }
  void Seed(int32_t seed) {
    seed_pending = true;
    seed_value = seed;
    pending = 0;
  }
};

namespace mpsft {

// Records msg as the context's last error and returns code.
int CtxFail(mpsft_ctx *ctx, int code, const std::string &msg);

// ---- integer and window helpers (engine.cu) ----
bool IsPow2(int64_t n);
// Deterministic Miller-Rabin, exact for n < 3.2e9.
bool IsPrime(int64_t n);
// A length the solver supports: prime or a power of two in [3, 2^31 - 1].
bool SupportedN(int64_t n);
// a^{-1} mod m by the extended Euclidean algorithm; 0 if not invertible.
int32_t InverseMod(int64_t a, int64_t m);
// NumBits (src/iterate.cc:30-42).
int32_t NumBits(int32_t n, int32_t bins);
// Window scalars, in the reference's operation order (src/window.cc:28-51).
struct WinParams {
  int32_t p = 0, p2 = 0, folds = 0;
  double width = 0, sigma_f = 0, sigma_t = 0, erf_d = 0;
};
WinParams MakeWindow(int32_t bins, double delta);
// log2 of the Bluestein transform size M (the power of two >= 2 bins - 1).
int FFTLog2(int32_t bins);
// The transform of one Iterate call (src/integer.h:68-82).
struct Transform {
  int32_t a, b, c, a_inv;
};
// e^{2 pi i (b q mod n)/n} (re, im) as the reference's
// Sinusoid(MulMod(b, q, n) / n).
void RowPhase(int32_t b, int32_t q, int32_t n, double *re, double *im);
// The per-iteration scalars of it (everything but its buffers) for one
// signal, bins, bits, window delta, transform and trials q's.
void FillIter(SigIter *it, const mpsft_signal *sig, int32_t bins, int32_t bits,
              double delta, const Transform &tf, const int32_t *q,
              int32_t trials);
// The same with the window's scalars given.
void FillIter(SigIter *it, const mpsft_signal *sig, int32_t bins, int32_t bits,
              const WinParams &w, const Transform &tf, const int32_t *q,
              int32_t trials);
// MPSFT_OK when n is a length the solver supports (prime or a power of two in
// [3, 2^31 - 1]); otherwise records why.
int CtxCheckN(mpsft_ctx *ctx, int64_t n);

}  // namespace mpsft
