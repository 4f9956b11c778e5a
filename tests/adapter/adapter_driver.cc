// Example caller of the GPU binners through the reference's own factory and
// Iterate (test harness of the adapter build). Without arguments it checks
// that the patched factories return the GPU binners; "bin" runs the
// known-answer binning case of src/binner_test.cc:54-75 through
// BinInTime::Create(kBinInTimeGPU, ...); "iterate" runs Iterate with both GPU
// binner types and IterateGPU on a two-mode signal.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>

#include "binner_gpu.h"
#include "iterate.h"
#include "sincos.h"

using namespace mps;

int main(int argc, char **argv) {
  MainInit(argc, argv);
  const int32_t n = 1109, bins = 5, bits = 2;
  Window win(n, bins, 1e-6);
  std::unique_ptr<BinInTime> bt(BinInTime::Create(kBinInTimeGPU, win, bits));
  std::unique_ptr<BinInFreq> bf(BinInFreq::Create(kBinInFreqGPU, win, bits));
  if (!dynamic_cast<BinInTimeGPU *>(bt.get()) ||
      !dynamic_cast<BinInFreqGPU *>(bf.get())) {
    std::printf("factory did not return the GPU binners\n");
    return 2;
  }
  std::printf("factory: BinInTimeGPU, BinInFreqGPU\n");
  if (argc < 2) return 0;

  // one mode {550: 2}, as src/binner_test.cc:57-70
  CplexArray x(n);
  for (int32_t t = 0; t < n; ++t) {
    x[t] = 2.0 * Sinusoid(double(MulMod(550, t, n)) / double(n));
  }
  if (std::strcmp(argv[1], "bin") == 0) {
    Transform tf(n, 3, 847, 45);
    CplexMatrix out(1 + 2 * bits, bins);
    bt->Run(x, tf, 106, &out);
    std::printf("bin 0,1: %.6f %.6f\n", RE(out[0][1]), IM(out[0][1]));
    ModeMap mm;
    mm[550] = Cplex(2.0, 0.0);
    bf->Run(mm, tf, 106, &out);
    double mx = 0;
    for (int32_t r = 0; r < out.rows(); ++r) {
      for (int32_t b = 0; b < bins; ++b) mx = std::max(mx, std::abs(out[r][b]));
    }
    std::printf("time + freq max: %.3e\n", mx);
    return 0;
  }
  if (std::strcmp(argv[1], "iterate") == 0) {
    IterateOptions opt;
    opt.bins = 11;
    opt.trials = 5;
    opt.window_threshold = 0.1;
    opt.bin_in_time_type = kBinInTimeGPU;
    opt.bin_in_freq_type = kBinInFreqGPU;
    ModeMap mm, mm_gpu;
    RandomSeed(3);
    Iterate(x, opt, &mm);
    RandomSeed(3);
    IterateGPU(x, opt, &mm_gpu);
    std::printf("iterate: %zu modes (factory binners), %zu modes (IterateGPU)\n",
                mm.size(), mm_gpu.size());
    return 0;
  }
  return 1;
}
