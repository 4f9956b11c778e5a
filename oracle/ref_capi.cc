// C wrapper around the reference's own classes (jiaweichiu/mpsft src/*.cc,
// compiled unmodified from the reference tree by oracle/Makefile into
// oracle/_ref/). Test infrastructure only: it lets the tests run the reference
// itself on the same inputs as this project's oracle restatement and the CUDA
// path. Implements oracle_capi.h.
#include <algorithm>
#include <cstring>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "base.h"
#include "binner.h"
#include "freqid.h"
#include "gen.h"
#include "integer.h"
#include "iterate.h"
#include "window.h"

// Demo1 keeps the signal private; open it up so that Demo1::Run itself can be
// run on the caller's signal. Every header it needs is already included above.
#define private public
#include "demo1.h"
#undef private

#include "oracle_capi.h"

using namespace mps;

namespace {

void CopyIn(const double *x, CplexArray *a) {
  std::memcpy(reinterpret_cast<void *>(a->data()), x,
              sizeof(double) * 2 * a->size());
}

void CopyMatrixIn(const double *src, CplexMatrix *m) {
  for (int32_t r = 0; r < m->rows(); ++r) {
    std::memcpy(reinterpret_cast<void *>((*m)[r].data()),
                src + 2 * int64_t(r) * m->cols(),
                sizeof(double) * 2 * m->cols());
  }
}

void CopyMatrixOut(const CplexMatrix &m, double *dst) {
  for (int32_t r = 0; r < m.rows(); ++r) {
    std::memcpy(dst + 2 * int64_t(r) * m.cols(),
                reinterpret_cast<const void *>(m[r].data()),
                sizeof(double) * 2 * m.cols());
  }
}

int WriteSorted(const ModeMap &mm, int32_t *out_k, double *out_c,
                int32_t cap) {
  std::vector<std::pair<int32_t, Cplex>> v(mm.begin(), mm.end());
  std::sort(v.begin(), v.end(),
            [](const std::pair<int32_t, Cplex> &l,
               const std::pair<int32_t, Cplex> &r) { return l.first < r.first; });
  if (int64_t(v.size()) > cap) {
    return -1;
  }
  for (size_t i = 0; i < v.size(); ++i) {
    out_k[i] = v[i].first;
    out_c[2 * i] = RE(v[i].second);
    out_c[2 * i + 1] = IM(v[i].second);
  }
  return int(v.size());
}

} // namespace

extern "C" {

void orc_seed(int32_t seed) { RandomSeed(seed); }
int32_t orc_random_int32(void) { return RandomInt32(); }
double orc_random_normal(void) { return RandomNormal(); }

int32_t orc_num_bits(int32_t n, int32_t bins) {
  // NumBits is file-local in src/iterate.cc; its definition is one loop:
  // count halvings of n while n >= bins, at least 1 (src/iterate.cc:30-42).
  if (n < bins) return 1;
  int32_t out = 0;
  while (n >= bins) {
    n >>= 1;
    ++out;
  }
  return out;
}

int32_t orc_window(int32_t n, int32_t bins, double delta, double *wt,
                   int32_t cap) {
  Window win(n, bins, delta);
  if (wt != nullptr && cap >= win.p()) {
    std::memcpy(wt, win.wt(), sizeof(double) * win.p());
  }
  return win.p();
}

double orc_window_sample_in_freq(int32_t n, int32_t bins, double delta,
                                 double xi) {
  Window win(n, bins, delta);
  return win.SampleInFreq(xi);
}

void orc_transform(int32_t n, int32_t *out) {
  Transform tf(n);
  out[0] = tf.a;
  out[1] = tf.b;
  out[2] = tf.c;
  out[3] = tf.a_inv;
}

int32_t orc_transform_inverse(int32_t n, int32_t a) {
  Transform tf(n, a, 0, 0);
  return tf.a_inv;
}

int orc_bin_in_time(int type, int32_t n, int32_t bins, int32_t bits,
                    double delta, int32_t a, int32_t b, int32_t c, int32_t q,
                    const double *x, double *out) {
  Window win(n, bins, delta);
  Transform tf(n, a, b, c);
  CplexArray xa(n);
  CopyIn(x, &xa);
  CplexMatrix m(1 + 2 * bits, bins);
  std::unique_ptr<BinInTime> bt(BinInTime::Create(type, win, bits));
  bt->Run(xa, tf, q, &m);
  CopyMatrixOut(m, out);
  return 0;
}

int orc_bin_in_freq(int type, int32_t n, int32_t bins, int32_t bits,
                    double delta, int32_t a, int32_t b, int32_t c, int32_t q,
                    const int32_t *k0, const double *coef, int32_t mcount,
                    double *out) {
  Window win(n, bins, delta);
  Transform tf(n, a, b, c);
  ModeMap mm;
  for (int32_t i = 0; i < mcount; ++i) {
    mm[k0[i]] = Cplex(coef[2 * i], coef[2 * i + 1]);
  }
  CplexMatrix m(1 + 2 * bits, bins);
  CopyMatrixIn(out, &m);
  std::unique_ptr<BinInFreq> bf(BinInFreq::Create(type, win, bits));
  bf->Run(mm, tf, q, &m);
  CopyMatrixOut(m, out);
  return 0;
}

int orc_mat_pencil(const double *u, double *sigma) {
  return MatPencil(Cplex(u[0], u[1]), Cplex(u[2], u[3]), Cplex(u[4], u[5]),
                   sigma)
             ? 1
             : 0;
}

int orc_iterate(int32_t n, const double *x, int32_t bins, double window_delta,
                int32_t trials, double bin_threshold, double window_threshold,
                double sv_threshold, int bin_in_time_type,
                int bin_in_freq_type, int32_t *mm_k, double *mm_c,
                int32_t *mm_size, int32_t mm_cap) {
  CplexArray xa(n);
  CopyIn(x, &xa);
  IterateOptions opt;
  opt.bins = bins;
  opt.window_delta = window_delta;
  opt.trials = trials;
  opt.bin_threshold = bin_threshold;
  opt.window_threshold = window_threshold;
  opt.sv_threshold = sv_threshold;
  opt.bin_in_time_type = bin_in_time_type;
  opt.bin_in_freq_type = bin_in_freq_type;
  ModeMap mm;
  for (int32_t i = 0; i < *mm_size; ++i) {
    mm[mm_k[i]] = Cplex(mm_c[2 * i], mm_c[2 * i + 1]);
  }
  const bool found = Iterate(xa, opt, &mm);
  const int cnt = WriteSorted(mm, mm_k, mm_c, mm_cap);
  if (cnt < 0) return -1;
  *mm_size = cnt;
  return found ? 1 : 0;
}

int orc_demo1_run(int32_t n, const double *x, int32_t k, double sigma,
                  int32_t trials, int32_t min_bins, double window_delta,
                  double window_threshold, int32_t max_stale_iter,
                  int32_t seed, int32_t *out_k, double *out_c, int32_t cap,
                  int32_t *iters) {
  Demo1Options opt;
  opt.trials = trials;
  opt.min_bins = min_bins;
  opt.window_delta = window_delta;
  opt.window_threshold = window_threshold;
  opt.max_stale_iter = max_stale_iter;
  // The constructor synthesises its own signal (here of length 1 with no
  // modes, which consumes two normal draws); the caller's signal replaces it
  // and the RNG is seeded after construction, right before Demo1::Run.
  Demo1 demo(opt, 1, 0, sigma);
  demo.k_ = k;
  demo.x_.resize(n);
  CopyIn(x, &demo.x_);
  RandomSeed(seed);
  demo.Run();
  if (iters) *iters = -1;
  return WriteSorted(demo.found_mm_, out_k, out_c, cap);
}

int orc_generate_mode_map(int32_t n, int32_t k, int32_t *out_k, double *out_c) {
  ModeMap mm;
  GenerateModeMap(n, k, &mm);
  return WriteSorted(mm, out_k, out_c, k);
}

int orc_demo_signal(int32_t n, int32_t k, double sigma, int xhat_kind,
                    double *x, int32_t *out_k, double *out_c) {
  ModeMap mm;
  GenerateModeMap(n, k, &mm);
  CplexArray xh(n);
  if (xhat_kind == 0) {
    GenerateXhat(n, mm, sigma, &xh);
  } else {
    GenerateXhatAlt(n, mm, sigma, &xh);
  }
  CplexArray xt(n);
  FFTPlan plan(n, FFTW_BACKWARD);
  plan.Run(xh, &xt);
  std::memcpy(x, reinterpret_cast<const void *>(xt.data()), sizeof(double) * 2 * n);
  return WriteSorted(mm, out_k, out_c, k);
}

void orc_post_analyze(int32_t n, const double *xh, const int32_t *true_k,
                      int32_t true_count, const int32_t *found_k,
                      const double *found_c, int32_t found_count, double *out) {
  // Demo1::PostAnalyze itself on a Demo1 whose spectrum, true map and found
  // map are the caller's (the constructor's own length-1 signal is replaced).
  static Demo1Options opt;
  Demo1 demo(opt, 1, 0, 1.0);
  demo.x_.resize(n);
  demo.xh_.resize(n);
  CopyIn(xh, &demo.xh_);
  demo.mm_.clear();
  for (int32_t i = 0; i < true_count; ++i) demo.mm_[true_k[i]] = Cplex(1.0, 0.0);
  demo.found_mm_.clear();
  for (int32_t i = 0; i < found_count; ++i) {
    demo.found_mm_[found_k[i]] = Cplex(found_c[2 * i], found_c[2 * i + 1]);
  }
  std::ostringstream os;
  os.precision(17);
  demo.PostAnalyze(os);
  std::istringstream is(os.str());
  for (int i = 0; i < 9; ++i) {
    std::string tok;
    is >> tok;
    out[i] = std::strtod(tok.c_str(), nullptr);
  }
}

} // extern "C"
