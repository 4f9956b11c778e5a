// Drop-in GPU binners for the reference's own code; see binner_gpu.h.
#include "binner_gpu.h"

#include <glog/logging.h>

#include <cstdlib>
#include <cstring>
#include <utility>

namespace mps {

namespace {

// The reference aborts through glog CHECKs; a failed library call does the
// same here, with the library's message.
void Check(int status, const mpsft_ctx *ctx, const char *what) {
  if (status == MPSFT_OK) return;
  LOG(FATAL) << "mpsft-gb300 " << what << ": "
             << mpsft_status_string(status) << " ("
             << (ctx ? mpsft_last_error(ctx) : "no context") << ")";
}

// Row-major (rows x cols) complex matrix <-> the reference's CplexMatrix,
// whose rows are separate arrays (src/base.h:138-151).
void MatrixToRows(const CplexMatrix &m, std::vector<double> *dst) {
  dst->resize(2 * size_t(m.rows()) * m.cols());
  for (int32_t r = 0; r < m.rows(); ++r) {
    std::memcpy(dst->data() + 2 * size_t(r) * m.cols(), m[r].data(),
                sizeof(double) * 2 * m.cols());
  }
}

void RowsToMatrix(const std::vector<double> &src, CplexMatrix *m) {
  for (int32_t r = 0; r < m->rows(); ++r) {
    std::memcpy((*m)[r].data(), src.data() + 2 * size_t(r) * m->cols(),
                sizeof(double) * 2 * m->cols());
  }
}

}  // namespace

// ---------------------------------------------------------------- session
GpuSession &GpuSession::ForThisThread() {
  static thread_local GpuSession session;
  return session;
}

mpsft_ctx *GpuSession::ctx() {
  if (!ctx_) {
    const char *dev = std::getenv("MPSFT_DEVICE");
    const int rc = mpsft_ctx_create(dev ? std::atoi(dev) : 0, &ctx_);
    if (rc != MPSFT_OK) {
      ctx_ = nullptr;
      LOG(FATAL) << "mpsft-gb300 context: " << mpsft_status_string(rc)
                 << " (is a CUDA device present?)";
    }
  }
  return ctx_;
}

const mpsft_signal *GpuSession::Upload(const CplexArray &x) {
  mpsft_ctx *c = ctx();
  if (sig_ && sig_n_ == x.size()) {
    Check(mpsft_signal_write(c, sig_, x.data()), c, "signal write");
    return sig_;
  }
  if (sig_) mpsft_signal_free(sig_);
  sig_ = nullptr;
  Check(mpsft_signal_upload(c, x.data(), x.size(), MPSFT_C128, &sig_), c,
        "signal upload");
  sig_n_ = x.size();
  return sig_;
}

GpuSession::~GpuSession() {
  if (sig_) mpsft_signal_free(sig_);
  if (ctx_) mpsft_ctx_destroy(ctx_);
}

// ------------------------------------------------------------- BinInTime
BinInTimeGPU::BinInTimeGPU(const Window &win, int32_t bits)
    : BinInTime(win, bits) {}

void BinInTimeGPU::Run(const CplexArray &x, const Transform &tf, int32_t q,
                       CplexMatrix *out) {
  CHECK_EQ(out->rows(), 1 + 2 * bits_);
  CHECK_EQ(out->cols(), win_.bins());
  GpuSession &s = GpuSession::ForThisThread();
  const mpsft_signal *sig = s.Upload(x);
  rows_.resize(2 * size_t(out->rows()) * out->cols());
  Check(mpsft_bin_in_time_wt(s.ctx(), sig, win_.bins(), bits_, win_.p(),
                             win_.wt(), tf.a, tf.b, tf.c, q, s.precision(),
                             rows_.data(), 0),
        s.ctx(), "BinInTime");
  RowsToMatrix(rows_, out);
}

// ------------------------------------------------------------- BinInFreq
BinInFreqGPU::BinInFreqGPU(const Window &win, int32_t bits)
    : BinInFreq(win, bits) {}

void BinInFreqGPU::Run(const ModeMap &mm, const Transform &tf, int32_t q,
                       CplexMatrix *out) {
  CHECK_EQ(out->rows(), 1 + 2 * bits_);
  const int32_t bins = win_.bins();
  const int32_t n = win_.n();
  k0_.clear();
  coef_.clear();
  wf_.clear();
  for (const auto &kv : mm) {
    // the mode's bin and offset in it, as BinInFreqV1 forms them
    // (src/binner.cc:571-575), then the binner's own window response
    const int32_t k1 = MulAddPosMod(tf.a, kv.first, tf.b, n);
    const int32_t bin = int32_t(int64_t(k1) * int64_t(bins) / int64_t(n));
    const double xi = (double(bin) + 0.5) / double(bins) - double(k1) / double(n);
    k0_.push_back(kv.first);
    coef_.push_back(RE(kv.second));
    coef_.push_back(IM(kv.second));
    wf_.push_back(win_.SampleInFreq(xi));
  }
  MatrixToRows(*out, &rows_);
  GpuSession &s = GpuSession::ForThisThread();
  Check(mpsft_bin_in_freq_wf(s.ctx(), n, bins, bits_, tf.a, tf.b, tf.c, q,
                             k0_.data(), coef_.data(), wf_.data(),
                             int64_t(k0_.size()), rows_.data()),
        s.ctx(), "BinInFreq");
  RowsToMatrix(rows_, out);
}

// --------------------------------------------------------------- Iterate
bool IterateGPU(const CplexArray &x, const IterateOptions &opt, ModeMap *mm) {
  const int32_t n = x.size();
  // Iterate's draws, in its order: the Window and NumBits draw nothing, then
  // Transform(n) (a, b, c), then one q per trial (src/iterate.cc:89-104)
  const Transform tf(n);
  std::vector<int32_t> q(opt.trials > 0 ? opt.trials : 1);
  for (int32_t t = 0; t < opt.trials; ++t) q[t] = RandomInt32() % n;

  std::vector<int32_t> k(mm->size() + size_t(opt.bins) + 16);
  std::vector<double> c(2 * k.size());
  int32_t size = 0;
  for (const auto &kv : *mm) {
    k[size] = kv.first;
    c[2 * size] = RE(kv.second);
    c[2 * size + 1] = IM(kv.second);
    ++size;
  }
  mpsft_iterate_options o;
  std::memset(&o, 0, sizeof(o));
  o.bins = opt.bins;
  o.window_delta = opt.window_delta;
  o.trials = opt.trials;
  o.bin_threshold = opt.bin_threshold;
  o.window_threshold = opt.window_threshold;
  o.sv_threshold = opt.sv_threshold;
  GpuSession &s = GpuSession::ForThisThread();
  o.precision = s.precision();
  const mpsft_signal *sig = s.Upload(x);
  int32_t found = 0;
  Check(mpsft_iterate_draws(s.ctx(), sig, &o, tf.a, tf.b, tf.c, tf.a_inv,
                            q.data(), k.data(), c.data(), &size,
                            int32_t(k.size()), &found),
        s.ctx(), "Iterate");
  mm->clear();
  for (int32_t i = 0; i < size; ++i) {
    (*mm)[k[i]] = Cplex(c[2 * i], c[2 * i + 1]);
  }
  return found != 0;
}

}  // namespace mps
