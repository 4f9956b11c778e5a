// FP64 discrete Fourier transform of any length, written for the oracle.
// Test infrastructure only: it backs the fftw3 stand-in that the reference's
// sources are compiled against, and the oracle's own restatement of the
// reference's size-B FFT (`FFTPlan::Run`, src/base.cc:86-97, which calls FFTW's
// unnormalised `fftw_execute_dft`). Both use this file, so they agree bit for
// bit.
//
// Definition (unnormalised, like FFTW):
//   out[k] = sum_j in[j] * exp(sign * 2*pi*i * j*k / n),  sign = -1 forward.
//
// Algorithm: recursive mixed-radix decimation in time over the prime factors
// of n (generic radix-p butterflies, O(n * sum of factors)); when a prime factor
// exceeds kMaxDirectRadix, Bluestein's chirp-z method over a power-of-two
// transform. Every twiddle exp(sign*2*pi*i*m/n) is evaluated from the exact
// integer m mod n.
#pragma once

#include <cmath>
#include <complex>
#include <cstdint>
#include <memory>
#include <vector>

namespace fft64 {

using cd = std::complex<double>;

constexpr int kMaxDirectRadix = 4099;

inline cd Twiddle(int64_t m, int64_t n, int sign) {
  m %= n;
  if (m < 0) m += n;
  const double ang = 2.0 * M_PI * double(m) / double(n);
  return cd(std::cos(ang), sign * std::sin(ang));
}

inline std::vector<int> Factor(int n) {
  std::vector<int> f;
  for (int p = 2; (int64_t)p * p <= n; ++p) {
    while (n % p == 0) {
      f.push_back(p);
      n /= p;
    }
  }
  if (n > 1) f.push_back(n);
  return f;
}

class Plan {
public:
  Plan(int n, int sign) : n_(n), sign_(sign) {
    if (n_ <= 0) return;
    fac_ = Factor(n_);
    int maxp = 1;
    for (int p : fac_) maxp = p > maxp ? p : maxp;
    bluestein_ = maxp > kMaxDirectRadix;
    tmp_.resize(maxp);
    if (!bluestein_) {
      tw_.resize(n_);
      for (int k = 0; k < n_; ++k) tw_[k] = Twiddle(k, n_, sign_);
      scratch_.resize(n_);
    } else {
      m_ = 1;
      while (m_ < 2 * n_ - 1) m_ <<= 1;
      // chirp[k] = exp(sign * pi*i * k^2 / n), k^2 reduced mod 2n exactly.
      chirp_.resize(n_);
      for (int64_t k = 0; k < n_; ++k) {
        const int64_t k2 = (k * k) % (2 * int64_t(n_));
        const double ang = M_PI * double(k2) / double(n_);
        chirp_[k] = cd(std::cos(ang), sign_ * std::sin(ang));
      }
      pow2_.reset(new Plan(m_, -1));
      pow2_inv_.reset(new Plan(m_, +1));
      std::vector<cd> b(m_, cd(0, 0));
      b[0] = std::conj(chirp_[0]);
      for (int k = 1; k < n_; ++k) b[k] = b[m_ - k] = std::conj(chirp_[k]);
      bhat_.resize(m_);
      pow2_->Run(b.data(), bhat_.data());
      work_.resize(m_);
      work2_.resize(m_);
    }
  }

  int n() const { return n_; }

  // out may alias in.
  void Run(const cd *in, cd *out) {
    if (n_ <= 0) return;
    if (!bluestein_) {
      Rec(in, 1, scratch_.data(), n_, 0, 1);
      for (int k = 0; k < n_; ++k) out[k] = scratch_[k];
      return;
    }
    // Bluestein: out[k] = chirp[k] * sum_j (in[j]*chirp[j]) * conj(chirp[k-j]).
    for (int j = 0; j < m_; ++j) work_[j] = cd(0, 0);
    for (int j = 0; j < n_; ++j) work_[j] = in[j] * chirp_[j];
    pow2_->Run(work_.data(), work2_.data());
    for (int j = 0; j < m_; ++j) work2_[j] *= bhat_[j];
    pow2_inv_->Run(work2_.data(), work_.data());
    const double inv = 1.0 / double(m_);
    for (int k = 0; k < n_; ++k) out[k] = work_[k] * chirp_[k] * inv;
  }

private:
  // out[0..n) = DFT_n of in[0], in[s], ..., in[(n-1)s]; level uses factor fi.
  // tws: stride into tw_ so that tw_[e*tws] = exp(sign*2*pi*i*e/n).
  void Rec(const cd *in, int64_t s, cd *out, int n, size_t fi, int64_t tws) {
    if (n == 1) {
      out[0] = in[0];
      return;
    }
    const int p = fac_[fi];
    const int m = n / p;
    for (int j = 0; j < p; ++j) {
      Rec(in + j * s, s * p, out + j * m, m, fi + 1, tws * p);
    }
    cd *tmp = tmp_.data(); // butterflies of one level never nest
    for (int k = 0; k < m; ++k) {
      for (int j = 0; j < p; ++j) tmp[j] = out[j * m + k];
      for (int qq = 0; qq < p; ++qq) {
        const int64_t kk = k + int64_t(qq) * m;
        cd acc = tmp[0];
        for (int j = 1; j < p; ++j) {
          const int64_t e = (int64_t(j) * kk) % n;
          acc += tmp[j] * tw_[e * tws];
        }
        out[kk] = acc;
      }
    }
  }

  int n_;
  int sign_;
  std::vector<int> fac_;
  bool bluestein_ = false;
  std::vector<cd> tw_;
  std::vector<cd> scratch_;
  std::vector<cd> tmp_;
  int m_ = 0;
  std::vector<cd> chirp_;
  std::vector<cd> bhat_;
  std::vector<cd> work_, work2_;
  std::unique_ptr<Plan> pow2_, pow2_inv_;
};

} // namespace fft64
