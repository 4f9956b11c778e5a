// CPU oracle: this project's FP64 restatement of the MPSFT recovery loop of
// jiaweichiu/mpsft. TEST INFRASTRUCTURE ONLY. It is the checker for the CUDA
// path (tests, smoke()) and the timed CPU baseline in bench.py; the product
// path never links or calls it.
//
// Each function follows the reference's arithmetic step by step (same
// operation order, IEEE double, no FMA contraction), so that on one host it
// agrees bit for bit with the reference compiled by oracle/Makefile
// (oracle/_ref), which the tests check. Citations are to files of the
// reference project.
//
// Implements oracle_capi.h.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <limits>
#include <random>
#include <unordered_map>
#include <utility>
#include <vector>

#include "fft64.h"
#include "oracle_capi.h"

namespace {

using Cplex = std::complex<double>;
using ModeMap = std::unordered_map<int32_t, Cplex>;

// ---------------------------------------------------------------------------
// RNG: one global mt19937 seeded with 123534, int32 draws from
// uniform_int_distribution<int32_t> over [0, 2^31-1] (src/base.cc:32-56).
std::mt19937 g_rng(123534);
std::uniform_int_distribution<int32_t> g_uid32;
std::normal_distribution<double> g_nd;

int32_t DrawInt32() { return g_uid32(g_rng); }
double DrawNormal() { return g_nd(g_rng); }

// ---------------------------------------------------------------------------
// Modular arithmetic in int64, truncated to int32 (src/integer.h:47-66).
inline int32_t MulMod(int64_t a, int64_t b, int64_t d) {
  return int32_t((a * b) % d);
}
inline int32_t MulPosMod(int64_t a, int64_t b, int64_t d) {
  const int32_t x = MulMod(a, b, d);
  return x >= 0 ? x : int32_t(x + d);
}
inline int32_t MulAddMod(int64_t a, int64_t b, int64_t c, int64_t d) {
  return int32_t((a * b + c) % d);
}
inline int32_t MulAddPosMod(int64_t a, int64_t b, int64_t c, int64_t d) {
  const int32_t x = MulAddMod(a, b, c, d);
  return x >= 0 ? x : int32_t(x + d);
}

inline double PosModOne(double x) { return x - std::floor(x); }

// e^{2 pi i f} (src/sincos.h:42-45).
inline Cplex Sinusoid(double f) {
  f *= (2.0 * M_PI);
  return Cplex(std::cos(f), std::sin(f));
}

// sin(x)/x with the Taylor guard of src/sincos.cc:69-88.
double SincPi(double x) {
  const double t0 = std::numeric_limits<double>::epsilon();
  const double t2 = std::sqrt(t0);
  const double tn = std::sqrt(t2);
  if (x < 0) x = -x;
  if (x >= tn) return std::sin(x) / x;
  double r = 1.0;
  if (x >= t0) {
    const double x2 = x * x;
    r -= x2 / 6.0;
    if (x >= t2) r += (x2 * x2) / 120.0;
  }
  return r;
}

// (a, b, c, a_inv): y_t = x_{a t + c} e^{2 pi i b t / n} (src/integer.h:68-82).
struct Perm {
  int32_t a, b, c, a_inv;
};

bool IsPow2(int64_t n) { return n > 0 && (n & (n - 1)) == 0; }

// Inverse of a mod m by the extended Euclidean algorithm; equals the
// reference's Fermat inverse (src/integer.cc:27-40) for prime m. Returns 0 when
// a is not invertible.
int32_t InverseMod(int64_t a, int64_t m) {
  int64_t r0 = m, r1 = ((a % m) + m) % m, s0 = 0, s1 = 1;
  while (r1 != 0) {
    const int64_t qt = r0 / r1;
    int64_t t = r0 - qt * r1;
    r0 = r1;
    r1 = t;
    t = s0 - qt * s1;
    s0 = s1;
    s1 = t;
  }
  if (r0 != 1) return 0;
  return int32_t(((s0 % m) + m) % m);
}

// Transform(n) (src/integer.cc:44-49): draws a, b, c in that order; for
// power-of-two n, a is made odd (a |= 1) so that it is invertible.
Perm DrawPerm(int32_t n) {
  Perm p;
  p.a = (DrawInt32() % (n - 1)) + 1;
  p.b = DrawInt32() % n;
  p.c = DrawInt32() % n;
  if (IsPow2(n)) p.a |= 1;
  p.a_inv = InverseMod(p.a, n);
  return p;
}

// NumBits (src/iterate.cc:30-42).
int32_t NumBits(int32_t n, int32_t bins) {
  if (n < bins) return 1;
  int32_t out = 0;
  while (n >= bins) {
    n >>= 1;
    ++out;
  }
  return out;
}

// ---------------------------------------------------------------------------
// Smoothed boxcar window (src/window.cc:28-81).
struct Win {
  int32_t n, bins, p;
  double width, sigma_f, sigma_t;
  std::vector<int32_t> t;  // 0, 1..p2, -p2..-1
  std::vector<double> wt;  // window at t

  Win(int32_t n_, int32_t bins_, double delta) : n(n_), bins(bins_) {
    width = 1.0 / (2.0 * bins);
    const double sq = std::sqrt(-std::log(delta));
    sigma_f = 0.5 / (bins * 2.0 * M_SQRT2 * sq);
    sigma_t = 1.0 / ((2.0 * M_PI) * sigma_f);
    const double tmp = 2.0 * M_SQRT2 * sigma_t * sq + 1;
    int32_t f = int32_t(std::ceil(tmp / double(bins)));
    if (f % 2 == 0) ++f;
    p = f * bins;
    const int32_t p2 = (p - 1) / 2;
    t.resize(p);
    wt.resize(p);
    for (int32_t i = 0; i < p; ++i) t[i] = i <= p2 ? i : i - p;
    wt[0] = width;
    for (int32_t i = 1; i < p; ++i) wt[i] = InTime(t[i]);
  }
  double InTime(int32_t i) const {
    const double tt = double(i);
    const double u = tt * M_PI * sigma_f;
    return width * SincPi(tt * M_PI * width) * std::exp(-2.0 * u * u);
  }
  double InFreq(double xi) const {
    const double c = 0.5 * width;
    const double d = M_SQRT2 * M_PI * sigma_t;
    return 0.5 * (std::erf((xi + c) * d) - std::erf((xi - c) * d));
  }
};

// Bin matrix: rows x bins, row-major.
struct Bins {
  int32_t rows, cols;
  std::vector<Cplex> v;
  Bins(int32_t r, int32_t c) : rows(r), cols(c), v(size_t(r) * c) {}
  Cplex *row(int32_t r) { return v.data() + size_t(r) * cols; }
  const Cplex *row(int32_t r) const { return v.data() + size_t(r) * cols; }
};

// tau of row r: q, q + B 2^s (r = 2s+1), q - B 2^s (r = 2s+2)
// (src/binner.cc:42-50).
int32_t RowTau(int32_t q, int32_t bins, int32_t r) {
  if (r == 0) return q;
  if (r & 1) return q + bins * (1 << ((r - 1) / 2));
  return q - bins * (1 << (r / 2 - 1));
}

// Time-domain binning with the even/odd split of BinInTimeV4::Run
// (src/binner.cc:394-521); the arithmetic of each step follows it in order.
void BinTimeV4(const Win &w, int32_t bits, const Cplex *x, const Perm &tf,
               int32_t q, fft64::Plan *plan, Bins *out) {
  const int32_t bins = w.bins, n = w.n, p = w.p;
  const double delta = -0.5 / double(bins);
  std::vector<Cplex> s1(p), s2(p);

  std::fill(s1.begin(), s1.begin() + bins, Cplex(0, 0));
  for (int32_t i = 0; i < p; ++i) {
    const int32_t t = w.t[i];
    const int32_t j = MulAddPosMod(tf.a, int64_t(t) + int64_t(q), tf.c, n);
    const int32_t k = MulMod(tf.b, int64_t(t) + int64_t(q), n);
    const double f = double(k) / double(n) + PosModOne(delta * double(t));
    s1[i % bins] += (x[j] * Sinusoid(f)) * w.wt[i];
  }
  plan->Run(s1.data(), out->row(0));

  const Cplex bq = Sinusoid(double(MulMod(tf.b, q, n)) / double(n));
  const double br = bq.real(), bi = bq.imag();
  for (int32_t bit = 0; bit < bits; ++bit) {
    const int32_t offset = bins * (1 << bit);
    for (int32_t i = 0; i < p; ++i) {
      const int64_t ts = int64_t(w.t[i]) + int64_t(offset);
      const int32_t j1 = MulAddPosMod(tf.a, int64_t(q) + ts, tf.c, n);
      const int32_t j2 = MulAddPosMod(tf.a, int64_t(q) - ts, tf.c, n);
      const int32_t k1 = MulMod(tf.b, ts, n);
      const double f =
          double(k1) / double(n) + PosModOne(delta * double(w.t[i]));
      const double x1r = x[j1].real(), x1i = x[j1].imag();
      const double x2r = x[j2].real(), x2i = x[j2].imag();
      // x1 * bq and conj(x2 * bq), then the even / odd combinations.
      const double e2 = br * x1r - bi * x1i;
      const double e3 = br * x1i + bi * x1r;
      const double e4 = br * x2r - bi * x2i;
      const double e5 = -br * x2i - bi * x2r;
      const double f2 = 0.5 * (e2 + e4);
      const double f3 = 0.5 * (e3 + e5);
      const double f4 = 0.5 * (e3 - e5);
      const double f5 = 0.5 * (e4 - e2);
      const double ang = 2.0 * M_PI * f;
      const double ss = std::sin(ang), cc = std::cos(ang);
      const double g2 = f2 * cc - f3 * ss;
      const double g3 = f2 * ss + f3 * cc;
      const double g4 = f4 * cc - f5 * ss;
      const double g5 = f4 * ss + f5 * cc;
      s1[i] = Cplex(g2, g3);
      s2[i] = Cplex(g4, g5);
      s1[i] *= w.wt[i];
      s2[i] *= w.wt[i];
    }
    const int32_t folds = p / bins;
    for (int32_t fo = 1; fo < folds; ++fo) {
      for (int32_t j = 0; j < bins; ++j) {
        s1[j] += s1[fo * bins + j];
        s2[j] += s2[fo * bins + j];
      }
    }
    Cplex *ur = out->row(2 * bit + 1);
    Cplex *ui = out->row(2 * bit + 2);
    plan->Run(s1.data(), ur);
    plan->Run(s2.data(), ui);
    for (int32_t b = 0; b < bins; ++b) {
      const Cplex cr = ur[b], ci = ui[b];
      ur[b] = cr + Cplex(-ci.imag(), ci.real());
      const Cplex cic = std::conj(ci);
      ui[b] = std::conj(cr) + Cplex(-cic.imag(), cic.real());
    }
  }
}

// Direct statement of the binning, BinInTimeV0::Run (src/binner.cc:81-111):
// each row is the size-B DFT of the folded, windowed, modulated samples. Any
// binner type other than 4 selects this one.
void BinTimeDirect(const Win &w, int32_t bits, const Cplex *x, const Perm &tf,
                   int32_t q, fft64::Plan *plan, Bins *out) {
  const int32_t bins = w.bins, n = w.n, p = w.p;
  const double delta = -0.5 / double(bins);
  std::vector<Cplex> s(bins);
  for (int32_t r = 0; r < out->rows; ++r) {
    const int32_t tau = RowTau(q, bins, r);
    std::fill(s.begin(), s.end(), Cplex(0, 0));
    for (int32_t i = 0; i < p; ++i) {
      const int32_t t = w.t[i];
      const int32_t j = MulAddPosMod(tf.a, int64_t(t) + int64_t(tau), tf.c, n);
      const int32_t k = MulMod(tf.b, int64_t(t) + int64_t(tau), n);
      const double f = double(k) / double(n) + PosModOne(delta * double(t));
      s[i % bins] += (x[j] * Sinusoid(f)) * w.wt[i];
    }
    plan->Run(s.data(), out->row(r));
  }
}

// Frequency-domain subtraction of found modes, BinInFreqV1::Run
// (src/binner.cc:565-591).
void BinFreqV1(const Win &w, int32_t bits, const ModeMap &mm, const Perm &tf,
               int32_t q, Bins *out) {
  const int32_t bins = w.bins, n = w.n;
  for (const auto &kv : mm) {
    const int32_t k0 = kv.first;
    const int32_t k1 = MulAddPosMod(tf.a, k0, tf.b, n);
    const int32_t bin = int32_t(int64_t(k1) * int64_t(bins) / int64_t(n));
    const double xi =
        (double(bin) + 0.5) / double(bins) - double(k1) / double(n);
    const double wf = w.InFreq(xi);
    const double f =
        double(MulAddMod(q, k1, int64_t(tf.c) * int64_t(k0), n)) / double(n);
    const Cplex base = wf * kv.second * Sinusoid(f);
    out->row(0)[bin] -= base;
    for (int32_t bit = 0; bit < bits; ++bit) {
      const int32_t offset = bins * (1 << bit);
      const Cplex fac = Sinusoid(double(MulMod(offset, k1, n)) / double(n));
      out->row(2 * bit + 1)[bin] -= base * fac;
      out->row(2 * bit + 2)[bin] -= base * std::conj(fac);
    }
  }
}

// 2x2 matrix pencil [[u0, u2], [u1, u0]] (src/freqid.cc:27-48): singular
// values from the Hermitian eigenproblem of A^H A (sigma1 = |det A| / sigma0),
// vote = Im(conj(v00) v10) < 0 for the dominant right singular vector v.
bool Pencil(Cplex u0, Cplex u1, Cplex u2, double *sigma) {
  const double m00 = std::norm(u0) + std::norm(u1);
  const double m11 = std::norm(u2) + std::norm(u0);
  const Cplex m01 = std::conj(u0) * u2 + std::conj(u1) * u0;
  const double hd = 0.5 * (m00 - m11);
  const double r = std::sqrt(hd * hd + std::norm(m01));
  const double lmax = 0.5 * (m00 + m11) + r;
  const double s0 = std::sqrt(lmax > 0 ? lmax : 0.0);
  const double det = std::abs(u0 * u0 - u2 * u1);
  sigma[0] = s0;
  sigma[1] = s0 > 0 ? det / s0 : 0.0;
  Cplex v0, v1;
  if (std::norm(m01) == 0.0) {
    v0 = m00 >= m11 ? Cplex(1) : Cplex(0);
    v1 = m00 >= m11 ? Cplex(0) : Cplex(1);
  } else if (m00 >= m11) {
    v0 = Cplex(lmax - m11);
    v1 = std::conj(m01);
  } else {
    v0 = m01;
    v1 = Cplex(lmax - m00);
  }
  const double nrm = std::sqrt(std::norm(v0) + std::norm(v1));
  v0 /= nrm;
  v1 /= nrm;
  return std::imag(std::conj(v0) * v1) < 0;
}

struct IterOpts {
  int32_t bins = 0;
  double window_delta = 1e-6;
  int32_t trials = 1;
  double bin_threshold = 0;
  double window_threshold = 0;
  double sv_threshold = 0;
  int btype = 4;
  int ftype = 1;
};

// IdentifyFreq (src/iterate.cc:44-76): per bit, majority vote of the trials'
// pencils; any pencil with sigma1 / 2 > sv_threshold rejects the bin.
std::pair<double, bool> Identify(const IterOpts &opt, int32_t b, int32_t bits,
                                 const std::vector<Bins> &coefs) {
  double sigma[2];
  int32_t xs = 0;
  for (int32_t bit = 0; bit < bits; ++bit) {
    int32_t count = 0;
    for (int32_t tr = 0; tr < opt.trials; ++tr) {
      const Bins &a = coefs[tr];
      if (Pencil(a.row(0)[b], a.row(2 * bit + 1)[b], a.row(2 * bit + 2)[b],
                 sigma)) {
        ++count;
      }
      if (opt.sv_threshold > 0 && sigma[1] * 0.5 > opt.sv_threshold) {
        return std::make_pair(0.0, false);
      }
    }
    xs <<= 1;
    if (count > opt.trials / 2) ++xs;
  }
  return std::make_pair(double(2 * xs + 1) / double(1 << (bits + 1)), true);
}

// Iterate (src/iterate.cc:80-176).
bool IterateOnce(const Cplex *x, int32_t n, const IterOpts &opt, ModeMap *mm) {
  bool found = false;
  const int32_t trials = opt.trials, bins = opt.bins;
  Win win(n, bins, opt.window_delta);
  const int32_t bits = NumBits(n, bins);
  const Perm tf = DrawPerm(n);
  fft64::Plan plan(bins, -1);
  std::vector<double> qs;
  std::vector<Bins> coefs;
  coefs.reserve(trials);
  for (int32_t tr = 0; tr < trials; ++tr) {
    const int32_t q = DrawInt32() % n;
    qs.push_back(q);
    coefs.emplace_back(1 + 2 * bits, bins);
    if (opt.btype == 4) {
      BinTimeV4(win, bits, x, tf, q, &plan, &coefs.back());
    } else {
      BinTimeDirect(win, bits, x, tf, q, &plan, &coefs.back());
    }
    BinFreqV1(win, bits, *mm, tf, q, &coefs.back());
  }
  for (int32_t b = 0; b < bins; ++b) {
    if (opt.bin_threshold > 0) {
      double e = 0;
      for (int32_t tr = 0; tr < trials; ++tr) {
        const Cplex u = coefs[tr].row(0)[b];
        e += u.real() * u.real() + u.imag() * u.imag();
      }
      e /= trials;
      if (e < opt.bin_threshold * opt.bin_threshold) continue;
    }
    const auto res = Identify(opt, b, bits, coefs);
    if (!res.second) continue;
    const double xi1 = res.first;
    const int32_t k1 =
        int32_t(std::round(double(n) * (double(b) + xi1) / double(bins)));
    const double xi0 = double(k1) / double(n) - (double(b) + 0.5) / double(bins);
    const double wf = win.InFreq(xi0);
    if (std::abs(wf) < opt.window_threshold) continue;

    Cplex sum = 0;
    for (int32_t tr = 0; tr < trials; ++tr) {
      const Bins &a = coefs[tr];
      const double f = -double(MulMod(int64_t(qs[tr]), k1, n)) / double(n);
      const Cplex fac = Sinusoid(f);
      sum += a.row(0)[b] * fac;
      for (int32_t bit = 0; bit < bits; ++bit) {
        const double f2 = -double(MulMod(bins * (1 << bit), k1, n)) / double(n);
        const Cplex fac2 = Sinusoid(f2);
        const Cplex g1 = fac * fac2;
        const Cplex g2 = fac * std::conj(fac2);
        sum += a.row(2 * bit + 1)[b] * g1;
        sum += a.row(2 * bit + 2)[b] * g2;
      }
    }
    Cplex coef = sum / double(trials * (1 + 2 * bits));
    const int32_t k0 = MulPosMod(tf.a_inv, int64_t(k1) - int64_t(tf.b), n);
    coef *= Sinusoid(-double(MulMod(tf.c, k0, n)) / double(n));
    coef /= wf;
    (*mm)[k0] += coef;
    found = true;
  }
  return found;
}

int WriteSorted(const ModeMap &mm, int32_t *ok, double *oc, int32_t cap) {
  std::vector<std::pair<int32_t, Cplex>> v(mm.begin(), mm.end());
  std::sort(v.begin(), v.end(),
            [](const std::pair<int32_t, Cplex> &l,
               const std::pair<int32_t, Cplex> &r) { return l.first < r.first; });
  if (int64_t(v.size()) > cap) return -1;
  for (size_t i = 0; i < v.size(); ++i) {
    ok[i] = v[i].first;
    oc[2 * i] = v[i].second.real();
    oc[2 * i + 1] = v[i].second.imag();
  }
  return int(v.size());
}

const Cplex *AsCplex(const double *p) {
  return reinterpret_cast<const Cplex *>(p);
}

} // namespace

extern "C" {

void orc_seed(int32_t seed) { g_rng.seed(seed); }
int32_t orc_random_int32(void) { return DrawInt32(); }
double orc_random_normal(void) { return DrawNormal(); }
int32_t orc_num_bits(int32_t n, int32_t bins) { return NumBits(n, bins); }

int32_t orc_window(int32_t n, int32_t bins, double delta, double *wt,
                   int32_t cap) {
  Win w(n, bins, delta);
  if (wt != nullptr && cap >= w.p) {
    std::memcpy(wt, w.wt.data(), sizeof(double) * w.p);
  }
  return w.p;
}

double orc_window_sample_in_freq(int32_t n, int32_t bins, double delta,
                                 double xi) {
  return Win(n, bins, delta).InFreq(xi);
}

void orc_transform(int32_t n, int32_t *out) {
  const Perm p = DrawPerm(n);
  out[0] = p.a;
  out[1] = p.b;
  out[2] = p.c;
  out[3] = p.a_inv;
}

int32_t orc_transform_inverse(int32_t n, int32_t a) {
  return InverseMod(a, n);
}

int orc_bin_in_time(int type, int32_t n, int32_t bins, int32_t bits,
                    double delta, int32_t a, int32_t b, int32_t c, int32_t q,
                    const double *x, double *out) {
  Win w(n, bins, delta);
  Perm tf{a, b, c, InverseMod(a, n)};
  fft64::Plan plan(bins, -1);
  Bins m(1 + 2 * bits, bins);
  if (type == 4) {
    BinTimeV4(w, bits, AsCplex(x), tf, q, &plan, &m);
  } else {
    BinTimeDirect(w, bits, AsCplex(x), tf, q, &plan, &m);
  }
  std::memcpy(out, m.v.data(), sizeof(Cplex) * m.v.size());
  return 0;
}

int orc_bin_in_freq(int type, int32_t n, int32_t bins, int32_t bits,
                    double delta, int32_t a, int32_t b, int32_t c, int32_t q,
                    const int32_t *k0, const double *coef, int32_t mcount,
                    double *out) {
  (void)type;
  Win w(n, bins, delta);
  Perm tf{a, b, c, InverseMod(a, n)};
  ModeMap mm;
  for (int32_t i = 0; i < mcount; ++i) {
    mm[k0[i]] = Cplex(coef[2 * i], coef[2 * i + 1]);
  }
  Bins m(1 + 2 * bits, bins);
  std::memcpy(reinterpret_cast<void *>(m.v.data()), out,
              sizeof(Cplex) * m.v.size());
  BinFreqV1(w, bits, mm, tf, q, &m);
  std::memcpy(out, m.v.data(), sizeof(Cplex) * m.v.size());
  return 0;
}

int orc_mat_pencil(const double *u, double *sigma) {
  return Pencil(Cplex(u[0], u[1]), Cplex(u[2], u[3]), Cplex(u[4], u[5]), sigma)
             ? 1
             : 0;
}

int orc_iterate(int32_t n, const double *x, int32_t bins, double window_delta,
                int32_t trials, double bin_threshold, double window_threshold,
                double sv_threshold, int bin_in_time_type,
                int bin_in_freq_type, int32_t *mm_k, double *mm_c,
                int32_t *mm_size, int32_t mm_cap) {
  IterOpts opt;
  opt.bins = bins;
  opt.window_delta = window_delta;
  opt.trials = trials;
  opt.bin_threshold = bin_threshold;
  opt.window_threshold = window_threshold;
  opt.sv_threshold = sv_threshold;
  opt.btype = bin_in_time_type;
  opt.ftype = bin_in_freq_type;
  ModeMap mm;
  for (int32_t i = 0; i < *mm_size; ++i) {
    mm[mm_k[i]] = Cplex(mm_c[2 * i], mm_c[2 * i + 1]);
  }
  const bool found = IterateOnce(AsCplex(x), n, opt, &mm);
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
  // Demo1::Run (src/demo1.cc:36-59). The stale counter is never reset.
  g_rng.seed(seed);
  IterOpts opt;
  opt.window_delta = window_delta;
  opt.window_threshold = window_threshold;
  opt.trials = trials;
  ModeMap found;
  int32_t stale = 0, it = 0;
  for (; stale < max_stale_iter; ++it) {
    opt.bins = std::max<int32_t>((k - int32_t(found.size())) * 2 + 1, min_bins);
    opt.bin_threshold = 3.0 * sigma / std::sqrt(double(opt.bins));
    opt.sv_threshold = 1.0 * sigma / std::sqrt(double(opt.bins));
    if (!IterateOnce(AsCplex(x), n, opt, &found)) ++stale;
  }
  if (iters) *iters = it;
  return WriteSorted(found, out_k, out_c, cap);
}

int orc_generate_mode_map(int32_t n, int32_t k, int32_t *out_k, double *out_c) {
  // GenerateModeMap (src/gen.cc:27-39): draw a position (RandomInt32() is
  // non-negative, so UnsafePosMod is the remainder), skip repeats, then two
  // normals for the coefficient. The reference builds the coefficient as
  // Cplex(RandomNormal(), RandomNormal()); g++ evaluates those two arguments
  // right to left, so the imaginary part takes the first draw.
  ModeMap mm;
  while (int32_t(mm.size()) < k) {
    const int32_t idx = DrawInt32() % n;
    if (mm.count(idx)) continue;
    const double im = DrawNormal();
    const double re = DrawNormal();
    Cplex coef(re, im);
    coef /= std::abs(coef);
    mm[idx] = coef;
  }
  return WriteSorted(mm, out_k, out_c, k);
}

int orc_demo_signal(int32_t n, int32_t k, double sigma, int xhat_kind,
                    double *x, int32_t *out_k, double *out_c) {
  // GenerateModeMap, then GenerateXhat / GenerateXhatAlt (src/gen.cc:27-89),
  // then FFTPlan(n, FFTW_BACKWARD) (src/demo1.cc:27-34). Each complex normal
  // is Cplex(RandomNormal(), RandomNormal()), imaginary part first (g++
  // evaluates the two arguments right to left); the noise energy subtracts
  // the mode positions in the map's own iteration order.
  ModeMap mm;
  while (int32_t(mm.size()) < k) {
    const int32_t idx = DrawInt32() % n;
    if (mm.count(idx)) continue;
    const double im = DrawNormal();
    const double re = DrawNormal();
    Cplex coef(re, im);
    coef /= std::abs(coef);
    mm[idx] = coef;
  }
  std::vector<Cplex> xh(n, Cplex(0.0, 0.0));
  if (xhat_kind == 0) {
    double noise_energy = 0;
    for (int32_t i = 0; i < n; ++i) {
      const double im = DrawNormal();
      const double re = DrawNormal();
      xh[i] = Cplex(re, im);
      noise_energy += re * re + im * im;
    }
    for (const auto &kv : mm) {
      const Cplex v = xh[kv.first];
      noise_energy -= v.real() * v.real() + v.imag() * v.imag();
    }
    const double factor = sigma / std::sqrt(noise_energy);
    for (int32_t i = 0; i < n; ++i) xh[i] *= factor;
    for (const auto &kv : mm) xh[kv.first] = kv.second;
  } else {
    for (const auto &kv : mm) xh[kv.first] = kv.second;
    const double scale = sigma / std::sqrt(2 * n);
    for (int32_t i = 0; i < n; ++i) {
      const double im = DrawNormal();
      const double re = DrawNormal();
      xh[i] += Cplex(re, im) * scale;
    }
  }
  fft64::Plan plan(n, +1);
  plan.Run(xh.data(), reinterpret_cast<Cplex *>(x));
  return WriteSorted(mm, out_k, out_c, k);
}

void orc_post_analyze(int32_t n, const double *xh, const int32_t *true_k,
                      int32_t true_count, const int32_t *found_k,
                      const double *found_c, int32_t found_count, double *out) {
  // Demo1::PostAnalyze (src/demo1.cc:61-112): found modes at true positions
  // are hits, the others misses, each with the error |c - xh_k|; then the
  // sparse found spectrum against xh over all n frequencies.
  const Cplex *x = AsCplex(xh);
  std::unordered_map<int32_t, int> is_true;
  for (int32_t i = 0; i < true_count; ++i) is_true[true_k[i]] = 1;
  std::vector<Cplex> xh2(n, Cplex(0.0, 0.0));
  int32_t hit = 0, miss = 0;
  double hit_l1 = 0, hit_l2 = 0, miss_l1 = 0, miss_l2 = 0;
  for (int32_t i = 0; i < found_count; ++i) {
    const Cplex c(found_c[2 * i], found_c[2 * i + 1]);
    xh2[found_k[i]] = c;
    const double err = std::abs(c - x[found_k[i]]);
    if (is_true.count(found_k[i])) {
      ++hit;
      hit_l1 += err;
      hit_l2 += err * err;
    } else {
      ++miss;
      miss_l1 += err;
      miss_l2 += err * err;
    }
  }
  double sum1 = 0, sum2 = 0, max_err = 0;
  for (int32_t i = 0; i < n; ++i) {
    const double err = std::abs(xh2[i] - x[i]);
    sum1 += err;
    sum2 += err * err;
    max_err = std::max(max_err, err);
  }
  out[0] = hit;
  out[1] = hit_l1 / hit;
  out[2] = std::sqrt(hit_l2 / hit);
  out[3] = miss;
  out[4] = miss_l1 / miss;
  out[5] = std::sqrt(miss_l2 / miss);
  out[6] = sum1 / n;
  out[7] = std::sqrt(sum2 / n);
  out[8] = max_err;
}

} // extern "C"
