// Host-side checks of integer helpers shared by the kernels (compiled and run
// by tests/test_host_arith.py; no GPU is used):
//  * RoundK1, the division-free k1 rounding of the decide kernels, against
//    the same rounding computed with a 64-bit division;
//  * StashRows, the rows the FP32 fold stashes, against its capacity and the
//    an-eighth-of-the-signal rule.
// Prints one line per check and exits non-zero on any mismatch.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>

#include "../../mpsft_gb300/csrc/common.cuh"
#include "../../mpsft_gb300/csrc/decide.cuh"

namespace {

// k1 = round(n (beta + (2 xs + 1) / 2^{L+1}) / B) with a 64-bit division, and
// the FP64 expression within 2^-18 of a half-integer.
int64_t RoundK1Div(int64_t n, int beta, uint32_t xs, int L, int B) {
  const uint64_t den = uint64_t(B) << (L + 1);
  const uint64_t num = uint64_t(n) * ((uint64_t(beta) << (L + 1)) + 2 * uint64_t(xs) + 1);
  const uint64_t q = num / den;
  const uint64_t r = num - q * den;
  const uint64_t d = 2 * r > den ? 2 * r - den : den - 2 * r;
  if (d <= (den >> 17)) {
    const double xi1 = std::ldexp(2.0 * double(xs) + 1.0, -(L + 1));
    return int64_t(std::round(double(n) * (double(beta) + xi1) / double(B)));
  }
  return int64_t(q) + (2 * r >= den ? 1 : 0);
}

int NumBitsOf(int64_t n, int B) {
  if (n < B) return 1;
  int L = 0;
  while (n >= B) {
    n >>= 1;
    ++L;
  }
  return L;
}

}  // namespace

int main() {
  using namespace mpsft;
  std::mt19937_64 g(20261204);
  long bad = 0, total = 0;
  const int64_t ns[] = {3,       5,       65537,   1 << 16,    1 << 20,   1048573,
                        4194301, 1 << 22, 1 << 26, 2147483647, 1 << 30};
  for (int64_t n : ns) {
    for (int rep = 0; rep < 100000; ++rep) {
      int B = 1 + 2 * int(g() % 4100);
      if (B > n) B = int(n % 2 ? n : n - 1);
      const int L = NumBitsOf(n, B);
      const int beta = int(g() % uint64_t(B));
      const uint32_t xs = uint32_t(g() % (uint64_t(1) << L));
      SigIter it{};
      it.n = int32_t(n);
      it.bins = B;
      SetBinsFixedPoint(&it);
      ++total;
      if (RoundK1(n, beta, xs, L, B, it.psi) != RoundK1Div(n, beta, xs, L, B)) ++bad;
    }
  }
  std::printf("round_k1 checked %ld mismatches %ld\n", total, bad);
  long sbad = 0, stotal = 0;
  for (int rep = 0; rep < 20000; ++rep) {
    SigIter it{};
    unsigned char dummy = 0;
    it.stash = &dummy;
    it.n = int32_t(1) << (16 + int(g() % 11));
    it.trials = 1 + 2 * int(g() % 3);
    it.rows = 1 + 2 * int(1 + g() % 20);
    it.p = int32_t(31 * (1 + 2 * (g() % 2000)));
    it.stash_cap = int64_t(g() % (int64_t(1) << 22));
    const int s = StashRows(it);
    const int64_t need = int64_t(s) * it.p * it.trials;
    bool ok = (s == 0 || s == 1 || s == it.rows) && need <= it.stash_cap;
    if (s == it.rows && it.rows > 1) ok = ok && need <= int64_t(it.n) / 8;
    if (s == 0) ok = ok && int64_t(it.p) * it.trials > it.stash_cap;
    it.stash = nullptr;
    ok = ok && StashRows(it) == 0;
    ++stotal;
    if (!ok) ++sbad;
  }
  std::printf("stash_rows checked %ld mismatches %ld\n", stotal, sbad);
  return (bad || sbad) ? 1 : 0;
}
