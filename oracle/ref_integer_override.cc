// Replacement for the reference's src/integer.cc (Transform constructors),
// linked into the oracle/_ref build of the reference in place of that file.
// Test infrastructure only.
//
// The reference draws a uniformly in [1, n-1] and inverts it with Fermat's
// little theorem (src/integer.cc:27-49), which is valid only for prime n. For
// n = 2^k an even a is not invertible, so this override keeps the same draws
// (a, then b, then c, from the same RNG calls) and, for power-of-two n only,
// forces a odd with a |= 1. The inverse is computed with the extended
// Euclidean algorithm, which equals Fermat's result for prime n. For prime n
// the override therefore returns exactly what the reference returns.
#include "integer.h"

namespace mps {

namespace {

bool IsPow2(int64_t n) { return n > 0 && (n & (n - 1)) == 0; }

int32_t InvModEuclid(int64_t a, int64_t m) {
  int64_t r0 = m, r1 = ((a % m) + m) % m;
  int64_t s0 = 0, s1 = 1;
  while (r1 != 0) {
    const int64_t qt = r0 / r1;
    int64_t t = r0 - qt * r1;
    r0 = r1;
    r1 = t;
    t = s0 - qt * s1;
    s0 = s1;
    s1 = t;
  }
  if (r0 != 1) {
    return 0; // not invertible; the binners never read a_inv
  }
  return int32_t(((s0 % m) + m) % m);
}

} // namespace

Transform::Transform(int32_t n) {
  a = (RandomInt32() % (n - 1)) + 1;
  b = RandomInt32() % n;
  c = RandomInt32() % n;
  if (IsPow2(n)) {
    a |= 1;
  }
  a_inv = InvModEuclid(a, n);
}

Transform::Transform(int32_t n, int32_t a, int32_t b, int32_t c) {
  this->a = a;
  this->b = b;
  this->c = c;
  this->a_inv = InvModEuclid(a, n);
}

} // namespace mps
