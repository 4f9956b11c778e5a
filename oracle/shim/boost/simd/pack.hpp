// Stand-in for the part of Boost.SIMD (NumScale, 4.x) that the reference uses
// (src/binner.cc:302-488, src/sincos_test.cc:46-58): pack<double> with four
// lanes (the AVX2 width the reference was built for), lane-wise arithmetic,
// aligned_load / aligned_store, sin and sincos. Written for this project; only
// the names follow Boost.SIMD. Each lane calls std::sin / std::cos. Test
// infrastructure only.
#pragma once

#include <cmath>
#include <cstddef>
#include <utility>

namespace boost {
namespace alignment {}
namespace simd {

template <typename T, std::size_t N = 4> struct pack {
  T v[N];
  pack() = default;
  explicit pack(T s) {
    for (std::size_t i = 0; i < N; ++i) v[i] = s;
  }
};

template <typename P> constexpr std::size_t cardinal_of() { return 4; }

template <typename P> inline P aligned_load(const double *p) {
  P r;
  for (std::size_t i = 0; i < 4; ++i) r.v[i] = p[i];
  return r;
}
template <typename P> inline P load(const double *p) {
  return aligned_load<P>(p);
}

template <typename T, std::size_t N>
inline void aligned_store(const pack<T, N> &a, T *p) {
  for (std::size_t i = 0; i < N; ++i) p[i] = a.v[i];
}
template <typename T, std::size_t N>
inline void store(const pack<T, N> &a, T *p) {
  aligned_store(a, p);
}

#define SHIM_BS_BINOP(op)                                                      \
  template <typename T, std::size_t N>                                         \
  inline pack<T, N> operator op(const pack<T, N> &a, const pack<T, N> &b) {    \
    pack<T, N> r;                                                              \
    for (std::size_t i = 0; i < N; ++i) r.v[i] = a.v[i] op b.v[i];             \
    return r;                                                                  \
  }                                                                            \
  template <typename T, std::size_t N>                                         \
  inline pack<T, N> operator op(T s, const pack<T, N> &b) {                    \
    pack<T, N> r;                                                              \
    for (std::size_t i = 0; i < N; ++i) r.v[i] = s op b.v[i];                  \
    return r;                                                                  \
  }                                                                            \
  template <typename T, std::size_t N>                                         \
  inline pack<T, N> operator op(const pack<T, N> &a, T s) {                    \
    pack<T, N> r;                                                              \
    for (std::size_t i = 0; i < N; ++i) r.v[i] = a.v[i] op s;                  \
    return r;                                                                  \
  }
SHIM_BS_BINOP(+)
SHIM_BS_BINOP(-)
SHIM_BS_BINOP(*)
SHIM_BS_BINOP(/)
#undef SHIM_BS_BINOP

template <typename T, std::size_t N>
inline pack<T, N> operator-(const pack<T, N> &a) {
  pack<T, N> r;
  for (std::size_t i = 0; i < N; ++i) r.v[i] = -a.v[i];
  return r;
}

template <typename T, std::size_t N> inline pack<T, N> sin(const pack<T, N> &a) {
  pack<T, N> r;
  for (std::size_t i = 0; i < N; ++i) r.v[i] = std::sin(a.v[i]);
  return r;
}

// Returns (sin(a), cos(a)) lane-wise.
template <typename T, std::size_t N>
inline std::pair<pack<T, N>, pack<T, N>> sincos(const pack<T, N> &a) {
  std::pair<pack<T, N>, pack<T, N>> r;
  for (std::size_t i = 0; i < N; ++i) {
    r.first.v[i] = std::sin(a.v[i]);
    r.second.v[i] = std::cos(a.v[i]);
  }
  return r;
}

} // namespace simd
} // namespace boost
