// Coefficient estimation for a fixed frequency set, and its adjoint.
//
// With the identified set held fixed (no identification, no subtraction of
// other modes), Iterate's coefficient estimate (src/iterate.cc:146-171) is a
// linear map c = A x. For each given k0 with k1 = (a k0 + b) mod n, bin
// beta = floor(k1 B / n) and xi0 = k1/n - (beta + 1/2)/B:
//   c(k0) = s_k sum_t sum_r U_{t,r}[beta] e^{-2 pi i tau_{t,r} k1 / n},
//   s_k   = e^{-2 pi i c k0 / n} / (wf(xi0) T (1 + 2L)),
// where U_{t,r} are BinInTime's bins of row tau_{t,r} (q_t, q_t +- B 2^s):
//   U_tau[beta] = sum_{|t| <= p2} x[(a (tau + t) + c) mod n] wt(t)
//                 e^{2 pi i b (tau + t) / n} e^{-2 pi i t (2 beta + 1) / (2B)}.
// The adjoint dx = A^H g (g = dL/dc in torch's convention) is
//   G_{t,r}[beta] = sum_{k in beta} conj(s_k) g_k e^{2 pi i tau_{t,r} k1 / n},
//   H_{t,r}[m]    = sum_beta G_{t,r}[beta] e^{2 pi i beta m / B}   (inverse DFT),
//   dx[(a (tau + t) + c) mod n] += wt(t) e^{-2 pi i b (tau + t) / n}
//                                  e^{pi i t / B} H_{t,r}[t mod B],
// i.e. per-bin spreading over the rows, an inverse size-B DFT, unfolding to
// the window support and a windowed scatter-add at the permuted indices.
// All in FP64; the scatter-add uses FP64 atomics (rows overlap in x).
#include "common.cuh"
#include "launch.h"

namespace mpsft {

namespace {

__device__ inline int64_t RowOffset(int r, int64_t B) {
  if (r == 0) return 0;
  const int s = (r - 1) / 2;
  return (r & 1) ? (B << s) : -(B << s);
}

struct ModeSetup {
  int64_t k1;
  int beta;
  double2 s;  // e^{-2 pi i c k0 / n} / (wf T (1 + 2L))
};

__device__ inline ModeSetup SetupMode(const SigIter &it, int32_t k0) {
  const int64_t n = it.n, B = it.bins;
  const ModN mod{uint32_t(n), it.n_inv};
  ModeSetup m;
  m.k1 = mod(int64_t(it.a) * k0 + it.b);
  m.beta = int(mod.quot(m.k1 * B));
  const double xi0 = double(m.k1) / double(n) - (double(m.beta) + 0.5) / double(B);
  const double wf = WindowInFreq(it, xi0);
  const double scale = 1.0 / (wf * double(it.trials * (1 + 2 * it.bits)));
  m.s = cscale(Phase64(it, -int64_t(it.c) * k0), scale);
  return m;
}

// forward: one thread per mode, bins from ubuf (trials x rows x bins_cap)
__global__ void k_estimate(const SigIter *__restrict__ its, const int32_t *k0s,
                           int64_t m, double2 *coef) {
  const SigIter &it = *its;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const ModeSetup ms = SetupMode(it, k0s[i]);
  double2 acc = make_double2(0.0, 0.0);
  for (int t = 0; t < it.trials; ++t) {
    for (int r = 0; r < it.rows; ++r) {
      const int64_t tau = int64_t(it.q[t]) + RowOffset(r, it.bins);
      const double2 u = it.ubuf[(size_t(t) * it.rows + r) * it.bins_cap + ms.beta];
      acc = cadd(acc, cmul(u, Phase64(it, -tau * ms.k1)));
    }
  }
  coef[i] = cmul(acc, ms.s);
}

// adjoint, step 1: G (in the fold buffer, zeroed) += conj(s_k) g_k
// e^{2 pi i tau k1 / n}, stored conjugated for the forward FFT that follows
// (conj(DFT(conj(G))) is the inverse DFT of G).
__global__ void k_adjoint_spread(const SigIter *__restrict__ its,
                                 const int32_t *k0s, const double2 *g,
                                 int64_t m) {
  const SigIter &it = *its;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const ModeSetup ms = SetupMode(it, k0s[i]);
  const double2 w = cmul(cconj(ms.s), g[i]);
  double2 *G = reinterpret_cast<double2 *>(it.fold);
  for (int t = 0; t < it.trials; ++t) {
    for (int r = 0; r < it.rows; ++r) {
      const int64_t tau = int64_t(it.q[t]) + RowOffset(r, it.bins);
      const double2 v = cconj(cmul(w, Phase64(it, tau * ms.k1)));
      double2 *dst = G + (size_t(t) * it.rows + r) * it.bins_cap + ms.beta;
      atomicAdd(&dst->x, v.x);
      atomicAdd(&dst->y, v.y);
    }
  }
}

// adjoint, step 3: after ubuf = DFT(conj(G)) (row FFT with unit row
// factors), H = conj(ubuf); one thread per (trial, row, t) scatters into dx.
__global__ void k_adjoint_scatter(const SigIter *__restrict__ its, double2 *dx) {
  const SigIter &it = *its;
  const int64_t p = it.p;
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= int64_t(it.trials) * it.rows * p) return;
  const int64_t tt = idx % p;
  const int r = int((idx / p) % it.rows);
  const int t = int(idx / (p * it.rows));
  const int64_t n = it.n, B = it.bins;
  const int64_t ts = tt - it.p2;  // t in [-p2, p2]
  const int64_t tau = int64_t(it.q[t]) + RowOffset(r, B);
  const ModN mod{uint32_t(n), it.n_inv};
  const int64_t u = mod(tau + ts);
  const uint32_t j = mod(int64_t(it.a) * u + it.c);
  const int m = int(PosMod(ts, B));
  const double2 h = cconj(it.ubuf[(size_t(t) * it.rows + r) * it.bins_cap + m]);
  double sn, cs;
  sincospi(double(ts) / double(B), &sn, &cs);  // e^{pi i t / B}
  const double w = it.wt64[ts < 0 ? -ts : ts];
  const double2 v = cscale(cmul(cmul(h, make_double2(cs, sn)),
                                Phase64(it, -int64_t(it.b) * u)),
                           w);
  atomicAdd(&dx[j].x, v.x);
  atomicAdd(&dx[j].y, v.y);
}

}  // namespace

void LaunchEstimate(const SigIter *d_it, const int32_t *k0, int64_t m,
                    double2 *coef, cudaStream_t s) {
  if (m <= 0) return;
  k_estimate<<<unsigned((m + 127) / 128), 128, 0, s>>>(d_it, k0, m, coef);
}

void LaunchAdjointSpread(const SigIter *d_it, const int32_t *k0, const double2 *g,
                         int64_t m, cudaStream_t s) {
  if (m > 0) {
    k_adjoint_spread<<<unsigned((m + 127) / 128), 128, 0, s>>>(d_it, k0, g, m);
  }
}

void LaunchAdjointScatter(const SigIter *d_it, int64_t items, double2 *dx,
                          cudaStream_t s) {
  if (items <= 0) return;
  k_adjoint_scatter<<<unsigned((items + 255) / 256), 256, 0, s>>>(d_it, dx);
}

}  // namespace mpsft
