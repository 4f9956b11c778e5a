// Stand-in for the part of FFTW 3's C API that the reference uses
// (src/base.cc:86-97: fftw_plan_dft_1d, fftw_execute_dft, fftw_destroy_plan).
// Written for this project; only the names and signatures follow FFTW. The
// transform is oracle/fft64.h (unnormalised, sign -1 forward / +1 backward).
// Test infrastructure only.
#pragma once

#include "../fft64.h"

typedef double fftw_complex[2];
typedef fft64::Plan *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

inline fftw_plan fftw_plan_dft_1d(int n, fftw_complex *, fftw_complex *,
                                  int sign, unsigned) {
  return new fft64::Plan(n, sign);
}

inline void fftw_execute_dft(const fftw_plan p, fftw_complex *in,
                             fftw_complex *out) {
  p->Run(reinterpret_cast<const fft64::cd *>(in),
         reinterpret_cast<fft64::cd *>(out));
}

inline void fftw_destroy_plan(fftw_plan p) { delete p; }
