/* C interface shared by the two CPU oracles (test infrastructure only):
 *   oracle/_ref/libref*.so  - the reference's own sources (jiaweichiu/mpsft,
 *                             src/*.cc) compiled here against project-written
 *                             stand-in headers, wrapped by ref_capi.cc;
 *   oracle/liboracle.so     - this project's restatement, mpsft_oracle.cc.
 * Both export exactly these symbols so that tests can drive either one, and
 * compare them, through the same Python wrapper (oracle/oracle.py).
 *
 * Complex arrays are interleaved (re, im) doubles. A bin matrix is
 * rows x bins complex values, row-major, rows = 1 + 2*bits. The random draws
 * (Transform, q) come from one global std::mt19937 with
 * std::uniform_int_distribution<int32_t>, as in src/base.cc:32-56.
 */
#ifndef MPSFT_ORACLE_CAPI_H_
#define MPSFT_ORACLE_CAPI_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* mps::RandomSeed / mps::RandomInt32 (src/base.cc:52-53). */
void orc_seed(int32_t seed);
int32_t orc_random_int32(void);
/* mps::RandomNormal (src/base.cc:55): std::normal_distribution<double> on the
 * same engine (RandomSeed reseeds the engine only, src/base.cc:52). */
double orc_random_normal(void);

/* NumBits (src/iterate.cc:30-42). */
int32_t orc_num_bits(int32_t n, int32_t bins);

/* Window (src/window.cc:28-81). Returns p; writes wt[0..p) (index order
 * t = 0, 1..p2, -p2..-1) when wt != NULL and cap >= p. */
int32_t orc_window(int32_t n, int32_t bins, double delta, double *wt,
                   int32_t cap);
double orc_window_sample_in_freq(int32_t n, int32_t bins, double delta,
                                 double xi);

/* Transform(n) drawn from the global RNG: out = {a, b, c, a_inv}
 * (src/integer.cc:44-49; power-of-two n uses odd a, see
 * ref_integer_override.cc). */
void orc_transform(int32_t n, int32_t *out);
/* a_inv of Transform(n, a, b, c) (src/integer.cc:51-56). */
int32_t orc_transform_inverse(int32_t n, int32_t a);

/* BinInTime::Create(type)->Run (src/binner.cc:58-521). Overwrites out. */
int orc_bin_in_time(int type, int32_t n, int32_t bins, int32_t bits,
                    double delta, int32_t a, int32_t b, int32_t c, int32_t q,
                    const double *x, double *out);

/* BinInFreq::Create(type)->Run (src/binner.cc:526-591). Subtracts from out
 * the window responses of the m modes (k0[i], coef[2i], coef[2i+1]). */
int orc_bin_in_freq(int type, int32_t n, int32_t bins, int32_t bits,
                    double delta, int32_t a, int32_t b, int32_t c, int32_t q,
                    const int32_t *k0, const double *coef, int32_t m,
                    double *out);

/* MatPencil (src/freqid.cc:27-48): u = {u0, u1, u2} interleaved; writes
 * sigma[0..2); returns the vote (1 = upper half). */
int orc_mat_pencil(const double *u, double *sigma);

/* Iterate (src/iterate.cc:80-176) with IterateOptions fields as arguments.
 * The mode map is passed in and out as (mm_k[i], mm_c[2i..2i+1]),
 * i < *mm_size <= mm_cap; on return it holds the updated map, sorted by k.
 * Returns 1 if something was found, 0 if not, -1 if mm_cap was too small. */
int orc_iterate(int32_t n, const double *x, int32_t bins, double window_delta,
                int32_t trials, double bin_threshold, double window_threshold,
                double sv_threshold, int bin_in_time_type,
                int bin_in_freq_type, int32_t *mm_k, double *mm_c,
                int32_t *mm_size, int32_t mm_cap);

/* Demo1::Run (src/demo1.cc:36-59) on the caller's signal x with
 * Demo1Options {trials, min_bins, window_delta, window_threshold,
 * max_stale_iter}; k is the sparsity, sigma the noise level used for the
 * thresholds. Seeds the global RNG with seed, then draws from it as it goes
 * (3 + trials draws per Iterate call, src/iterate.cc:92-104). Writes the
 * found modes sorted by k; returns their count, or -1 if cap was too small.
 * *iters receives the number of Iterate calls. */
int orc_demo1_run(int32_t n, const double *x, int32_t k, double sigma,
                  int32_t trials, int32_t min_bins, double window_delta,
                  double window_threshold, int32_t max_stale_iter,
                  int32_t seed, int32_t *out_k, double *out_c, int32_t cap,
                  int32_t *iters);

/* GenerateModeMap (src/gen.cc:27-39) on the global RNG: k distinct positions
 * RandomInt32() mod n with coefficients (RandomNormal(), RandomNormal())
 * normalised to modulus 1. Writes them sorted by position; returns k. */
int orc_generate_mode_map(int32_t n, int32_t k, int32_t *out_k, double *out_c);

/* Demo1's signal (src/demo1.cc:27-34) on the global RNG as it stands (seed it
 * first): GenerateModeMap (k modes), then GenerateXhat (xhat_kind 0,
 * src/gen.cc:55-75: unit normals rescaled so that the noise outside the
 * modes has energy sigma^2) or GenerateXhatAlt (xhat_kind 1, src/gen.cc:77-89),
 * then the unnormalised backward FFT. Writes x (n values) and the modes
 * sorted by position; returns k. Later draws continue the same stream, as
 * the reference's tests' Iterate calls do. */
int orc_demo_signal(int32_t n, int32_t k, double sigma, int xhat_kind,
                    double *x, int32_t *out_k, double *out_c);

/* Demo1::PostAnalyze (src/demo1.cc:61-112) for the spectrum xh (n values),
 * the true positions true_k and the found modes (found_k, found_c). out
 * receives {hit, hit_l1, hit_l2, miss, miss_l1, miss_l2, l1, l2, max_err}. */
void orc_post_analyze(int32_t n, const double *xh, const int32_t *true_k,
                      int32_t true_count, const int32_t *found_k,
                      const double *found_c, int32_t found_count, double *out);

#ifdef __cplusplus
}
#endif

#endif /* MPSFT_ORACLE_CAPI_H_ */
