/* mpsft-gb300: C ABI of a GB300 (sm_103a) implementation of the Matrix
 * Pencil Sparse Fourier Transform recovery loop of jiaweichiu/mpsft.
 *
 * Every entry point returns an int status (MPSFT_OK = 0). Nothing aborts: the
 * reference's glog CHECKs become status codes, and mpsft_last_error() gives the
 * message of the last failure on a context. All sizes are plain integers and
 * all buffers plain pointers; complex arrays are interleaved (re, im).
 *
 * Threading: one context per host thread. A context owns one CUDA stream
 * (or borrows the caller's, mpsft_ctx_set_stream) and its work buffers.
 *
 * Reference interfaces replaced (file:line in jiaweichiu/mpsft):
 *   mpsft_bin_in_time   BinInTime::Run         src/binner.h:30-41, src/binner.cc:394-521
 *   mpsft_bin_in_time_wt  the same, windowed by the binner's own Window table
 *                       (src/binner.h:30-38, src/window.h:27-32)
 *   mpsft_bin_in_freq   BinInFreq::Run         src/binner.h:123-133, src/binner.cc:565-591
 *   mpsft_bin_in_freq_wf  the same, with Window::SampleInFreq's responses given
 *                       (src/binner.cc:575-580, src/window.cc:77-81)
 *   mpsft_iterate_draws Iterate on the caller's Transform and q draws
 *                       (src/iterate.cc:92-104, src/integer.h:75-82)
 *   mpsft_mat_pencil    MatPencil              src/freqid.h:28, src/freqid.cc:27-48
 *   mpsft_iterate       Iterate                src/iterate.h:65, src/iterate.cc:80-176
 *   mpsft_solve         Demo1::Run             src/demo1.h:39, src/demo1.cc:36-59
 *   mpsft_solve_batched (no counterpart: many Demo1::Run solves in one launch sequence)
 *   mpsft_solve_batched_packed  the same, results of all signals in one pair of arrays
 *   mpsft_window_*      Window                 src/window.h:25-55, src/window.cc:28-81
 *   mpsft_rng_*         RandomSeed/RandomInt32 src/base.h:61-62, src/base.cc:52-53
 *   mpsft_num_bits      NumBits                src/iterate.cc:30-42
 */
#ifndef MPSFT_GB300_H_
#define MPSFT_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  MPSFT_OK = 0,
  MPSFT_ERR_INVALID = 1,       /* bad argument (even bins, trials even, ...)  */
  MPSFT_ERR_UNSUPPORTED_N = 2, /* n must be prime or a power of two           */
  MPSFT_ERR_CUDA = 3,          /* a CUDA runtime call failed                  */
  MPSFT_ERR_CAPACITY = 4,      /* found-mode table or output buffer too small */
  MPSFT_ERR_ITER_CAP = 5,      /* iteration cap reached before the stop rule  */
  MPSFT_ERR_NONFINITE = 6,     /* NaN or Inf met in the bins                  */
  MPSFT_ERR_NOMEM = 7          /* device allocation failed                    */
};

/* ---- element types and precisions -------------------------------------- */
enum { MPSFT_C64 = 1, MPSFT_C128 = 2 };
/* FP32: binning, fold (compensated) and size-B FFT in FP32; mode subtraction,
 *       pencil, thresholds and coefficients in FP64.
 * FP64: everything in FP64 (the plain per-signal path). */
/* FP64_DIRECT (mpsft_bin_in_time only): every bin as a direct sum over the
 * window support, without the fold and the size-B FFT (the evaluation the
 * FP32 path uses for its near-tie bins): float-float products and 64-sample
 * block sums (about 2^-47 relative), block totals in FP64; slow, for
 * checking. */
enum { MPSFT_PREC_FP32 = 0, MPSFT_PREC_FP64 = 1, MPSFT_PREC_FP64_DIRECT = 2 };

typedef struct mpsft_ctx mpsft_ctx;
typedef struct mpsft_signal mpsft_signal;
typedef struct mpsft_rng mpsft_rng;

/* ---- context ------------------------------------------------------------ */
int mpsft_ctx_create(int device, mpsft_ctx **out);
int mpsft_ctx_destroy(mpsft_ctx *ctx);
/* Launch on the caller's CUDA stream (cudaStream_t) instead of the context's
 * own; NULL restores the context's stream. */
int mpsft_ctx_set_stream(mpsft_ctx *ctx, void *stream);
/* Time every binning-kernel launch with CUDA events (0 = off, default). The
 * totals are reported in mpsft_stats. */
int mpsft_ctx_set_profiling(mpsft_ctx *ctx, int enable);
/* One timed binning launch (gather, window, modulate, fold) of a call made
 * with profiling on. */
typedef struct {
  int32_t iteration;  /* iteration of the call's loop (0 = the first)        */
  int32_t signals;    /* signals the launch binned                           */
  int32_t max_bins;   /* largest and smallest bins among them                */
  int32_t min_bins;
  int32_t precision;  /* MPSFT_PREC_FP32 or MPSFT_PREC_FP64 (the FP64 kernels */
                      /* that an FP32 call runs for the signals its          */
                      /* precision policy sends there)                       */
  int64_t gathers;    /* samples the launch gathered (the FP32 kernels read  */
                      /* each sample of overlapping row windows once)        */
  int64_t bytes;      /* algorithmic bytes: 32 (one sector) per sample of    */
                      /* every row's window, as the reference reads them     */
                      /* (p per row), + the window table + the fold output   */
  double ms;          /* duration from CUDA events around the launch         */
} mpsft_bin_launch;
/* The binning launches of the context's last call made with profiling on, in
 * launch order: writes min(cap, total) records to out and the total to
 * *count. */
int mpsft_ctx_bin_launches(const mpsft_ctx *ctx, mpsft_bin_launch *out,
                           int32_t cap, int32_t *count);
/* Solve-graph timeline (0 = off, default): with it on, the iteration kernels
 * of a solve graph record their kernel id and the device clock when their
 * first block starts. mpsft_ctx_timeline gives the last solve's records in
 * start order (kernel[j]: 1 plan, 2 window32, 3 fold, 4 Bluestein tables,
 * 5 mode preparation, 6 bucketing, 7 row transform, 8 decisions, 9 listed
 * bins' mode terms, 10 merge, 11 re-binning, 12 listed bins' FP64
 * decisions, 13 stop rule, 14 FP64 window; us[j] microseconds after the
 * first) and their number (at most 16384). */
int mpsft_ctx_set_timeline(mpsft_ctx *ctx, int enable);
int mpsft_ctx_timeline(const mpsft_ctx *ctx, int32_t *kernel, double *us,
                       int32_t cap, int32_t *count);
const char *mpsft_last_error(const mpsft_ctx *ctx);
const char *mpsft_status_string(int status);

/* ---- random draws (the reference's global RNG, made explicit) ----------- */
/* std::mt19937 with std::uniform_int_distribution<int32_t> over
 * [0, 2^31 - 1]; mpsft_rng_create(123534) is the state MainInit leaves. */
int mpsft_rng_create(int32_t seed, mpsft_rng **out);
int mpsft_rng_destroy(mpsft_rng *rng);
/* Reseeds the engine only, as RandomSeed does: a normal draw held back by
 * the normal distribution (the second of a pair) survives the reseed. */
int mpsft_rng_seed(mpsft_rng *rng, int32_t seed);
/* rngs[i] reseeded with seeds[i], i < count (mpsft_rng_seed each). */
int mpsft_rng_seed_many(mpsft_rng *const *rngs, const int32_t *seeds, int32_t count);
int32_t mpsft_rng_int32(mpsft_rng *rng);
/* count draws of std::normal_distribution<double> on the same engine (the
 * reference's RandomNormal, src/base.cc:55), into out or discarded (out =
 * NULL): positions the stream after the reference's signal construction. */
int mpsft_rng_normals(mpsft_rng *rng, int64_t count, double *out);

/* ---- small host helpers -------------------------------------------------- */
/* NumBits: 1 + floor(log2(n / bins)) counted by halving (1 if n < bins). */
int32_t mpsft_num_bits(int32_t n, int32_t bins);
/* Window support p for (bins, delta); 0 on bad arguments. */
int32_t mpsft_window_support(int32_t n, int32_t bins, double delta);
/* Window tables computed on the device: wt[i] for i in [0, p) in the
 * reference's index order t = 0, 1..p2, -p2..-1 (host output). */
int mpsft_window_table(mpsft_ctx *ctx, int32_t n, int32_t bins, double delta,
                       double *wt_host, int32_t cap);

/* ---- signals (x resident on the device across calls) -------------------- */
/* Copies n complex samples of type dtype from host memory. */
int mpsft_signal_upload(mpsft_ctx *ctx, const void *x_host, int64_t n,
                        int dtype, mpsft_signal **out);
/* Wraps n samples already in device memory (not copied, not freed). */
int mpsft_signal_wrap_device(mpsft_ctx *ctx, const void *x_device, int64_t n,
                             int dtype, mpsft_signal **out);
int mpsft_signal_free(mpsft_signal *sig);
/* Copies n new samples (the signal's own n and dtype) from host memory into
 * an existing signal; pinned host memory makes the copy asynchronous with
 * respect to the host until the next solve call. */
int mpsft_signal_write(mpsft_ctx *ctx, mpsft_signal *sig, const void *x_host);
/* Copies the signal's n samples (its dtype) to host memory; returns when
 * they are there. */
int mpsft_signal_read(mpsft_ctx *ctx, const mpsft_signal *sig, void *x_host);

/* mpsft_signal_write for count signals in one call, enqueued on stream (a
 * cudaStream_t; NULL = the context's stream). The call touches no context
 * state (errors are returned, not recorded as the context's last error), so
 * a second host thread may issue the next batch's copies on its own stream
 * while a solve of the same context runs; the caller orders the solve after
 * the copies (an event recorded on stream). */
int mpsft_signal_write_many(mpsft_ctx *ctx, mpsft_signal *const *sigs,
                            const void *const *x_host, int32_t count,
                            void *stream);

/* ---- BinInTime::Run ------------------------------------------------------- */
/* Overwrites out with the (1 + 2*bits) x bins bin matrix of signal sig for the
 * transform (a, b, c) and offset q: row 0 is tau = q, row 2s+1 is
 * q + bins*2^s, row 2s+2 is q - bins*2^s. out is host memory of complex128
 * (out_on_device = 0) or device memory (out_on_device = 1), row-major. */
int mpsft_bin_in_time(mpsft_ctx *ctx, const mpsft_signal *sig, int32_t bins,
                      int32_t bits, double delta, int32_t a, int32_t b,
                      int32_t c, int32_t q, int precision, double *out,
                      int out_on_device);

/* BinInTime::Run of a binner built from the reference's Window
 * (src/binner.h:30-38: BinInTime(const Window &win, int32_t bits)): the
 * window is the Window's own table, wt = Window::wt() (src/window.h:32), p =
 * Window::p(), in its index order t = 0, 1..p2, -p2..-1; the window's delta
 * (private to Window) is not needed. p must be an odd multiple of bins and the
 * table even (wt[p - i] == wt[i]), as Window builds it. FP64 precisions bin
 * with the table as given, FP32 with it rounded to FP32. Otherwise as
 * mpsft_bin_in_time. */
int mpsft_bin_in_time_wt(mpsft_ctx *ctx, const mpsft_signal *sig, int32_t bins,
                         int32_t bits, int32_t p, const double *wt, int32_t a,
                         int32_t b, int32_t c, int32_t q, int precision,
                         double *out, int out_on_device);

/* ---- BinInTime::Run without device allocation --------------------------- */
/* No counterpart in the reference. The same bins as mpsft_bin_in_time, for
 * callers that cannot call cudaMalloc (a caller-managed memory pool, a plugin
 * host that forbids allocation after start-up): x_device (n samples of dtype)
 * and out_device ((1 + 2*bits) x bins complex128, row-major) are the caller's
 * device memory, and the work runs asynchronously on stream (a cudaStream_t;
 * NULL = the legacy default stream). Scratch is one fixed array of about
 * 2.5 MiB compiled into the library and held on every GPU that loads it.
 * Limits: bins <= 2047, bits <= 20, window folds p/bins <= 80; larger sizes
 * return MPSFT_ERR_CAPACITY. n must be prime or a power of two, as for
 * mpsft_bin_in_time (MPSFT_ERR_UNSUPPORTED_N otherwise). Every call resolves
 * the array's address on the current device (cudaGetSymbolAddress, which
 * allocates nothing) and passes its descriptor as a kernel argument, so it
 * copies nothing from host memory; the FFT twiddle table in the array is
 * filled on the device by the first call after the library's device code is
 * loaded. Calls share the array, so calls that overlap on the GPU race; calls
 * on one stream are ordered and safe. */
int mpsft_bin_in_time_noalloc(const void *x_device, int64_t n, int dtype,
                              int32_t bins, int32_t bits, double delta,
                              int32_t a, int32_t b, int32_t c, int32_t q,
                              int precision, double *out_device, void *stream);

/* ---- BinInFreq::Run ------------------------------------------------------- */
/* Subtracts from the host bin matrix inout ((1 + 2*bits) x bins complex128)
 * the window responses of the m modes (k0[i], coef[2i] + i coef[2i+1]). */
int mpsft_bin_in_freq(mpsft_ctx *ctx, int32_t n, int32_t bins, int32_t bits,
                      double delta, int32_t a, int32_t b, int32_t c, int32_t q,
                      const int32_t *k0, const double *coef, int64_t m,
                      double *inout);

/* BinInFreq::Run of a binner built from the reference's Window
 * (src/binner.h:123-133): wf[i] is mode i's window response
 * Window::SampleInFreq(xi_i) (src/window.cc:77-81) at xi_i =
 * (bin_i + 1/2)/bins - k1_i/n, k1_i = (a k0[i] + b) mod n, bin_i =
 * floor(k1_i bins / n) (src/binner.cc:571-575), evaluated by the caller's
 * Window, so that no window delta is needed. Each mode's term is
 * wf[i] coef_i e^{2 pi i (q k1_i + c k0[i])/n} (src/binner.cc:577-580), times
 * the row factors. Otherwise as mpsft_bin_in_freq. */
int mpsft_bin_in_freq_wf(mpsft_ctx *ctx, int32_t n, int32_t bins, int32_t bits,
                         int32_t a, int32_t b, int32_t c, int32_t q,
                         const int32_t *k0, const double *coef, const double *wf,
                         int64_t m, double *inout);

/* ---- coefficient estimation for a fixed frequency set, and its adjoint ---
 * No entry point of the reference corresponds: these expose, as a linear map
 * of x, the coefficient estimate of Iterate (src/iterate.cc:146-171) with the
 * identified frequencies held fixed (no identification, no subtraction of
 * other modes), and its adjoint (for gradients through the estimate). For
 * each given k0 (k1 = (a k0 + b) mod n, beta = floor(k1 bins / n),
 * xi0 = k1/n - (beta + 1/2)/bins, rows tau = q_t, q_t +- bins 2^s):
 *   c(k0) = e^{-2 pi i c k0/n} / (wf(xi0) trials (1 + 2 bits))
 *           * sum_t sum_rows U_{t,row}[beta] e^{-2 pi i tau k1 / n}
 * with U the FP64 bins of mpsft_bin_in_time. FP64 throughout. */
typedef struct {
  int32_t bins;            /* odd                                          */
  int32_t bits;            /* rows = 1 + 2 bits                           */
  int32_t trials;          /* 1 .. 15                                      */
  double window_delta;
  int32_t a, b, c;         /* the transform of the estimate               */
  int32_t q[15];           /* q of each trial                              */
} mpsft_estimate_setup;

/* c = A x: writes coef[2i], coef[2i+1] (host) for the m given k0. */
int mpsft_estimate(mpsft_ctx *ctx, const mpsft_signal *sig,
                   const mpsft_estimate_setup *setup, const int32_t *k0,
                   int64_t m, double *coef);

/* dx = A^H g for a signal of length n: g[2i], g[2i+1] (host, m entries) is
 * the gradient with respect to c(k0[i]) in the conjugate-Wirtinger
 * convention (torch's); writes dx[2j], dx[2j+1] (host, n entries). */
int mpsft_adjoint(mpsft_ctx *ctx, int32_t n, const mpsft_estimate_setup *setup,
                  const int32_t *k0, int64_t m, const double *g, double *dx);

/* ---- MatPencil (batched) -------------------------------------------------- */
/* For each i < count: the 2x2 pencil [[u0, u2], [u1, u0]] with
 * u = (u0, u1, u2) = u3[6i .. 6i+6) (interleaved complex); writes
 * sigma[2i], sigma[2i+1] and vote[i] (1 = upper half). Host buffers. */
int mpsft_mat_pencil(mpsft_ctx *ctx, const double *u3, int64_t count,
                     double *sigma, int32_t *vote);

/* ---- Iterate -------------------------------------------------------------- */
typedef struct {
  int32_t bins;            /* odd number of bins B                          */
  double window_delta;     /* reference default 1e-6                        */
  int32_t trials;          /* odd; reference default 1                      */
  double bin_threshold;    /* 0 = off                                       */
  double window_threshold; /* must be > 0, as in the reference              */
  double sv_threshold;     /* 0 = off                                       */
  int32_t precision;       /* MPSFT_PREC_FP32 or MPSFT_PREC_FP64            */
  double near_tie_margin;  /* FP32: decisions closer to their threshold     */
                           /* than margin * 2^-24 * (bin rms) are near ties */
                           /* (0 = default 256)                             */
} mpsft_iterate_options;

/* One Iterate call: draws (a, b, c) and one q per trial from rng, bins the
 * signal, subtracts the modes already in the map, identifies and estimates.
 * The mode map is passed in and out as (mm_k[i], mm_c[2i..2i+1]),
 * i < *mm_size <= mm_cap (host memory); on return it is sorted by k.
 * *found = 1 if something was added. */
int mpsft_iterate(mpsft_ctx *ctx, const mpsft_signal *sig,
                  const mpsft_iterate_options *opt, mpsft_rng *rng,
                  int32_t *mm_k, double *mm_c, int32_t *mm_size,
                  int32_t mm_cap, int32_t *found);

/* mpsft_iterate with the draws made by the caller: the transform as the
 * reference's Transform holds it (a, b, c, a_inv; src/integer.h:75-82, drawn
 * by Transform(n), src/integer.cc:44-49) and q[t] for each of opt->trials
 * trials (RandomInt32() % n, src/iterate.cc:102-104), all in [0, n). a_inv is
 * used as given (k0 = a_inv (k1 - b) mod n, src/iterate.cc:169), as the
 * reference does. This is the drop-in for Iterate driven by the reference's
 * own global RNG. */
int mpsft_iterate_draws(mpsft_ctx *ctx, const mpsft_signal *sig,
                        const mpsft_iterate_options *opt, int32_t a, int32_t b,
                        int32_t c, int32_t a_inv, const int32_t *q,
                        int32_t *mm_k, double *mm_c, int32_t *mm_size,
                        int32_t mm_cap, int32_t *found);

/* ---- Demo1::Run ------------------------------------------------------------ */
typedef struct {
  int32_t k;               /* sparsity S used to size the bins              */
  double sigma;            /* noise level: bin_threshold = 3 sigma/sqrt(B), */
                           /* sv_threshold = sigma/sqrt(B)                  */
  int32_t trials;          /* odd                                           */
  int32_t min_bins;        /* reference default 101 (benchmarks: 51)        */
  double window_delta;     /* reference default 1e-6 (benchmarks: 1e-5)     */
  double window_threshold; /* reference default 0.1                         */
  int32_t max_stale_iter;  /* reference default 3 (benchmarks: 5)           */
  int32_t max_iter;        /* cap on Iterate calls; 0 = 64 + 8*k            */
  int32_t precision;       /* MPSFT_PREC_FP32 or MPSFT_PREC_FP64            */
  int32_t mode_capacity;   /* found-mode table size; 0 = automatic          */
  double near_tie_margin;  /* as in mpsft_iterate_options (0 = default)     */
} mpsft_solve_options;

/* Fills opt with the reference's Demo1Options defaults (src/demo1.h:25-33)
 * and FP32 precision; k and sigma must still be set. */
void mpsft_solve_options_default(mpsft_solve_options *opt);

typedef struct {
  int32_t iterations;     /* Iterate calls made                              */
  int32_t found;          /* distinct modes in the result                    */
  int64_t gathers;        /* samples gathered by the binning kernel          */
  int64_t bin_bytes;      /* algorithmic bytes of the binning launches (32   */
                          /* per sample of every row's window, p per row)    */
  int32_t bin_launches;   /* binning launches timed (profiling on)           */
  double bin_ms;          /* summed binning-kernel time (profiling on)       */
  int32_t escalated;      /* FP32 near-tie escalations to FP64 (bins)        */
  int32_t status;         /* per-signal status (batched calls)               */
  int64_t kernel_launches;/* CUDA kernels launched by the call               */
  int32_t unresolved;     /* iterations whose FP32 near ties could not be    */
                          /* redone in FP64 (bins > 4096); 0 otherwise       */
  int32_t fp64_iterations;/* FP32 path: iterations run on the FP64 kernels   */
                          /* because rounding was not small against noise    */
  double loop_ms;         /* device time of the call's iteration loop (from  */
                          /* the first iteration's start to the last one's   */
                          /* end; the rest of the call is setup and results) */
} mpsft_stats;

/* One full recovery (the Demo1::Run loop) of sig. Draws 3 + trials values
 * from rng per Iterate call, in the reference's order. Writes up to cap
 * found modes sorted by k (host memory) and their count. */
int mpsft_solve(mpsft_ctx *ctx, const mpsft_signal *sig,
                const mpsft_solve_options *opt, mpsft_rng *rng,
                int32_t *out_k, double *out_c, int32_t cap, int32_t *count,
                mpsft_stats *stats);

/* Many independent recoveries advanced together, one iteration of every
 * active signal per launch sequence. Signal i uses opts[i] and rngs[i]
 * (all precisions must agree) and writes out_k[i], out_c[i] (cap[i] entries)
 * and count[i]. stats may be NULL; otherwise it has nsig entries. */
int mpsft_solve_batched(mpsft_ctx *ctx, const mpsft_signal *const *sigs,
                        const mpsft_solve_options *opts, int32_t nsig,
                        mpsft_rng *const *rngs, int32_t *const *out_k,
                        double *const *out_c, const int32_t *cap,
                        int32_t *count, mpsft_stats *stats);

/* mpsft_solve_batched with every signal's results in one pair of arrays:
 * signal i's modes (sorted by k) at [offsets[i], offsets[i + 1]) of out_k
 * and out_c (out_cap entries in all; offsets has nsig + 1 entries). A signal
 * whose modes do not fit in what is left gets MPSFT_ERR_CAPACITY, its
 * stored prefix and its full count in count[i]. */
int mpsft_solve_batched_packed(mpsft_ctx *ctx, const mpsft_signal *const *sigs,
                               const mpsft_solve_options *opts, int32_t nsig,
                               mpsft_rng *const *rngs, int32_t *out_k, double *out_c,
                               int64_t out_cap, int64_t *offsets, int32_t *count,
                               mpsft_stats *stats);

/* ---- autotuner of the FP32 binning's launch shape ------------------------
 * No counterpart in the reference (its binning shapes are fixed by the caller,
 * src/binner_bench.cc:28-33). The FP32 fold has mpsft_fold_shape_count()
 * launch shapes: threads sharing a bin (2, 4, 8) and folds in flight per
 * thread (4, 8) of the row pairs, with the row cluster (row 0 and the pairs
 * whose windows overlap, each sample gathered once) on or off; every shape
 * computes the same sums up to FP32 rounding, so the frequency sets are the
 * same. A context keeps a table: key (ceil(log2 bins), ceil(log2 n),
 * ceil(log2 signals per launch), complex128 input) -> shape, bins being those
 * a solve sizes its launches for (the batch's largest, or 4 min_bins + 1 once
 * every signal needs at most that many); launches whose key is not in the
 * table use shape 0. */
int32_t mpsft_fold_shape_count(void);
/* Times every shape on one batched FP32 solve of these signals (each shape
 * repeats times, the draws from RNGs seeded seed + i, the caller's RNGs
 * untouched), CUDA events around every binning launch, and records for each
 * bins class of the solve's launches the shape with the least total time. */
int mpsft_autotune(mpsft_ctx *ctx, const mpsft_signal *const *sigs,
                   const mpsft_solve_options *opts, int32_t nsig, int32_t seed,
                   int32_t repeats);
/* The table as text (one line per key: bins_log2 n_log2 signals_log2
 * complex128 shape microseconds); load replaces the context's table. */
int mpsft_tuning_save(mpsft_ctx *ctx, const char *path);
int mpsft_tuning_load(mpsft_ctx *ctx, const char *path);
int32_t mpsft_tuning_size(const mpsft_ctx *ctx);
/* Every FP32 binning launch of the context uses shape (-1 = the table's
 * choice, the default). */
int mpsft_ctx_set_fold_shape(mpsft_ctx *ctx, int32_t shape);

/* ---- test data and result analysis (Demo1's constructor and PostAnalyze) -- */
/* GenerateModeMap (src/gen.cc:27-39) on rng: count distinct positions
 * k = RandomInt32() mod n, each with coefficient (RandomNormal(),
 * RandomNormal()) / |.|, drawn in the reference's order from rng's one
 * engine. Writes out_k[count] (in draw order) and out_c[2 count]
 * (interleaved). Host only. */
int mpsft_generate_mode_map(mpsft_rng *rng, int32_t n, int32_t count,
                            int32_t *out_k, double *out_c);

/* A signal generated on the device: x_t = sum_j coef_j e^{2 pi i k_j t / n}
 * + noise_t, the unnormalised backward FFT of the spectrum that
 * GenerateXhatAlt builds (src/gen.cc:77-89, src/demo1.cc:27-34). The mode
 * part is an FP64 inverse FFT (cuFFT Z2Z, loaded at first use) of the
 * sparse spectrum; noise_t is complex Gaussian with E|noise_t|^2 = sigma^2
 * (real and imaginary parts N(0, sigma^2 / 2)), the time-domain form of
 * GenerateXhatAlt's per-frequency variance sigma^2 / n, from a
 * counter-based generator keyed by seed: sample t takes outputs 2t and 2t+1
 * of the SplitMix64 sequence started at seed (u = ((z >> 11) + 1) 2^-53) through
 * the Box-Muller transform. The values differ from the reference's
 * sequential mt19937 draws; the distribution is the same. k must be distinct
 * positions in [0, n); coef is interleaved (re, im); dtype MPSFT_C64 or
 * MPSFT_C128 (the sum is formed in FP64, then rounded). */
int mpsft_signal_generate(mpsft_ctx *ctx, int64_t n, const int32_t *k,
                          const double *coef, int64_t count, double sigma,
                          uint64_t seed, int dtype, mpsft_signal **out);

/* xhat = FFT(x) / n of a resident signal in FP64 (cuFFT Z2Z forward):
 * out receives n complex128 values, interleaved, in host or device memory
 * (any pointer the CUDA runtime can address). */
int mpsft_signal_spectrum(mpsft_ctx *ctx, const mpsft_signal *sig, double *out);

/* Demo1::PostAnalyze (src/demo1.cc:61-112), computed on the device. */
typedef struct {
  int32_t hit;       /* found positions that are true positions */
  int32_t miss;      /* the other found positions */
  double hit_l1;     /* mean |c - xhat_k| over the hits (NaN when none) */
  double hit_l2;     /* sqrt(mean |c - xhat_k|^2) over the hits */
  double miss_l1;    /* the same over the misses */
  double miss_l2;
  double l1;         /* over all n frequencies, the found spectrum (c at */
  double l2;         /* found positions, 0 elsewhere) against xhat: mean, */
  double max_err;    /* root mean square and maximum of |difference| */
} mpsft_analysis;

/* Compares found modes (found_k distinct, found_c interleaved) with the true
 * positions true_k and with the signal's spectrum xhat = FFT(x) / n (the
 * reference compares with the generated spectrum, of which the signal is
 * the exact backward transform). */
int mpsft_post_analyze(mpsft_ctx *ctx, const mpsft_signal *sig,
                       const int32_t *true_k, int64_t true_count,
                       const int32_t *found_k, const double *found_c,
                       int64_t found_count, mpsft_analysis *out);

#ifdef __cplusplus
}
#endif

#endif /* MPSFT_GB300_H_ */
