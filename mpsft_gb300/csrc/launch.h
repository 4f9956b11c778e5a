// Host-side launchers of the sm_103a kernels (one translation unit each).
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace mpsft {

// True while the calling thread captures a solve graph: the iteration
// kernels are then launched with programmatic stream serialization (each
// starts with PdlEnter), so that a kernel's launch overlaps the end of the
// kernel before it.
extern thread_local bool g_launch_pdl;

template <typename... P, typename... A>
inline void Launch(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem,
                   cudaStream_t s, A... args) {
  if (!g_launch_pdl) {
    kernel<<<grid, block, smem, s>>>(args...);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, static_cast<P>(args)...);
}

// The FFT twiddle table (kTwiddleEntries entries, TwiddleAt).
void LaunchTwiddles(float2 *tw32, double2 *tw64, cudaStream_t s);
// dst (device) = src_dev (device address of pinned, mapped host memory), any
// alignment and size.
void LaunchCopyMapped(const void *src_dev, void *dst, size_t bytes, cudaStream_t s);
// A one-thread kernel that holds the stream for ns nanoseconds.
void LaunchDelay(unsigned long long ns, cudaStream_t s);

// FP64 unit-phase tables ph_lo / ph_hi of every signal (n and the table
// pointers set); entries = the largest table length of the signals.
void LaunchPhaseTables(const SigIter *d_its, int nsig, int64_t entries,
                       cudaStream_t s);
inline int64_t PhaseTableEntries(int64_t n) {
  const int64_t lo = int64_t(1) << PhaseTableK(n);
  const int64_t hi = PhaseTableHi(n);
  return lo > hi ? lo : hi;
}

// Window tables at |t| in [0, p2] of every active signal: LaunchWindow
// evaluates in FP64 and fills wt64, wtff and wt32 (rounded); the FP32 path
// splits this into LaunchWindow32 (wt32 evaluated in FP32, for the binning)
// and LaunchWindow64 (wt64 and wtff, on a side stream).
void LaunchWindow(const SigIter *d_its, int nsig, int max_p2, cudaStream_t s);
void LaunchWindow32(const SigIter *d_its, int nsig, int max_p2, cudaStream_t s);
void LaunchWindow64(const SigIter *d_its, int nsig, int max_p2, cudaStream_t s);

// Bluestein chirp and FFT(conjugate chirp) of every active signal.
// fp64 selects double tables.
// cond: only signals whose iteration is redone in FP64 (more near-tie bins
// than their list holds) take part (here and in the launchers below).
void LaunchBluesteinSetup(const SigIter *d_its, int nsig, int max_m, bool fp64,
                          const float2 *tw32, const double2 *tw64,
                          cudaStream_t s, bool cond = false);

// Launch shapes of the FP32 fold (the autotuner's choices): threads per bin
// (split) and folds in flight per thread (batch) of the pair groups, the row
// cluster on or off; shape 0 is the default.
constexpr int kFoldShapes = 12;
struct FoldShape {
  int split, batch, bins_per_cta;
  bool cluster;
};
FoldShape FoldShapeOf(int shape);

// Fold of the windowed, modulated, permuted samples (the time-domain part of
// BinInTime::Run). x_c128 selects double2 input, fp64 the FP64 arithmetic,
// shape the FP32 launch shape.
void LaunchBinFold(const SigIter *d_its, int nsig, int max_bins, int max_bits,
                   int max_trials, bool x_c128, bool fp64, cudaStream_t s,
                   bool cond = false, int shape = 0);

// Size-B FFT of every folded row, times e^{2 pi i b q / n}, into ubuf.
void LaunchRowFFT(const SigIter *d_its, int nsig, int max_rows,
                  int max_trials, int max_m, bool fp64, const float2 *tw32,
                  const double2 *tw64, cudaStream_t s, bool cond = false);

// Per found mode: k1, bin, window response and the per-trial row-0 term
// (FP32 terms on the FP32 path, FP64 terms on the FP64 path and for signals
// the FP32 path runs on its FP64 kernels; cond: only those redone in FP64).
void LaunchModePrep(const SigIter *d_its, int nsig, int max_cap, cudaStream_t s,
                    bool cond = false);

// Empty mode tables and control words of every signal.
void LaunchClearTables(const SigIter *d_its, int nsig, int max_cap,
                       cudaStream_t s);
// Occupied table entries of every signal, packed: signal s to keys / coefs
// [o_s, o_s + counts[s]) with o_s = counts[0] + ... + counts[s - 1], sorted by
// k0 (sorted[s] = 1; 0: insertion order, the table exceeded half its
// capacity). max_cap: the largest table capacity.
void LaunchExportTables(const SigIter *d_its, int nsig, int max_cap,
                        int32_t *keys, double2 *coefs, int32_t *counts,
                        int32_t *sorted, cudaStream_t s);

// mean |x|^2 of each signal into energy[sig * kEnergyStride] (two
// deterministic passes): over every sample (per_block = 0), or estimated
// from kEnergyBlocks evenly spread runs of per_block samples.
constexpr int kEnergyBlocks = 256;
constexpr int kEnergyStride = kEnergyBlocks + 1;
void LaunchEnergy(const void *const *x, const int64_t *n, int nsig, bool c128,
                  double *energy, cudaStream_t s, int per_block = 0);

// Lists of table slots per bin (counting sort by bin); prep: the mode
// preparation of LaunchModePrep first, in the same kernel.
void LaunchBucket(const SigIter *d_its, int nsig, int max_bins, int max_cap,
                  cudaStream_t s, bool prep = false);

// Per-bin mode subtraction, energy test, pencil votes and coefficient
// estimation (the bin loop of Iterate); writes the candidates. With
// subtract_only, only the mode subtraction of BinInFreq::Run is applied to
// ubuf in place.
// mark_listed: the FP32 pass holds its listed bins back from the merge
// (cand_valid + kCandListed); their FP64 decision merges them.
void LaunchDecide(const SigIter *d_its, int nsig, int max_bins, int max_trials,
                  bool fp32, bool subtract_only, cudaStream_t s,
                  bool cond = false, bool mark_listed = false);

// Re-binning of the near-tie bins listed by the FP32 decide pass (direct sums
// over the window support in float-float arithmetic with FP64 block totals).
// prepare: run the listed bins' preparation first (a solve's decide kernel
// prepares the bins it lists itself). max_listed: the largest esc_cap.
void LaunchRebin(const SigIter *d_its, int nsig, int max_listed, bool x_c128,
                 bool prepare, cudaStream_t s);
// FP64 decisions of the listed bins on their re-binned rows. redo: the
// conditional FP64 kernels follow (signals whose list overflowed are redone
// whole); without them such signals are reported unresolved.
// merge: each decided bin goes into the table right away (the other bins'
// merge runs beside the re-binning).
void LaunchDecideListed(const SigIter *d_its, int nsig, int max_trials,
                        bool redo, bool merge, cudaStream_t s);

// Candidates -> mode table (mm[k0] += coef).
void LaunchMerge(const SigIter *d_its, int nsig, int max_bins, cudaStream_t s);
// FP64 row-0 terms of the listed near-tie bins' found modes and their sums
// in every row of the bin (esc_msub, for the FP64 decisions), beside the
// re-binning.
void LaunchListedTerms(const SigIter *d_its, int nsig, int max_trials, cudaStream_t s);

// The spilled candidates of each signal into its table (InsertSpills), for
// iterations that no k_finish follows.
void LaunchInsertSpills(const SigIter *d_its, int nsig, cudaStream_t s);

// Inserts / accumulates explicit (k0, coef) pairs into one signal's table.
void LaunchTableInsert(const SigIter *d_it, const int32_t *k0,
                       const double2 *coef, int64_t m, cudaStream_t s);

// Device-side control of a solve: iteration planning and the stop rule
// (sets the while condition of the solve graph when set_condition).
// k_plan runs signals needing at most max_bins bins (ahead: plans the
// iteration after the running one, for signals at fixed bins); k_finish
// continues the loop while a signal with work needs bins in
// (cond_lo, cond_hi] (exclude_fixed: and more than its min_bins), and drops
// the iteration planned ahead into its_ahead (if not null) of a signal that
// stopped.
void LaunchPlan(SolveCtl *ctl, SigIter *its, int nsig, int32_t max_bins,
                cudaStream_t s, bool ahead = false);
void LaunchFinish(SolveCtl *ctl, SigIter *its, int nsig,
                  cudaGraphConditionalHandle handle, bool set_condition,
                  int32_t cond_lo, int32_t cond_hi, cudaStream_t s,
                  SigIter *its_ahead = nullptr, bool exclude_fixed = false);

// Batched 2x2 pencils.
void LaunchPencil(const double2 *u3, int64_t count, double *sigma,
                  int32_t *vote, cudaStream_t s);

// Coefficient estimate of a fixed frequency set from the bins in ubuf
// (c = A x), and the pieces of its adjoint: spread g, conjugated, over the
// rows of the fold buffer (zeroed by the caller), then, after a row FFT with
// unit row factors into ubuf, scatter-add into dx (zeroed, n entries).
void LaunchEstimate(const SigIter *d_it, const int32_t *k0, int64_t m,
                    double2 *coef, cudaStream_t s);
void LaunchAdjointSpread(const SigIter *d_it, const int32_t *k0, const double2 *g,
                         int64_t m, cudaStream_t s);
void LaunchAdjointScatter(const SigIter *d_it, int64_t items, double2 *dx,
                          cudaStream_t s);

// Whether the kernels with large blocks or shared memory can be launched on
// the current device in their largest configuration (checked when a context
// is created, so that a resource limit fails loudly instead of silently
// skipping a launch).
bool WindowKernelsLaunchable();
bool FftKernelsLaunchable();
bool DecideKernelsLaunchable();
bool RebinKernelsLaunchable();
bool ControlKernelsLaunchable();

}  // namespace mpsft
