// Internal host-side interface of the Fourier-domain UCB kernels (ucb_fd.cu).
#pragma once
#include <cuda_runtime.h>

#include "glass_common.cuh"

namespace glass {

// Device-resident inputs shared by every evaluation of a segment bank.
struct FdBankDev {
  int nseg = 0, NFFT = 0, format = 0;
  double *rho = nullptr;       // [nseg*NFFT] invC_A / invC_E (F-statistic weights of the E channel)
  double T = 0, t0 = 0, fstar = 0;
  int *qmin = nullptr;         // [nseg]
  float4 *w32 = nullptr;       // [nseg*NFFT]   whitened residual {A.re, A.im, E.re, E.im}, rounded to float
  float4 *w32lo = nullptr;     // [nseg*NFFT]   residual minus its float rounding (double-float pair with w32)
  float4 *g32 = nullptr;       // [nseg*NFFT*2] {GA2, GA1}, {GE2, GE1}
  float4 *g32lo = nullptr;     // [nseg*NFFT*2] the same minus their float rounding
  double *Q = nullptr;         // [nseg*(NFFT+1)] prefix sums of |w|^2 over both channels (FP64)
  double *QA = nullptr;        // [nseg*(NFFT+1)] the same for the A channel alone
  double2 *w64 = nullptr;      // [nseg*NFFT*2] {A}, {E}
  double2 *g64 = nullptr;      // [nseg*NFFT*4] GA2, GA1, GE2, GE1
  float2 *invc = nullptr;      // [nseg*NFFT] invC_A, invC_E over their value at the segment's bin 0
                               // (weights of the reference-indexed Fisher matrix)
};

// Per-size tables (orbit samples and FFT twiddles) for the bank's (T, t0).
struct FdTablesDev {
  OrbitSample64 *pos64[kNumBins] = {};
  OrbitSampleMix *mix[kNumBins] = {};
  GeoSampleMix *geo[kNumBins] = {};
  GeoSampleMix *geolo[kNumBins] = {};  // the same minus its float rounding (double-float slow part)
  float2 *tw32[kNumBins] = {};
  float4 *tw32x[kNumBins] = {};  // the same twiddles as hi + lo floats (mixed likelihood)
  double2 *tw64[kNumBins] = {};
  void *base = nullptr;  // single allocation backing all of the above
};

// Scratch of one batched evaluation.
// ints in FdWorkDev::bin_count (see there)
constexpr int kFdCounts = 2 * kNumBins + 6;

struct FdWorkDev {
  // per-size streams forked from the caller's stream after the slow-part
  // kernel, so that the per-size spectral kernels run concurrently (and become
  // parallel branches when the caller captures a CUDA graph)
  cudaStream_t side[kNumBins] = {};
  cudaEvent_t fork = nullptr, join[kNumBins] = {};
  int cap = 0;                  // proposals
  size_t series_bytes = 0;      // capacity of `series`
  ItemF64 *items64 = nullptr;   // [cap]
  ItemMix *itemsmix = nullptr;  // [cap]
  ItemGrad *itemsgrad = nullptr;  // [cap]
  // [kFdCounts]: per-size counts, fb_count, the CTA-done counters of the
  // persistent spectral kernel and of the re-evaluation kernel, three spare
  // ints, and the re-evaluation's per-size counts (hp_count)
  int *bin_count = nullptr;
  int *bin_list = nullptr;      // [kNumBins*cap]
  // Mixed precision: proposals whose error estimate exceeds the tolerance are
  // listed by size in hp_list (counts in hp_count, their total in fb_count)
  // and evaluated again in double-float (series in series2), in the same
  // launch sequence (fb_e1 = fb_e2 = 0: no re-evaluation)
  float fb_e1 = 0.f, fb_e2 = 0.f;
  int *hp_list = nullptr;                  // [kNumBins*cap]
  int *hp_count = nullptr;                 // bin_count + kNumBins + 6
  int *fb_count = nullptr;                 // bin_count + kNumBins
  void *series2 = nullptr;                 // [series_bytes]: double-float series of the listed proposals
  unsigned long long *fb_total = nullptr;  // proposals re-evaluated
  float *fb_inv_scale = nullptr;           // [fb_nscale]: 1 / per-proposal tolerance scale (null: 1)
  int fb_nscale = 0, fb_nscale_cap = 0;
  // every launch sequence leaves the counts at zero (the spectral kernel's last
  // CTA, or a trailing memset), so the next one needs no leading memset; false
  // when that is not known (a launch returned an error part-way)
  bool counts_zero = false;
  // launch shapes of the mixed path, chosen by the autotuner
  // (glass_gb300/tune.py, glass_gpu_set_tuning); 0: the built-in choice
  struct Tuning {
    int slow_block = 256;         // slow-part threads per CTA (128, 256, 512)
    int slow_ctas_per_sm = 0;     // cap on resident slow-part CTAs per SM
    int spec_ctas_per_sm = 0;     // cap on persistent spectral CTAs per SM
    int plan_per_cta = 0;         // proposals per plan CTA (8 .. 32)
  } tune;
  void *series = nullptr;       // 4 arm-combination series per proposal
  // optional timing of each phase of a step on the caller's stream: events
  // before the plan kernel, after it, after the slow-part kernel, after the
  // spectral kernels and after the re-evaluations that follow them (timing
  // events; only when phase_timing is set)
  bool phase_timing = false;
  bool phase_recorded = false;
  cudaEvent_t phase[5] = {};
};

// Host-side table construction for a bank: G and w tables, prefix sums.
void fd_build_bank_tables(int format, double T, double fstar, int NFFT, int nseg, const int *qmin, const double *rA,
                          const double *rE, const double *invCA, const double *invCE, float4 *w32, float4 *w32lo,
                          float4 *g32, double *Q, double2 *w64, double2 *g64, double *QA = nullptr,
                          float4 *g32lo = nullptr);

cudaError_t fd_build_orbit_tables(FdTablesDev &tab, double T, double t0, cudaStream_t stream);

// Enqueue plan + per-size kernels.  Returns the number of kernel launches
// through *nlaunch.
cudaError_t fd_dlogl_launch(const FdBankDev &bank, const FdTablesDev &tab, FdWorkDev &work, int precision,
                            int nitems, const int *item_seg, const double *params, const double *term_x,
                            double *dlogl, double *term_y, double *hh, int *status, int n_fixed, int num_sms,
                            cudaStream_t stream, int *nlaunch, double *term_ch = nullptr);

// Bytes of series scratch a batch of nitems proposals on segments of NFFT bins
// can need (every N is at most NFFT).
size_t fd_series_bytes(int nitems, int NFFT, int precision);

// Gradient of delta logL and Fisher matrix (ucb_grad.cu).  Sizes up to 1024;
// larger templates get status GLASS_ITEM_NONFINITE.
size_t fd_grad_series_bytes(int nitems, int NFFT);
cudaError_t fd_grad_launch(const FdBankDev &bank, const FdTablesDev &tab, FdWorkDev &work, int nitems,
                           const int *item_seg, const double *params, int N_fixed, int fisher_mode, double *term_y,
                           double *grad, double *fisher, int *status, int num_sms, cudaStream_t stream,
                           int *nlaunch);

// F-statistic of sky/frequency cells (ucb_fstat.cu).  Scratch for up to `cap`
// cells per launch sequence, sized for the largest filter of the segment size.
struct FsWorkDev {
  int cap = 0;
  void *mem = nullptr;
  void *cells = nullptr;     // [cap] per-cell constants
  int *bin_count = nullptr;  // [16]
  int *bin_list = nullptr;   // [9*cap]
  void *series = nullptr;    // 16 series of N complex doubles per cell
  size_t series_bytes = 0;
};
size_t fs_cell_bytes();
int fs_max_size(int NFFT);
cudaError_t fs_work_alloc(FsWorkDev &w, int cap, int NFFT);
void fs_work_free(FsWorkDev &w);
// cells[4 c] = f0, fdot, theta, phi; outputs as glass_gpu_fstat_batch.  Runs
// the cells in chunks of w.cap.
// cell_seg may be null: every cell on segment seg_const.
cudaError_t fs_launch(const FdBankDev &bank, const FdTablesDev &tab, const double *rho, FsWorkDev &w, int ncells,
                      const int *cell_seg, int seg_const, const double *cells, double *logl, double *fparams,
                      int *status, int num_sms, cudaStream_t stream, int *nlaunch);

// The frequency x sky grid of build_fstatistic_proposal
// (ucb/src/glass_ucb_proposal.c:927-943, 1085-1182) and its chirp-mass scan.
constexpr int kFsScan = 10;  // chirp masses 0.1, 0.2, ... 1.0 (:1099-1100)
struct FsGrid {
  int n_f, n_theta, n_phi;
  double fmin, d_f, d_theta, d_phi;
};
cudaError_t fs_grid_cells(const FsGrid &G, int g0, int n, double *cells, cudaStream_t stream);
cudaError_t fs_scan_mark(const double *logl0, int n, int *count, int *active, int *pos, cudaStream_t stream);
cudaError_t fs_scan_cells(const FsGrid &G, const int *active, int c0, int n, const double *fdot_tab, double *cells,
                          cudaStream_t stream);
cudaError_t fs_finalize(const double *logl0, const int *pos, const double *scan, int n, double *tensor,
                        cudaStream_t stream);

// Single waveform in the reference's output layout (legacy ucb_waveform).
// pos: N orbit samples (device), item: the source's FP64 constants (device,
// from source_geometry + make_item_f64), d6: 6 N complex scratch, out: 10*N
// doubles (device) = X,Y,Z,A,E.  tw: the N-point FP64 twiddle table
// (FdTablesDev::tw64 of the size).
cudaError_t fd_waveform_launch(const OrbitSample64 *pos, const ItemF64 *item, int N, int format, int NI, double T,
                               double fstar, double2 *d6, double *out, const double2 *tw, cudaStream_t stream);


}  // namespace glass
