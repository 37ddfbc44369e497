// Shared by the drop-in entry points: the calling thread's GPU context (one
// per host thread, created on first use on device $GLASS_GPU_DEVICE or 0), and
// the reference's way of failing (message on stderr, exit).
#pragma once
#include "../../include/glass_gb300.h"

// The reference's struct Wavelets (utils/src/glass_wavelet.h:25-75), restated
// field for field so that the drop-in entry points can read the grid from a
// caller's struct: the field order and types are the interface.
struct WaveletsLayout {
  int NF, NT;
  double cadence, dt, df;
  int frequency_steps, fdot_steps;
  double d_fdot;
  int oversample;
  double Omega, dOmega, domega, inv_root_dOmega, B, A, BW, deltaf;
  double *fdot, *window, *window_freq_forward;
  double norm;
  int N;
  double T;
  int kmin, kmax, imin, imax;
  int *n_table;
  double **table;
};

glass_gpu_ctx *dropin_ctx(const char *who);
[[noreturn]] void dropin_fail(const char *who);

// The calling thread's context with the wavelet grid of this WDM grid,
// segment (Tobs, t0) and orbit set up (kept while they stay the same).
glass_gpu_ctx *dropin_wavelet_grid(struct Orbit *orbit, struct Wavelets *wdm, double Tobs, double t0,
                                   const char *who);
