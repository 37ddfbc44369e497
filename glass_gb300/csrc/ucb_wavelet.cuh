// Wavelet-domain UCB waveform and sparse-pixel likelihood on the device.
// See ucb_wavelet.cu.
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace glass {

constexpr int kWvMaxOrb = 2048;  // orbit nodes (200 per year of observation)
constexpr int kWvMaxNT = 4096;   // pixels per layer
constexpr int kWvMaxLayers = 3;  // ucb_wavelet_layers gives 1..3 layers

// Per-source plan record, written by the plan kernel.
struct WvSrc {
  double k[3], ep[9], ec[9];
  double Ap, Ac, c2p, s2p;
  double fhet;
  int jmin, nl, jlo, c;  // first layer, layer count, first kept layer, kept layers per pixel time
  int status, pad;
};

// Device view of one wavelet segment: grid tables and data.
struct WvGridDev {
  int NF, NT, norb, kmin, kmax, N;  // N = kmax - kmin pixels
  int lmin, lmax;
  double Tobs, t0, wdt, wdf, A, norm_sqrtNF;
  const double *orb_t;    // [norb] orbit node times (even grid of the barycentre splines)
  const double *tssb;     // [norb] t0 + i Tobs/(norb-1) (grid of the TDI splines)
  const double *geo;      // [norb][21]: S/C positions / c (9), unit arms (9), arm lengths / c (3) at tssb
  const double *fac_orb;  // [3][norb]: h, l, mu of the spline system on orb_t
  const double *fac_ssb;  // [3][norb]: same on tssb
  const double *r0ds[kWvMaxLayers + 1];  // [NT (nl+1)][3] S/C 1 position / c at the downsampled times
  const double *win[kWvMaxLayers + 1];   // [NT/2 + 1] window of an (nl+1)-layer grid
  const double2 *tw[kWvMaxLayers + 1];   // [NT (nl+1)] e^{-2 pi i k / (NT (nl+1))}
  const double *res;      // [3][N] residual X, Y, Z
  const double *invC;     // [9][N] inverse noise covariance, [i][j][k]
  // mixed precision: FP32 twiddles and windows, the residual divided by the
  // segment's noise scale s as hi + lo floats, invC s^2 as floats, and per-pixel
  // r^T invC r (FP64); templates are produced divided by s
  const float2 *tw32[kWvMaxLayers + 1];
  const float *win32[kWvMaxLayers + 1];
  const float *r0hi[kWvMaxLayers + 1], *r0lo[kWvMaxLayers + 1];  // r0ds as hi + lo floats
  const float *res_hi, *res_lo;  // [3][N]
  const float *invC32;           // [9][N]
  const double *qpix;            // [N]
  double scale;                  // s
};

struct WvWorkDev {
  int cap = 0;
  WvSrc *src = nullptr;
  double *ssb = nullptr;   // [cap][2][4][norb] barycentre amplitude / phase splines
  double *resp = nullptr;  // [cap][7][norb] M (3), Mf (3), phase at S/C 1
  double *tdi = nullptr;   // [cap][3][2][4][norb] per-channel amplitude / phase splines
  double *coef = nullptr;  // [cap][3][kWvMaxLayers NT] coefficients, list order first
  // the mixed likelihood's re-evaluation list: total[0] counts the sources
  // re-evaluated over the context's life, count[0] those of the current
  // launch, list[k] their indices
  unsigned long long *total = nullptr;
  int *count = nullptr, *list = nullptr;
};

// Host-side grid description: orbit nodes and positions plus the WDM grid.
struct WvGridHost {
  double Tobs = 0, t0 = 0, wdt = 0, wdf = 0, A = 0, nx = 0;
  int NF = 0, NT = 0, kmin = 0, kmax = 0;
  std::vector<double> orb_t;    // orbit node times
  std::vector<double> orb_pos;  // [(3 s + d) norb + n] metres
};

// Orbit nodes of initialize_interpolated_analytic_orbits for (Tobs, t0).
void wv_analytic_orbit(double Tobs, double t0, std::vector<double> &t, std::vector<double> &pos);

// Builds the device tables of a grid into one allocation (*mem) and fills
// the tables part of *g (res / invC are set by wv_set_data).
cudaError_t wv_build_grid(const WvGridHost &h, WvGridDev *g, void **mem, cudaStream_t s);
size_t wv_work_bytes(int cap, int norb, int NT);
void wv_work_carve(WvWorkDev &w, void *base, int cap, int norb, int NT);

// wavelet_transform_timefreq_by_layers on a device series of NT (nl + 1)
// samples, in place (one CTA): nl layers from jmin, window win[NT/2 + 1],
// tw[k] = e^{-2 pi i k / (NT (nl + 1))}; NT (nl + 1) must have no prime factor
// above 3.
cudaError_t wdm_by_layers_launch(int NF, int NT, int jmin, int nl, const double *d_win, const double2 *d_tw,
                                 double *d_data, cudaStream_t s);
void wdm_unit_roots(int P, double2 *out);

// Waveform batch: plan, response, TDI splines, per-layer transforms.
// precision 1: samples with an FP64 phase and FP32 amplitude spline, FP32
// FFTs, FP32 coefficients (divided by g.scale) in w.coef.
cudaError_t wv_waveform_launch(const WvGridDev &g, const WvWorkDev &w, int precision, int n, const double *params,
                               int *status, cudaStream_t s, int *nlaunch);
// Sparse likelihood over each source's pixels (after wv_waveform_launch with
// the same precision).
// The mixed likelihood's error estimate: |delta logL error| <~ K sqrt((h|h)
// (r - h|r - h)), the FP32 template's error acting coherently along h - r.
// Measured on three 4096-source workloads (noise at median SNR 20 with 100
// injected sources, twice, and a louder population): the error stays below
// 9.7e-8 sqrt((h|h) (r - h|r - h)) wherever it exceeds 1e-4; K doubles that.
// With tol > 0 every source whose estimate exceeds tol (or whose mixed result
// is not finite) is evaluated again in FP64 in the same launch sequence.
constexpr double kWvMixedErrK = 2e-7;
cudaError_t wv_dlogl_launch(const WvGridDev &g, const WvWorkDev &w, int precision, int n, const double *term_x,
                            double *dlogl, double *term_y, double *hh, int *status, cudaStream_t s, int *nlaunch,
                            double tol = 0.0);
// Fisher matrices of n sources (ucb_fisher_wavelet) in FP64: pp is scratch for
// 16 n perturbed parameter vectors; needs 16 n <= w.cap; fisher[64 s + 8 i + j].
cudaError_t wv_fisher_launch(const WvGridDev &g, const WvWorkDev &w, int n, const double *params, double *pp,
                             int imin, int imax, double *fisher, int *status, cudaStream_t s, int *nlaunch);
// Per-item layer info and values in list order: info[4 i] = first layer,
// layer count, first kept layer, kept layers per time; xyz[(3 i + c) (kWvMaxLayers NT) + q].
cudaError_t wv_export(const WvGridDev &g, const WvWorkDev &w, int precision, int n, int *info, double *xyz,
                      cudaStream_t s);
// Host: the mixed-precision data (hi/lo residual, FP32 invC, per-pixel
// r^T invC r) of a segment from its FP64 residual and invC; sizes as WvGridDev.
void wv_mixed_data(int N, int NT, const double *rX, const double *rY, const double *rZ, const double *invC,
                   double *scale, std::vector<float> &res_hi, std::vector<float> &res_lo, std::vector<float> &invC32,
                   std::vector<double> &qpix);

}  // namespace glass
