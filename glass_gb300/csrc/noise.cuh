// Internal host-side interface of the noise-model likelihood (noise.cu).
#pragma once
#include <cuda_runtime.h>

namespace glass {

// Rows of the per-bin table (each N doubles): the frequency, cos(f/f*), the
// TDI transfer function -8 sin^2(f/f*), the acceleration and optical-metrology
// transfer functions, the foreground's 4 x^2 sin^2 x and f^(-7/3), and the
// data's XX, YY, ZZ, XY, XZ, YZ spectra.
enum {
  kTabF = 0, kTabCosx, kTabTdi, kTabAcc, kTabOms, kTabTgal, kTabFp73,
  kTabXX, kTabYY, kTabZZ, kTabXY, kTabXZ, kTabYZ, kNoiseTabRows
};
// One- and two-channel data (Michelson X; or A and E) keep the data's power
// |X|^2 (or |A|^2, |E|^2) and cos(2 f/f*) in the rows of XX, YY and ZZ.
enum { kTabP0 = kTabXX, kTabP1 = kTabYY, kTabCos2x = kTabZZ };

struct NoiseDev {
  int nch = 3;  // 3: X, Y, Z; 1: X; 2: A, E
  int N = 0;
  double T = 0, fmin = 0;
  double *tab = nullptr;      // kNoiseTabRows x N
  double *rsg = nullptr;      // 6 x N: the SGWB response (xx, yy, zz, xy, xz, yz) per bin, or null
  double *partial = nullptr;  // per-model chunk sums
  int partial_models = 0;     // models the partial buffer holds
};

void noise_build_table(double T, double fmin, int N, const double *X, const double *Y, const double *Z, double *tab);
// The same table for one channel (d0 = X) or two (d0, d1 = A, E).
void noise_build_table_ch(double T, double fmin, int N, int nch, const double *d0, const double *d1, double *tab);

// Wavelet-domain form (coarse-grained): layers lmin .. lmin + Nlayer - 1 of an
// NF x NT grid of layer width df, cells of Q pixels in time.
struct NoiseWvDev {
  int NF = 0, NT = 0, lmin = 0, Nlayer = 0, Q = 0, Ncoarse = 0;
  double df = 0;
  bool has_mod = false;
  double *tab = nullptr;      // kNoiseTabRows x Nlayer: layer-centre factors, then per-layer sums of P over q
  double *P = nullptr;        // 6 x Nlayer Ncoarse cell statistics (xx, yy, zz, xy, xz, yz)
  double *mod = nullptr;      // 6 x Ncoarse modulation of the foreground (or unused)
  double *rsg = nullptr;      // 6 x Nlayer: the SGWB response at the layer centres, or null
  double *partial = nullptr;  // per-model chunk sums
  int partial_models = 0;
  void *mem = nullptr;        // backs tab, P, mod
};

// Layer-centre factors (rows kTabF .. kTabFp73) at f = (lmin + j) df, the cell
// statistics P (coarse_grain_wavelet_data, noise/src/glass_noise_model.c:1057)
// of X, Y, Z (pixel i of layer j at i + j NT) and their per-layer sums (rows
// kTabXX .. kTabYZ).
void noise_wv_build(int NT, double df, int lmin, int Nlayer, int Q, const double *X, const double *Y, const double *Z,
                    double *tab, double *P);
int noise_wv_chunks(const NoiseWvDev &w);
// mode 0 instrument, 1 stationary foreground, 2 modulated foreground; plus,
// with sgwb (4 per model, template sg_type), the stochastic background;
// w.partial must hold nprop x noise_wv_chunks(w) (mode 2).
cudaError_t noise_wv_logl_launch(const NoiseWvDev &w, int mode, int nprop, const double *inst, const double *sgal,
                                 int sg_type, const double *sgwb, double *logl, cudaStream_t stream, int *nlaunch);

// SGWB templates (SGWB_t, noise/src/glass_noise_model.h:99-108) and their
// parameter counts
enum { kSgwbPowerlaw = 0, kSgwbLognormal = 1, kSgwbPhaseTransition = 2, kSgwbTypes = 3 };
constexpr int kSgwbParams[kSgwbTypes] = {2, 3, 4};
// The instrument's SGWB response at frequencies f[N] from the table rows
// resp[7 i ..] = f, XX, YY, ZZ, XY, XZ, YZ (i < nresp): R6[e N + n], e = xx,
// yy, zz, xy, xz, yz (0 at f = 0).  Returns 0, or -1 for a table the
// reference would refuse or cannot take a log of.
int noise_sgwb_rows(int nresp, const double *resp, int N, const double *f, double *R6);

// The spline noise model (one or two channels): the bins' frequencies, the
// transfer floor and each channel's data power |d|^2, all N doubles.
constexpr int kSplineMaxKnots = 512;
struct SplineNoiseDev {
  int nch = 0, N = 0;
  double *tab = nullptr;  // f, transfer, P0[, P1]: (2 + nch) x N
};
// logl[p] for nprop spline models: nknots[p] control points knot_f[p kmax ..],
// knot_C[(p nch + c) kmax ..] (device pointers)
cudaError_t spline_noise_launch(const SplineNoiseDev &s, int nprop, int kmax, const int *nknots, const double *knot_f,
                                const double *knot_C, double *logl, cudaStream_t stream, int *nlaunch);
int noise_chunks(int N);
// logl[p] for noise models inst[12 p ..] (sacc[6], soms[6]) and sgal[5 p ..]
// (or null: instrument only), plus, with sgwb[4 p ..] (or null), the SGWB of
// template sg_type (three channels only); nd.partial must hold nprop x
// noise_chunks(N).  Three channels: my_noise_log_likelihood; one or two:
// noise_log_likelihood (no 2 pi constant), link levels sacc[0], soms[0].
cudaError_t noise_logl_launch(const NoiseDev &nd, int nprop, const double *inst, const double *sgal, int sg_type,
                              const double *sgwb, double *logl, cudaStream_t stream, int *nlaunch);

}  // namespace glass
