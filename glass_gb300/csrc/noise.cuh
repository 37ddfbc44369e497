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

struct NoiseDev {
  int N = 0;
  double T = 0, fmin = 0;
  double *tab = nullptr;      // kNoiseTabRows x N
  double *partial = nullptr;  // per-model chunk sums
  int partial_models = 0;     // models the partial buffer holds
};

void noise_build_table(double T, double fmin, int N, const double *X, const double *Y, const double *Z, double *tab);
int noise_chunks(int N);
// logl[p] for noise models inst[12 p ..] (sacc[6], soms[6]) and sgal[5 p ..]
// (or null: instrument only); nd.partial must hold nprop x noise_chunks(N).
cudaError_t noise_logl_launch(const NoiseDev &nd, int nprop, const double *inst, const double *sgal, double *logl,
                              cudaStream_t stream, int *nlaunch);

}  // namespace glass
