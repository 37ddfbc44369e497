// Internal host-side interface of the on-device sampler kernels (sampler.cu).
#pragma once
#include <cuda_runtime.h>

namespace glass {

struct MhArgs {
  int n;
  const double *T, *dlogl, *logPx, *logPy, *logQxy, *logQyx, *snr;
  double *logL_x, *params_x;
  const double *params_y;
  unsigned int *seed;
  int *accepted;
};

struct PtArgs {
  int nens, NC;
  const double *temperature, *logL, *logLnorm;
  int *index;
  unsigned int *seed;
  double *acceptance;
};

struct FisherDrawArgs {
  int n;
  const double *params_x;  // 8 n: the source's current parameters
  const double *evec;      // 64 n: evec[64 i + 8 j + k] = fisher_evectr[j][k] of chain i
  const double *evalue;    // 8 n
  unsigned int *seed;
  double *params_y;  // 8 n
  double *logQ;      // n or NULL: 0, or -inf where a drawn parameter is NaN
  int *status;       // n or NULL: GLASS_DRAW_* of the chain
};

cudaError_t rand_r_fill_launch(int n, int count, unsigned int *seed, int *out, cudaStream_t stream);
cudaError_t mh_accept_launch(const MhArgs &a, cudaStream_t stream);
cudaError_t ptmcmc_launch(const PtArgs &a, cudaStream_t stream);
cudaError_t fisher_draw_launch(const FisherDrawArgs &a, cudaStream_t stream);

}  // namespace glass
