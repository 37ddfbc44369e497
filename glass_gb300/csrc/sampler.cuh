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

cudaError_t rand_r_fill_launch(int n, int count, unsigned int *seed, int *out, cudaStream_t stream);
cudaError_t mh_accept_launch(const MhArgs &a, cudaStream_t stream);
cudaError_t ptmcmc_launch(const PtArgs &a, cudaStream_t stream);

}  // namespace glass
