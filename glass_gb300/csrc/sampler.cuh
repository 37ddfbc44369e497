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

// Uniform priors of a model: prior[16 c + 2 k + {0, 1}] the bounds of
// parameter k, logPV[8 c + k] = log(max - min) (model->prior,
// model->logPriorVolume); c = i * stride (stride 0: one set for every chain).
struct PriorArgs {
  int n;
  const double *prior, *logPV;
  int stride;
  // draw_from_uniform_prior
  unsigned int *seed;
  double *params;  // 8 n, drawn (draw) or checked and wrapped in place (evaluate)
  double *out;     // n: logQ (draw) or logP (evaluate)
  // sky-location histogram (galaxy prior): skyhist[i nphi + j] over cells of
  // dcostheta x dphi from the prior's lower bounds; null: uniform sky
  const double *skyhist;
  double dcostheta, dphi;
  int nphi;
};

cudaError_t sym_eigen8_launch(int n, const double *matrix, double *evec, double *evalue, cudaStream_t stream);
cudaError_t prior_draw_launch(const PriorArgs &a, cudaStream_t stream);
cudaError_t ucb_prior_launch(const PriorArgs &a, cudaStream_t stream);
cudaError_t rand_r_fill_launch(int n, int count, unsigned int *seed, int *out, cudaStream_t stream);
cudaError_t mh_accept_launch(const MhArgs &a, cudaStream_t stream);
cudaError_t ptmcmc_launch(const PtArgs &a, cudaStream_t stream);
cudaError_t fisher_draw_launch(const FisherDrawArgs &a, cudaStream_t stream);

}  // namespace glass
