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
// The trans-dimensional (birth/death) step of ucb_rjmcmc for n chains, in two
// launches around the likelihood: chain i's live sources src[(i maxsrc + s) 8
// ..], s < Nlive[i].
struct RjArgs {
  int n, maxsrc;
  int *Nlive;
  const int *Neff;
  double *src;
  const double *prior, *logPV;
  int stride;
  double rjw[9];  // the proposals' rj weights (0: prior draw, 1: F-statistic draw, others 0)
  // the F-statistic proposal's grid (draw_from_fstatistic): density
  // tensor[(i n_theta + j) n_phi + k], cells d_f x d_theta x d_phi from
  // (qmin / T, -1, 0), maximum maxp
  const double *tensor;
  int n_f, n_theta, n_phi, qmin;
  double d_f, d_theta, d_phi, maxp, T;
  unsigned int *seed;
  // proposal: +1 birth / -1 death, the slot created or removed, the new (or
  // removed) source, the proposal densities, 0 or -inf (refused), the kind
  int *move, *slot, *kind, *status;
  double *params_y, *logQxy, *logQyx, *logPy;
  // acceptance
  const double *T_chain, *dlogl, *hh;
  int dlogl_is_term, prior_only;
  const double *skyhist;
  double dcostheta, dphi;
  int nphi;
  double *logL_x;
  int *accepted;
};

cudaError_t prior_draw_launch(const PriorArgs &a, cudaStream_t stream);
cudaError_t rj_propose_launch(const RjArgs &a, cudaStream_t stream);
cudaError_t rj_accept_launch(const RjArgs &a, cudaStream_t stream);
cudaError_t ucb_prior_launch(const PriorArgs &a, cudaStream_t stream);
cudaError_t rand_r_fill_launch(int n, int count, unsigned int *seed, int *out, cudaStream_t stream);
cudaError_t mh_accept_launch(const MhArgs &a, cudaStream_t stream);
cudaError_t ptmcmc_launch(const PtArgs &a, cudaStream_t stream);
cudaError_t fisher_draw_launch(const FisherDrawArgs &a, cudaStream_t stream);

}  // namespace glass
