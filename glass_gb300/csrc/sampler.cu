// On-device pieces of the GLASS sampler for sm_103a: the reference's
// random-number stream, the Metropolis-Hastings accept/reject tail of
// ucb_mcmc and the parallel-tempering exchange ptmcmc, for many chains at
// once, on state that stays in device memory between steps.
//
// The reference draws every random number of a chain from the C library's
// rand_r on that chain's seed (rand_r_U_0_1, utils/src/glass_utils.c:19-22);
// glass_rand_r below restates that published algorithm (three rounds of the
// linear congruence next = next * 1103515245 + 12345, 11 + 10 + 10 bits of
// their high halves), so a chain's seed advances exactly as the reference's
// does and its decisions are the reference's.

#include "../../include/glass_gb300.h"
#include "sampler.cuh"

namespace glass {

namespace {

__device__ __forceinline__ int glass_rand_r(unsigned int *seed) {
  unsigned int next = *seed;
  next *= 1103515245u;
  next += 12345u;
  int result = (int)((next / 65536u) % 2048u);
  next *= 1103515245u;
  next += 12345u;
  result <<= 10;
  result ^= (int)((next / 65536u) % 1024u);
  next *= 1103515245u;
  next += 12345u;
  result <<= 10;
  result ^= (int)((next / 65536u) % 1024u);
  *seed = next;
  return result;
}

// rand_r_U_0_1 (utils/src/glass_utils.c:19-22); RAND_MAX of the C library.
__device__ __forceinline__ double glass_u01(unsigned int *seed) {
  return (double)glass_rand_r(seed) / 2147483647.0;
}

__global__ void rand_r_fill_kernel(int n, int count, unsigned int *seed, int *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned int s = seed[i];
  for (int k = 0; k < count; k++) out[(size_t)i * count + k] = glass_rand_r(&s);
  seed[i] = s;
}

// ucb/src/glass_ucb_sampler.c:141-172, one thread per chain.
__global__ void mh_accept_kernel(MhArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  int acc = 0;
  double lpy = a.logPy[i];
  if (lpy > -INFINITY) {
    if (a.snr && a.snr[i] < 5.0) lpy = -INFINITY;  // rejection on SNR (:149-152)
    double logH = 0.0;
    logH += a.dlogl[i] / a.T[i];
    logH += lpy - a.logPx[i];
    logH += a.logQxy[i] - a.logQyx[i];
    unsigned int s = a.seed[i];
    const double loga = log(glass_u01(&s));
    a.seed[i] = s;
    if (isfinite(logH) && logH > loga) {
      acc = 1;
      a.logL_x[i] += a.dlogl[i];
#pragma unroll
      for (int k = 0; k < 8; k++) a.params_x[8 * (size_t)i + k] = a.params_y[8 * (size_t)i + k];
    }
  }
  if (a.accepted) a.accepted[i] = acc;
}

// utils/src/glass_sampler.c:19-63, one thread per ladder: the exchanges run
// from the hottest pair down and each sees the previous one's permutation.
__global__ void ptmcmc_kernel(PtArgs a) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.nens) return;
  const int NC = a.NC;
  int *idx = a.index + (size_t)e * NC;
  unsigned int *r = a.seed + (size_t)e * NC;
  double *acc = a.acceptance + (size_t)e * NC;
  const double *L = a.logL + (size_t)e * NC;
  const double *Ln = a.logLnorm ? a.logLnorm + (size_t)e * NC : nullptr;
  for (int b = NC - 1; b > 0; b--) {
    const int a0 = b - 1;
    acc[a0] = 0;
    const int olda = idx[a0], oldb = idx[b];
    if (olda < 0 || olda >= NC || oldb < 0 || oldb >= NC) continue;  // not a permutation: leave it
    const double heat1 = a.temperature[a0], heat2 = a.temperature[b];
    const double logL1 = L[olda] + (Ln ? Ln[olda] : 0.0);
    const double logL2 = L[oldb] + (Ln ? Ln[oldb] : 0.0);
    unsigned int s = r[a0];
    if (glass_u01(&s) < 1.0) {
      const double dlogL = logL2 - logL1;
      const double H = (heat2 - heat1) / (heat2 * heat1);
      const double alpha = exp(dlogL * H);
      const double beta = glass_u01(&s);
      if (alpha >= beta) {
        idx[a0] = oldb;
        idx[b] = olda;
        acc[a0] = 1;
      }
    }
    r[a0] = s;
  }
}

}  // namespace

cudaError_t rand_r_fill_launch(int n, int count, unsigned int *seed, int *out, cudaStream_t stream) {
  rand_r_fill_kernel<<<(n + 127) / 128, 128, 0, stream>>>(n, count, seed, out);
  return cudaGetLastError();
}

cudaError_t mh_accept_launch(const MhArgs &a, cudaStream_t stream) {
  mh_accept_kernel<<<(a.n + 255) / 256, 256, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t ptmcmc_launch(const PtArgs &a, cudaStream_t stream) {
  ptmcmc_kernel<<<(a.nens + 127) / 128, 128, 0, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace glass
