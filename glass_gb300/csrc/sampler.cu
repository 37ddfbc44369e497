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

// rand_r_N_0_1 (utils/src/glass_utils.c:24-35): Marsaglia's polar method on
// rand_r_U_0_1 pairs.  The rejection loop is bounded: a run of 4096 rejections
// has probability (1 - pi/4)^4096, and then the chain reports
// GLASS_DRAW_RNG_LIMIT instead of looping on.
__device__ __forceinline__ bool glass_n01(unsigned int *seed, double *z) {
  for (int it = 0; it < 4096; it++) {
    const double u = 2 * glass_u01(seed) - 1;
    const double v = 2 * glass_u01(seed) - 1;
    const double s = u * u + v * v;
    if (!(s >= 1 || s == 0)) {
      *z = u * sqrt(-2 * log(s) / s);
      return true;
    }
  }
  *z = 0.0;
  return false;
}

// draw_from_fisher (ucb/src/glass_ucb_proposal.c:348-391) for chain i by one
// thread, in the reference's order: eight N(0,1) amplitudes over
// sqrt(eigenvalue), one eigenvector picked by a ninth draw, the jump along
// it, the NaN and |cos| >= 1 repairs.
__device__ void fisher_draw_serial(const FisherDrawArgs &a, int i) {
  const double *x = a.params_x + 8 * (size_t)i;
  const double *ev = a.evec + 64 * (size_t)i;
  const double *el = a.evalue + 8 * (size_t)i;
  double *y = a.params_y + 8 * (size_t)i;
  unsigned int s = a.seed[i];
  int st = GLASS_DRAW_OK;
  double amps[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    double z;
    if (!glass_n01(&s, &z)) st = GLASS_DRAW_RNG_LIMIT;
    amps[k] = z / sqrt(el[k]);
  }
  // (int)(U * 8) is 8 when rand_r returns RAND_MAX (U = 1), where the
  // reference reads one column past the matrix; the last column is taken here
  int c = (int)(glass_u01(&s) * 8.0);
  if (c > 7) c = 7;
  double jump[8];
#pragma unroll
  for (int j = 0; j < 8; j++) {
    jump[j] = 0.0;
    jump[j] += amps[c] * ev[8 * j + c];
    if (jump[j] != jump[j]) jump[j] = 0.01 * x[j];
  }
  double p[8];
#pragma unroll
  for (int j = 0; j < 8; j++) p[j] = x[j] + jump[j];
  if (p[1] >= 1.) p[1] = x[1] - jump[1];
  if (p[1] <= -1.) p[1] = x[1] - jump[1];
  if (p[4] >= 1.) p[4] = x[4] - jump[4];
  if (p[4] <= -1.) p[4] = x[4] - jump[4];
  double logQ = 0.0;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    y[j] = p[j];
    if (p[j] != p[j]) logQ = -INFINITY;
  }
  if (logQ < 0.0 && st == GLASS_DRAW_OK) st = GLASS_DRAW_NAN;
  a.seed[i] = s;
  if (a.logQ) a.logQ[i] = logQ;
  if (a.status) a.status[i] = st;
}


// rand_r's linear congruence advanced k steps at once: next = A next + C.
__device__ __forceinline__ void lcg_jump(int k, unsigned int &A, unsigned int &C) {
  A = 1u;
  C = 0u;
  for (int j = 0; j < k; j++) {
    A *= 1103515245u;
    C = C * 1103515245u + 12345u;
  }
}

// The same draw with eight lanes per chain.  The polar method's pairs are
// independent given the stream, so the lanes generate the chain's next 48
// rand_r values at once (lane l takes values l, l + 8, ..., each rand_r being
// three steps of the congruence, reached by jumps), test the 24 pairs, and
// the k-th accepted pair gives lane k its amplitude: the FP64 log and sqrt of
// the eight amplitudes run side by side instead of one after another.  The
// ninth draw is the value after the eighth accepted pair, and the seed ends
// where it ends for the reference.  When the 48 values hold fewer than eight
// accepted pairs and the choice (probability about 1e-8), the chain's first
// lane redoes the draw in the reference's order.
__global__ void __launch_bounds__(128) fisher_draw_kernel(FisherDrawArgs a) {
  constexpr int V = 48;  // values per chain and pass: 24 pairs
  __shared__ int val[16][V];
  __shared__ unsigned int post[16][V];  // the seed after each value
  const int gi = threadIdx.x >> 3, sub = threadIdx.x & 7;
  const int i = blockIdx.x * 16 + gi;
  if (i >= a.n) return;  // all eight lanes of a chain leave together
  const unsigned int gmask = 0xffu << (threadIdx.x & 24);
  const unsigned int s0 = a.seed[i];
  {
    unsigned int A, C, A8, C8;
    lcg_jump(3 * sub, A, C);
    lcg_jump(24, A8, C8);
    unsigned int st = A * s0 + C;  // the state before value sub
    for (int q = 0; q < V / 8; q++) {
      unsigned int t = st;
      val[gi][sub + 8 * q] = glass_rand_r(&t);
      post[gi][sub + 8 * q] = t;
      st = A8 * st + C8;
    }
  }
  __syncwarp(gmask);
  // pair p accepted: s in (0, 1)
  unsigned int accmask = 0;
  for (int p = sub; p < V / 2; p += 8) {
    const double u = 2 * ((double)val[gi][2 * p] / 2147483647.0) - 1;
    const double v = 2 * ((double)val[gi][2 * p + 1] / 2147483647.0) - 1;
    const double s = u * u + v * v;
    if (!(s >= 1 || s == 0)) accmask |= 1u << p;
  }
  // OR over the chain's lanes
  for (int o = 4; o > 0; o >>= 1) accmask |= __shfl_xor_sync(gmask, accmask, o, 8);
  // pair of the k-th accepted (k = sub), and of the eighth
  int pk = -1, p7 = -1;
  {
    unsigned int m = accmask;
    for (int k = 0; k < 8 && m; k++) {
      const int p = __ffs(m) - 1;
      m &= m - 1;
      if (k == sub) pk = p;
      if (k == 7) p7 = p;
    }
  }
  const bool fast = p7 >= 0 && 2 * p7 + 2 < V;
  if (!fast) {
    if (sub == 0) fisher_draw_serial(a, i);
    return;
  }
  const double *x = a.params_x + 8 * (size_t)i;
  double amp;
  {
    const double u = 2 * ((double)val[gi][2 * pk] / 2147483647.0) - 1;
    const double v = 2 * ((double)val[gi][2 * pk + 1] / 2147483647.0) - 1;
    const double s = u * u + v * v;
    const double z = u * sqrt(-2 * log(s) / s);
    amp = z / sqrt(a.evalue[8 * (size_t)i + sub]);
  }
  int c = (int)(((double)val[gi][2 * p7 + 2] / 2147483647.0) * 8.0);
  if (c > 7) c = 7;
  const double ampc = __shfl_sync(gmask, amp, c, 8);
  // lane j: component j of the jump and of the drawn parameters
  const int j = sub;
  const double xj = x[j];
  double jump = 0.0;
  jump += ampc * a.evec[64 * (size_t)i + 8 * j + c];
  if (jump != jump) jump = 0.01 * xj;
  double y = xj + jump;
  if (j == 1 || j == 4) {
    if (y >= 1.) y = xj - jump;
    if (y <= -1.) y = xj - jump;
  }
  a.params_y[8 * (size_t)i + j] = y;
  const bool nan_any = __any_sync(gmask, y != y);
  if (sub == 0) {
    a.seed[i] = post[gi][2 * p7 + 2];
    if (a.logQ) a.logQ[i] = nan_any ? -INFINITY : 0.0;
    if (a.status) a.status[i] = nan_any ? GLASS_DRAW_NAN : GLASS_DRAW_OK;
  }
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

// Eigen-decomposition of one symmetric 8x8 matrix per thread (the Fisher
// matrix of a chain, for draw_from_fisher without a trip to the host), as
// the drop-in matrix_eigenstuff does it: cyclic Jacobi rotations until every
// off-diagonal entry is negligible against its two diagonal entries (every
// eigenvalue to full relative accuracy), pairs sorted by decreasing
// eigenvalue, each unit eigenvector's largest component positive.
// evec[64 i + 8 j + k] = component j of eigenvector k (fisher_evectr[j][k]).
__global__ void __launch_bounds__(32) sym_eigen8_kernel(int n, const double *matrix, double *evec, double *evalue) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a[8][8], v[8][8];
  const double *m = matrix + 64 * (size_t)i;
  for (int r = 0; r < 8; r++)
    for (int c = 0; c < 8; c++) {
      a[r][c] = 0.5 * (m[8 * r + c] + m[8 * c + r]);
      v[r][c] = r == c ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 64; sweep++) {
    int rotations = 0;
    for (int p = 0; p < 8; p++)
      for (int q = p + 1; q < 8; q++) {
        const double apq = a[p][q], app = a[p][p], aqq = a[q][q];
        if (!(fabs(apq) > 1e-18 * sqrt(fabs(app * aqq))) || !(fabs(apq) > 1e-300)) continue;
        rotations++;
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 8; k++) {
          const double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 8; k++) {
          const double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 8; k++) {
          const double vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - s * vkq;
          v[k][q] = s * vkp + c * vkq;
        }
      }
    if (rotations == 0) break;
  }
  int ord[8];
  for (int j = 0; j < 8; j++) ord[j] = j;
  for (int x = 1; x < 8; x++)
    for (int j = x; j > 0 && a[ord[j]][ord[j]] > a[ord[j - 1]][ord[j - 1]]; j--) {
      const int t = ord[j];
      ord[j] = ord[j - 1];
      ord[j - 1] = t;
    }
  double *ev = evec + 64 * (size_t)i;
  for (int j = 0; j < 8; j++) {
    const int c = ord[j];
    evalue[8 * (size_t)i + j] = a[c][c];
    int big = 0;
    for (int r = 1; r < 8; r++)
      if (fabs(v[r][c]) > fabs(v[big][c])) big = r;
    const double sg = v[big][c] < 0.0 ? -1.0 : 1.0;
    for (int r = 0; r < 8; r++) ev[8 * r + j] = sg * v[r][c];
  }
}


// ---------------------------------------------------------------- priors
// The reference's prior pieces on one parameter set p[8] with bounds pr[16]
// and log prior volumes lv[8]; each wraps p in place where the reference does,
// and each sums in the reference's own order.
constexpr double kTwoPi = 6.283185307179586;

// check_range (ucb/src/glass_ucb_prior.c:400-438): true when p is outside the
// prior (or NaN); longitude, polarisation and phase are wrapped in place (the
// wrapping loops stop after 64 turns, the reference's do not).
__device__ bool prior_check_range(double *p, const double *pr) {
  for (int k = 0; k < 8; k++)
    if (p[k] != p[k]) return true;
  if (p[0] < pr[0] || p[0] > pr[1]) return true;
  if (p[1] < pr[2] || p[1] > pr[3]) return true;
  if (p[2] < pr[4] || p[2] >= pr[5]) {
    p[2] = atan2(sin(p[2]), cos(p[2]));
    if (p[2] < 0.0) p[2] += kTwoPi;
  }
  if (p[3] < pr[6] || p[3] > pr[7]) return true;
  if (p[4] < pr[8] || p[4] > pr[9]) return true;
  for (int it = 0; it < 64 && p[5] < pr[10]; it++) p[5] += M_PI;
  for (int it = 0; it < 64 && p[5] > pr[11]; it++) p[5] -= M_PI;
  for (int it = 0; it < 64 && p[6] < pr[12]; it++) p[6] += kTwoPi;
  for (int it = 0; it < 64 && p[6] > pr[13]; it++) p[6] -= kTwoPi;
  if (p[7] < pr[14] || p[7] > pr[15]) return true;
  return false;
}

// evalaute_sky_location_prior (ucb/src/glass_ucb_prior.c:590-639): the galaxy
// histogram skyhist[i nphi + j] when given, else the uniform sky.
__device__ double prior_sky(double *p, const double *pr, const double *lv, const double *skyhist, double dcostheta,
                            double dphi, int nphi) {
  double logP = 0.0;
  if (skyhist) {
    if (p[1] < pr[2] || p[1] > pr[3]) return -INFINITY;
    if (pr[4] > 0.0 || pr[5] < kTwoPi) {
      if (p[2] < pr[4] || p[2] > pr[5]) return -INFINITY;
    } else {
      for (int it = 0; it < 64 && p[2] < 0; it++) p[2] += kTwoPi;
      for (int it = 0; it < 64 && p[2] > kTwoPi; it++) p[2] -= kTwoPi;
    }
    const int ci = (int)floor((p[1] - pr[2]) / dcostheta);
    const int cj = (int)floor((p[2] - pr[4]) / dphi);
    logP += skyhist[ci * nphi + cj];
  } else {
    if (p[1] < pr[2] || p[1] > pr[3]) return -INFINITY;
    logP -= lv[1];
    if (pr[4] > 0.0 || pr[5] < kTwoPi) {
      if (p[2] < pr[4] || p[2] > pr[5]) return -INFINITY;
    } else if (p[2] < pr[4] || p[2] >= pr[5]) {
      p[2] = atan2(sin(p[2]), cos(p[2]));
      if (p[2] < 0.0) p[2] += kTwoPi;
    }
    logP -= lv[2];
  }
  return logP;
}

// evaluate_uniform_priors (ucb/src/glass_ucb_prior.c:560-588)
__device__ double prior_uniform(double *p, const double *pr, const double *lv) {
  if (prior_check_range(p, pr)) return -INFINITY;
  double logP = 0.0;
  logP -= log(pr[1] - pr[0]);
  logP -= lv[3];
  logP -= lv[4];
  logP -= lv[5];
  logP -= lv[6];
  logP -= lv[7];
  return logP;
}

// evaluate_ucb_prior (ucb/src/glass_ucb_prior.c:536-556) on the blind-search
// path (no catalogue prior)
__device__ double prior_ucb(double *p, const double *pr, const double *lv, const double *skyhist, double dcostheta,
                            double dphi, int nphi) {
  if (prior_check_range(p, pr)) return -INFINITY;
  double logP = 0.0;
  logP += prior_sky(p, pr, lv, skyhist, dcostheta, dphi, nphi);
  logP += prior_uniform(p, pr, lv);
  return logP;
}

// draw_from_uniform_prior (utils/src/glass_sampler.c:96-107)
__device__ double prior_draw(double *p, const double *pr, const double *lv, unsigned int *s) {
  double logQ = 0.0;
  for (int k = 0; k < 8; k++) {
    p[k] = pr[2 * k] + glass_u01(s) * (pr[2 * k + 1] - pr[2 * k]);
    logQ -= lv[k];
  }
  return logQ;
}

__global__ void ucb_prior_kernel(PriorArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double *pr = a.prior + 16 * (size_t)i * a.stride;
  const double *lv = a.logPV + 8 * (size_t)i * a.stride;
  a.out[i] = prior_ucb(a.params + 8 * (size_t)i, pr, lv, a.skyhist, a.dcostheta, a.dphi, a.nphi);
}

// draw_from_uniform_prior, one thread per chain: the eight parameters from
// rand_r_U_0_1 in order, logQ = -sum of the log prior volumes.
__global__ void prior_draw_kernel(PriorArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double *pr = a.prior + 16 * (size_t)i * a.stride;
  const double *lv = a.logPV + 8 * (size_t)i * a.stride;
  unsigned int s = a.seed[i];
  a.out[i] = prior_draw(a.params + 8 * (size_t)i, pr, lv, &s);
  a.seed[i] = s;
}

// ------------------------------------------------- trans-dimensional step
// The F-statistic proposal's density (evaluate_fstatistic_proposal,
// ucb/src/glass_ucb_proposal.c:1640-1673): the uniform sky and the uniform
// priors, plus the log of the grid cell's density.
__device__ double fstat_density(double *p, const RjArgs &a, const double *pr, const double *lv) {
  double logP = 0.0;
  logP += prior_sky(p, pr, lv, nullptr, 1, 1, 1);
  logP += prior_uniform(p, pr, lv);
  const int i = (int)floor((p[0] - a.qmin) / (a.d_f * a.T));
  const int j = (int)floor((p[1] - -1) / a.d_theta);
  const int k = (int)floor((p[2]) / a.d_phi);
  if (i < 0 || i >= a.n_f) return -INFINITY;
  if (j < 0 || j >= a.n_theta) return -INFINITY;
  if (k < 0 || k >= a.n_phi) return -INFINITY;
  logP += log(a.tensor[((size_t)i * a.n_theta + j) * a.n_phi + k]);
  return logP;
}

// draw_from_fstatistic (ucb/src/glass_ucb_proposal.c:1526-1568): a draw from
// the prior, then rejection sampling of (f, cos theta, phi) on the grid.  A
// cell index equal to the grid size (a draw of exactly 1) is taken as the
// last cell and reported (the reference reads past its grid); the rejection
// loop stops after kRjMaxTries.
constexpr int kRjMaxTries = 1 << 20;
__device__ double fstat_draw(double *p, const RjArgs &a, const double *pr, const double *lv, unsigned int *s,
                             int *st) {
  prior_draw(p, pr, lv, s);
  double q = 0, costheta = 0, phi = 0, pc, alpha;
  int it = 0;
  do {
    const double i = glass_u01(s) * a.n_f;
    const double j = glass_u01(s) * a.n_theta;
    const double k = glass_u01(s) * a.n_phi;
    q = (double)(a.qmin) + i * a.d_f * a.T;
    costheta = -1. + j * a.d_theta;
    phi = k * a.d_phi;
    int ii = (int)i, jj = (int)j, kk = (int)k;
    if (ii >= a.n_f || jj >= a.n_theta || kk >= a.n_phi) {
      *st = GLASS_RJ_RNG_EDGE;
      ii = min(ii, a.n_f - 1);
      jj = min(jj, a.n_theta - 1);
      kk = min(kk, a.n_phi - 1);
    }
    pc = a.tensor[((size_t)ii * a.n_theta + jj) * a.n_phi + kk];
    alpha = glass_u01(s) * a.maxp;
    if (++it >= kRjMaxTries && pc < alpha) {
      *st = GLASS_RJ_RNG_LIMIT;
      return -INFINITY;
    }
  } while (pc < alpha);
  p[0] = q;
  p[1] = costheta;
  p[2] = phi;
  return fstat_density(p, a, pr, lv);
}

// ucb_rjmcmc (ucb/src/glass_ucb_sampler.c:454-483) up to the likelihood, with
// rj_birth_death (:175-249), one thread per chain, every draw in the
// reference's order: the proposal by rejection on the rj weights, the
// birth/death branch draw (always birth/death), birth or death, and the new
// source from the proposal (birth) or the source to remove and its proposal
// density (death).
__global__ void rj_propose_kernel(RjArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double *pr = a.prior + 16 * (size_t)i * a.stride;
  const double *lv = a.logPV + 8 * (size_t)i * a.stride;
  unsigned int s = a.seed[i];
  int st = GLASS_RJ_OK;
  int nprop = 0;
  for (int it = 0;; it++) {
    nprop = (int)floor(9 * glass_u01(&s));
    if (nprop > 8) {
      nprop = 8;  // a draw of exactly 1: the reference reads past its proposals
      st = GLASS_RJ_RNG_EDGE;
    }
    if (!(a.rjw[nprop] <= glass_u01(&s))) break;
    if (it + 1 >= kRjMaxTries) {
      st = GLASS_RJ_RNG_LIMIT;
      break;
    }
  }
  (void)glass_u01(&s);  // birth/death or split/merge: always birth/death
  const int Nx = a.Nlive[i];
  const double *x = a.src + (size_t)i * a.maxsrc * 8;
  double *y = a.params_y + 8 * (size_t)i;
  double lqxy = 0.0, lqyx = 0.0, lpy = 0.0;
  int move, slot;
  if (glass_u01(&s) < 0.5) {  // birth
    move = 1;
    slot = Nx;
    if (Nx + 1 < a.Neff[i] && Nx < a.maxsrc && st != GLASS_RJ_RNG_LIMIT) {
      lqyx = nprop == 0 ? prior_draw(y, pr, lv, &s) : fstat_draw(y, a, pr, lv, &s, &st);
      lqxy = 0;
    } else {
      lpy = -INFINITY;
    }
  } else {  // death
    move = -1;
    const int kill = (int)(glass_u01(&s) * (double)Nx);
    slot = kill;
    if (Nx - 1 > -1 && kill < a.maxsrc && st != GLASS_RJ_RNG_LIMIT) {
      for (int k = 0; k < 8; k++) y[k] = x[8 * (size_t)kill + k];
      lqyx = 0;
      if (nprop == 0) {
        for (int k = 0; k < 8; k++) lqxy -= lv[k];  // uniform_prior_density
      } else {
        double yk[8];  // the density may wrap its copy; the source is kept as it is
        for (int k = 0; k < 8; k++) yk[k] = y[k];
        lqxy = fstat_density(yk, a, pr, lv);
      }
    } else {
      lpy = -INFINITY;
    }
  }
  if (st == GLASS_RJ_RNG_LIMIT) lpy = -INFINITY;
  a.seed[i] = s;
  a.move[i] = move;
  a.slot[i] = slot;
  a.kind[i] = nprop;
  a.logQxy[i] = lqxy;
  a.logQyx[i] = lqyx;
  a.logPy[i] = lpy;
  if (a.status) a.status[i] = st;
}

// ucb_rjmcmc (ucb/src/glass_ucb_sampler.c:485-565) from the likelihood on,
// one thread per chain: the birth's SNR cut (rj_birth_death :205-210), the
// priors of the current and proposed source lists, the Hastings ratio, one
// draw, and on acceptance the proposed list and log-likelihood.
__global__ void rj_accept_kernel(RjArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double *pr = a.prior + 16 * (size_t)i * a.stride;
  const double *lv = a.logPV + 8 * (size_t)i * a.stride;
  const int Nx = a.Nlive[i], move = a.move[i], slot = a.slot[i];
  double *x = a.src + (size_t)i * a.maxsrc * 8;
  double *y = a.params_y + 8 * (size_t)i;
  double lpy = a.logPy[i];
  double dlogL = a.dlogl[i];
  if (a.dlogl_is_term && move < 0) dlogL = -dlogL - a.hh[i];  // the removed source's term and (h|h)
  if (move > 0 && lpy > -INFINITY && !a.prior_only && a.hh && sqrt(a.hh[i]) < 5.0) lpy = -INFINITY;
  double logPx = 0.0;
  const int Ny = Nx + move;
  // a list or slot outside the chain's maxsrc slots is refused, not read
  const bool inb = Nx >= 0 && Nx <= a.maxsrc && Ny >= 0 && Ny <= a.maxsrc &&
                   (move > 0 ? (move == 1 && slot == Nx) : (move == -1 && slot >= 0 && slot < Nx));
  if (!inb) lpy = -INFINITY;
  if (lpy > -INFINITY) {
    // The current list is evaluated (and wrapped) in place, as the reference
    // does; the proposed list's copies of it then give the same values as
    // the reference's copies taken before the wrapping.
    for (int n = 0; n < Nx; n++) logPx += prior_ucb(x + 8 * (size_t)n, pr, lv, a.skyhist, a.dcostheta, a.dphi, a.nphi);
    for (int n = 0; n < Ny; n++) {
      if (move > 0 && n == Nx) {
        lpy += prior_ucb(y, pr, lv, a.skyhist, a.dcostheta, a.dphi, a.nphi);
        continue;
      }
      double yn[8];
      const double *src = x + 8 * (size_t)((move > 0 || n < slot) ? n : n + 1);
      for (int k = 0; k < 8; k++) yn[k] = src[k];
      lpy += prior_ucb(yn, pr, lv, a.skyhist, a.dcostheta, a.dphi, a.nphi);
    }
  }
  double logH = 0.0;
  if (lpy > -INFINITY && !a.prior_only) logH += dlogL / a.T_chain[i];
  logH += lpy - logPx;
  logH += a.logQxy[i] - a.logQyx[i];
  unsigned int s = a.seed[i];
  const double loga = log(glass_u01(&s));
  a.seed[i] = s;
  int acc = 0;
  if (isfinite(logH) && logH > loga) {
    acc = 1;
    if (move > 0) {
      for (int k = 0; k < 8; k++) x[8 * (size_t)Nx + k] = y[k];
    } else {
      for (int n = slot; n < Ny; n++)
        for (int k = 0; k < 8; k++) x[8 * (size_t)n + k] = x[8 * (size_t)(n + 1) + k];
    }
    a.Nlive[i] = Ny;
    a.logL_x[i] += dlogL;
  }
  if (a.accepted) a.accepted[i] = acc;
}

}  // namespace

cudaError_t sym_eigen8_launch(int n, const double *matrix, double *evec, double *evalue, cudaStream_t stream) {
  // one warp per CTA: the chains' FP64 rotations spread over the SMs
  sym_eigen8_kernel<<<(n + 31) / 32, 32, 0, stream>>>(n, matrix, evec, evalue);
  return cudaGetLastError();
}

cudaError_t prior_draw_launch(const PriorArgs &a, cudaStream_t stream) {
  prior_draw_kernel<<<(a.n + 31) / 32, 32, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t ucb_prior_launch(const PriorArgs &a, cudaStream_t stream) {
  ucb_prior_kernel<<<(a.n + 31) / 32, 32, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t rand_r_fill_launch(int n, int count, unsigned int *seed, int *out, cudaStream_t stream) {
  rand_r_fill_kernel<<<(n + 127) / 128, 128, 0, stream>>>(n, count, seed, out);
  return cudaGetLastError();
}

cudaError_t mh_accept_launch(const MhArgs &a, cudaStream_t stream) {
  // one warp per CTA, like the exchanges below: the chains' FP64 log calls
  // are spread over as many SMs as there are warps
  mh_accept_kernel<<<(a.n + 31) / 32, 32, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t fisher_draw_launch(const FisherDrawArgs &a, cudaStream_t stream) {
  // eight lanes per chain, sixteen chains per CTA
  fisher_draw_kernel<<<(a.n + 15) / 16, 128, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t rj_propose_launch(const RjArgs &a, cudaStream_t stream) {
  rj_propose_kernel<<<(a.n + 31) / 32, 32, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t rj_accept_launch(const RjArgs &a, cudaStream_t stream) {
  rj_accept_kernel<<<(a.n + 31) / 32, 32, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t ptmcmc_launch(const PtArgs &a, cudaStream_t stream) {
  ptmcmc_kernel<<<(a.nens + 31) / 32, 32, 0, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace glass
