// Wavelet-domain UCB waveform (ucb/src/glass_ucb_waveform.c:1061-1240) and its
// sparse-pixel likelihood (utils/src/glass_model.c:624-691) for batches of
// sources on sm_103a, in FP64 with the reference's order of operations
// (compiled with -fmad=false), so that results agree with the reference to
// rounding.
//
// Per source the reference builds barycentre amplitude/phase splines on the
// orbit nodes, runs the LISA response on the ~200 nodes (8 delayed link terms
// per TDI channel, utils/src/glass_lisa.c:757-1074), turns each channel into
// amplitude/phase splines, samples the heterodyned signal at NT (nl + 1)
// points and applies the per-layer WDM transform
// (utils/src/glass_wavelet.c:544-611).  The GPU version splits that into:
//  * wv_plan_kernel    one thread per source: layers, geometry, the two
//                      barycentre splines (Thomas sweeps; the grid's own
//                      factors are precomputed, only the data sweeps remain);
//  * wv_resp_kernel    one thread per (source, orbit node): light-time shift
//                      and the X, Y, Z responses M, Mf;
//  * wv_tdi_kernel     one thread per (source, channel): amplitude sign flips,
//                      phase extraction and unwrapping (sequential scans as in
//                      utils/src/glass_math.c:1034-1052, 1244-1308), and the
//                      two channel splines;
//  * wv_layers_kernel  one CTA per (source, channel): the N_ds samples go
//                      straight into shared memory in digit-reversed order, an
//                      in-place mixed-radix (3, 4, 2) FFT gives the packed real
//                      spectrum, and each layer's windowed NT-point inverse FFT
//                      runs in a second shared buffer (3 NT complex doubles in
//                      all: 192 KB at NT = 4096, so the reference's own grid fits);
//  * wv_dlogl_kernel   one CTA per source: the nine XYZ cross terms of (d|h)
//                      and (h|h) over the source's pixels, gathered from the
//                      segment's residual and 3x3 inverse covariance.
// Everything that does not depend on the source (orbit splines, S/C positions
// at the spline nodes and at the downsampled times, windows, twiddles and the
// spline systems' factorisations) is built once per grid on the host.
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "glass_common.cuh"
#include "ucb_wavelet.cuh"
#include "wdm.cuh"

namespace glass {

namespace {

constexpr double kVEARTH = 0.00010103671;  // utils/src/glass_constants.h:89
constexpr double kSQRT2 = 1.41421356237309504880;
constexpr int kOrbSamplesPerYear = 200;     // utils/src/glass_lisa.h:37

// ------------------------------------------------------------ splines
// c points at [4][n] coefficients; value at x[j] + d.
__device__ __forceinline__ double spl_eval(const double *c, int n, int j, double d) {
  return c[j] + c[n + j] * d + c[2 * n + j] * d * d + c[3 * n + j] * d * d * d;
}

// even_sampled_search (utils/src/glass_math.c:393-402)
__device__ __forceinline__ int even_index(const double *x, int n, double v) {
  const double dx = x[1] - x[0];
  int j = (int)floor((v - x[0]) / dx);
  if (j < 0) j = 0;
  if (j > n - 1) j = n - 1;
  return j;
}

// binary_search (utils/src/glass_math.c:443-473): the largest node <= v; values
// outside the nodes, where the reference reads outside its array, are clamped.
__device__ __forceinline__ int bin_index(const double *x, int n, double v) {
  if (!(v > x[0])) return 0;
  if (v >= x[n - 1]) return v == x[n - 1] ? n - 1 : n - 2;
  const double dx = (x[n - 1] - x[0]) / (double)(n - 1);
  int j = (int)((v - x[0]) / dx);
  j = min(max(j, 0), n - 2);
  while (j > 0 && x[j] > v) j--;
  while (j < n - 2 && x[j + 1] <= v) j++;
  return j;
}

// The tile kernels below keep 4 arrays of n doubles per chain in shared memory,
// chains 4 n + 1 doubles apart: the sequential phases have the chains' threads
// at the same node index, which an unpadded stride would put on one bank.

// Natural cubic spline solve (utils/src/glass_math.c:101-175) on a grid whose
// factors fac = {h, l, mu} are precomputed, split for a CTA that handles many
// value arrays at once: spline_rhs for node i (the forward sweep's right-hand
// side, independent per node), spline_recurrence for one array on one thread
// (the two sequential sweeps on z, which holds the right-hand sides on entry
// and c2 on exit), spline_coeffs for node i (c1, c3).  Every value has the same
// FP64 expression as in one sequential sweep.
__device__ __forceinline__ double spline_rhs(const double *y, int i, const double *h) {
  return 3.0 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1]);
}
__device__ __forceinline__ void spline_recurrence(double *z, int N, const double *fac) {
  const double *h = fac, *l = fac + N, *mu = fac + 2 * N;
  double zprev = 0.0;
  z[0] = 0.0;
  for (int i = 1; i < N - 1; i++) {
    zprev = (z[i] - h[i - 1] * zprev) / l[i];
    z[i] = zprev;
  }
  z[N - 1] = 0.0;
  for (int i = N - 2; i >= 0; i--) z[i] = z[i] - mu[i] * z[i + 1];
}
// c0..c3 ([4][N], out) of node i from the values y and c2 = z
__device__ __forceinline__ void spline_coeffs(const double *y, const double *z, int i, int N, const double *h,
                                              double *out) {
  out[i] = y[i];
  out[2 * N + i] = z[i];
  if (i < N - 1) {
    out[N + i] = (y[i + 1] - y[i]) / h[i] - h[i] * (z[i + 1] + 2.0 * z[i]) / 3.0;
    out[3 * N + i] = (z[i + 1] - z[i]) / (3.0 * h[i]);
  } else {
    out[N + i] = 0.0;
    out[3 * N + i] = 0.0;
  }
}

// ------------------------------------------------------------ plan
// C sources per CTA of 128 threads, 4 norb doubles of shared memory per
// source: the per-source record on one thread per source, the barycentre
// amplitude and phase at the orbit nodes and the spline right-hand sides over
// all threads (node-parallel), the spline recurrences on one thread per array
// (2 C threads), the coefficients node-parallel.
template <int C>
__global__ void __launch_bounds__(128) wv_plan_kernel(WvGridDev g, int n, const double *params, WvSrc *srcs,
                                                      double *ssb, int *status) {
  extern __shared__ __align__(16) double psm[];
  __shared__ int s_ok[C];
  __shared__ double s_f0[C], s_phi0[C], s_fdot[C], s_A0[C];
  const int base = blockIdx.x * C;
  const int nsrc = min(C, n - base);
  const int norb = g.norb;
  const double Tobs = g.Tobs;
  if ((int)threadIdx.x < nsrc) {
    const int s = base + threadIdx.x;
    const double *p = params + 8 * (size_t)s;
    WvSrc S;
    bool ok = true;
    for (int q = 0; q < 8; q++) ok = ok && isfinite(p[q]);
    ok = ok && fabs(p[1]) <= 1.0 && fabs(p[4]) <= 1.0 && p[0] > 0.0;
    S.status = ok ? 0 : 1;
    S.jmin = S.nl = S.jlo = S.c = 0;
    if (ok) {
      // ucb_wavelet_layers
      const double fstart = p[0] / Tobs;
      const double fstop = (p[0] / Tobs + p[7] / Tobs / Tobs);
      double fmin, fmax;
      if (fstart < fstop) {
        fmin = fstart * (1.0 - kVEARTH);
        fmax = fstop * (1.0 + kVEARTH);
      } else {
        fmin = fstop * (1.0 - kVEARTH);
        fmax = fstart * (1.0 + kVEARTH);
      }
      const double jr = rint(fmin / g.wdf);
      if (!(fabs(jr) < 1e9)) {
        S.status = 1;
      } else {
        const int j = (int)jr;
        const double dfmin = fmin - j * g.wdf, dfmax = fmax - j * g.wdf;
        int jmin = j, jmax = j;
        if (dfmin < 0.0 && fabs(dfmin) > g.A / kPI2) jmin = j - 1;
        if (dfmax > 0.0 && fabs(dfmax) > g.A / kPI2) jmax = j + 1;
        S.jmin = jmin;
        S.nl = jmax - jmin + 1;
        const int jlo = max(jmin, g.lmin), jhi = min(jmin + S.nl, g.lmax);
        S.jlo = jlo;
        S.c = max(0, jhi - jlo);
      }
    }
    // geometry (LISA_polarization_tensor, utils/src/glass_lisa.c:1566-1596)
    const double costh = p[1], phi = p[2], cosi = p[4], psi = p[5];
    const double sinth = sqrt(1.0 - costh * costh), cosph = cos(phi), sinph = sin(phi);
    const double u[3] = {costh * cosph, costh * sinph, -sinth};
    const double v[3] = {sinph, -cosph, 0.};
    S.k[0] = -sinth * cosph;
    S.k[1] = -sinth * sinph;
    S.k[2] = -costh;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        S.ep[3 * i + j] = v[i] * v[j] - u[i] * u[j];
        S.ec[3 * i + j] = u[i] * v[j] + v[i] * u[j];
      }
    S.c2p = cos(2. * psi);
    S.s2p = sin(2. * psi);
    S.Ap = 0.5 * (1. + cosi * cosi);
    S.Ac = -cosi;
    S.fhet = (S.jmin - 1) * g.wdf;
    S.pad = 0;
    srcs[s] = S;
    if (status) status[s] = S.status;
    s_ok[threadIdx.x] = S.status == 0;
    s_f0[threadIdx.x] = p[0] / Tobs;
    s_phi0[threadIdx.x] = p[6];
    s_fdot[threadIdx.x] = p[7] / Tobs / Tobs;
    s_A0[threadIdx.x] = S.status == 0 ? exp(p[3]) : 0.0;
  }
  __syncthreads();
  // barycentre amplitude and phase on the orbit nodes (ucb_barycenter_waveform,
  // ucb/src/glass_ucb_waveform.c:330-362)
  for (int q = threadIdx.x; q < nsrc * norb; q += blockDim.x) {
    const int c = q / norb, i = q - c * norb;
    if (!s_ok[c]) continue;
    double *ya = psm + (size_t)c * (4 * norb + 1), *yp = ya + norb;
    const double f0 = s_f0[c], phi0 = s_phi0[c], fdot = s_fdot[c], fddot = 0.0;
    const double A0 = s_A0[c];
    const double t = g.orb_t[i];
    yp[i] = -phi0 + kPI2 * (f0 * t + 0.5 * fdot * t * t + 1.0 / 6.0 * fddot * t * t * t);
    ya[i] = A0 * (1.0 + 2.0 / 3.0 * fdot / f0 * t);
  }
  __syncthreads();
  const double *h = g.fac_orb;
  for (int q = threadIdx.x; q < nsrc * norb; q += blockDim.x) {
    const int c = q / norb, i = q - c * norb;
    if (!s_ok[c] || i == 0 || i == norb - 1) continue;
    double *ya = psm + (size_t)c * (4 * norb + 1), *yp = ya + norb, *za = ya + 2 * norb, *zp = ya + 3 * norb;
    za[i] = spline_rhs(ya, i, h);
    zp[i] = spline_rhs(yp, i, h);
  }
  __syncthreads();
  if ((int)threadIdx.x < 2 * nsrc) {
    const int c = threadIdx.x >> 1;
    if (s_ok[c]) spline_recurrence(psm + (size_t)c * (4 * norb + 1) + (2 + (threadIdx.x & 1)) * norb, norb, g.fac_orb);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nsrc * norb; q += blockDim.x) {
    const int c = q / norb, i = q - c * norb;
    if (!s_ok[c]) continue;
    const double *ya = psm + (size_t)c * (4 * norb + 1), *yp = ya + norb, *za = ya + 2 * norb, *zp = ya + 3 * norb;
    double *amp = ssb + (size_t)(base + c) * 8 * norb, *ph = amp + 4 * norb;
    spline_coeffs(ya, za, i, norb, h, amp);
    spline_coeffs(yp, zp, i, norb, h, ph);
  }
}

// ------------------------------------------------------------ response
struct Pol {
  double Ap, Ac, c2p, s2p;
  const double *amp, *ph;
  const double *x;
  int n;
};

__device__ __forceinline__ void hpc(const Pol &P, double t, double &hp, double &hc, double &hpf, double &hcf) {
  const int j = even_index(P.x, P.n, t);
  const double d = t - P.x[j];
  const double amp = spl_eval(P.amp, P.n, j, d), ph = spl_eval(P.ph, P.n, j, d);
  double sp, cp;
  sincos(ph, &sp, &cp);
  hp = amp * (P.Ap * P.c2p * cp + P.Ac * P.s2p * sp);
  hc = amp * (P.Ac * P.c2p * sp - P.Ap * P.s2p * cp);
  hpf = amp * (-P.Ap * P.c2p * sp + P.Ac * P.s2p * cp);
  hcf = amp * (P.Ac * P.c2p * cp + P.Ap * P.s2p * sp);
}

// One Michelson channel (vertex a, arms b and c) from eight delayed link
// terms; LISA_TDI_spline, utils/src/glass_lisa.c:769-887.
__device__ void tdi_channel(const Pol &P, double tn, int a, int b, int c, const double *App, const double *Apm,
                            const double *Acp, const double *Acm, const double *kr, const double *L, double &Mo,
                            double &Mfo) {
  double m = 0.0, mf = 0.0, hp, hc, hpf, hcf, t;
  t = tn - kr[a] - 2.0 * L[c] - 2.0 * L[b];
  hpc(P, t, hp, hc, hpf, hcf);
  m += hp * Apm[b] + hc * Acm[b];
  m -= hp * App[c] + hc * Acp[c];
  mf += hpf * Apm[b] + hcf * Acm[b];
  mf -= hpf * App[c] + hcf * Acp[c];
  t = tn - kr[b] - L[c] - 2.0 * L[b];
  hpc(P, t, hp, hc, hpf, hcf);
  m -= hp * Apm[c] + hc * Acm[c];
  m += hp * App[c] + hc * Acp[c];
  mf -= hpf * Apm[c] + hcf * Acm[c];
  mf += hpf * App[c] + hcf * Acp[c];
  t = tn - kr[c] - L[b] - 2.0 * L[c];
  hpc(P, t, hp, hc, hpf, hcf);
  m += hp * App[b] + hc * Acp[b];
  m -= hp * Apm[b] + hc * Acm[b];
  mf += hpf * App[b] + hcf * Acp[b];
  mf -= hpf * Apm[b] + hcf * Acm[b];
  t = tn - kr[a] - 2.0 * L[b];
  hpc(P, t, hp, hc, hpf, hcf);
  m -= hp * Apm[b] + hc * Acm[b];
  m += hp * Apm[c] + hc * Acm[c];
  mf -= hpf * Apm[b] + hcf * Acm[b];
  mf += hpf * Apm[c] + hcf * Acm[c];
  t = tn - kr[a] - 2.0 * L[c];
  hpc(P, t, hp, hc, hpf, hcf);
  m += hp * App[c] + hc * Acp[c];
  m -= hp * App[b] + hc * Acp[b];
  mf += hpf * App[c] + hcf * Acp[c];
  mf -= hpf * App[b] + hcf * Acp[b];
  t = tn - kr[c] - L[b];
  hpc(P, t, hp, hc, hpf, hcf);
  m -= hp * App[b] + hc * Acp[b];
  m += hp * Apm[b] + hc * Acm[b];
  mf -= hpf * App[b] + hcf * Acp[b];
  mf += hpf * Apm[b] + hcf * Acm[b];
  t = tn - kr[b] - L[c];
  hpc(P, t, hp, hc, hpf, hcf);
  m += hp * Apm[c] + hc * Acm[c];
  m -= hp * App[c] + hc * Acp[c];
  mf += hpf * Apm[c] + hcf * Acm[c];
  mf -= hpf * App[c] + hcf * Acp[c];
  t = tn - kr[a];
  hpc(P, t, hp, hc, hpf, hcf);
  m -= hp * Apm[c] + hc * Acm[c];
  m += hp * App[b] + hc * Acp[b];
  mf -= hpf * Apm[c] + hcf * Acm[c];
  mf += hpf * App[b] + hcf * Acp[b];
  Mo = m;
  Mfo = mf;
}

// LISA_spline_response (utils/src/glass_lisa.c:920-1074) at one node, plus the
// S/C-1 phase used as the reference phase (LISA_spacecraft_to_barycenter_time).
__global__ void wv_resp_kernel(WvGridDev g, int n, const WvSrc *srcs, const double *ssb, double *resp) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int norb = g.norb;
  if (idx >= (long long)n * norb) return;
  const int s = (int)(idx / norb), m = (int)(idx - (long long)s * norb);
  const WvSrc &S = srcs[s];
  if (S.status) return;
  const double *amp = ssb + (size_t)s * 8 * norb, *ph = amp + 4 * norb;
  const double t = g.tssb[m];
  const double *G = g.geo + 21 * (size_t)m;
  double x[3][3], nv[3][3], L[3];
  for (int i = 0; i < 3; i++)
    for (int d = 0; d < 3; d++) {
      x[i][d] = G[3 * i + d];
      nv[i][d] = G[9 + 3 * i + d];
    }
  for (int i = 0; i < 3; i++) L[i] = G[18 + i];
  const double k[3] = {S.k[0], S.k[1], S.k[2]};
  double kr0 = 0.0;
  for (int d = 0; d < 3; d++) kr0 += k[d] * x[0][d];
  const double tsc = t - kr0;
  double *out = resp + (size_t)s * 7 * norb;
  {
    const int j = even_index(g.orb_t, norb, tsc);
    out[6 * norb + m] = spl_eval(ph, norb, j, tsc - g.orb_t[j]);
  }
  double kr[3], kn[3], dp[3], dc[3], App[3], Apm[3], Acp[3], Acm[3];
  for (int i = 0; i < 3; i++) {
    kr[i] = 0.0;
    for (int d = 0; d < 3; d++) kr[i] += k[d] * x[i][d];
  }
  for (int i = 0; i < 3; i++) {
    kn[i] = 0.0;
    for (int d = 0; d < 3; d++) kn[i] += k[d] * nv[i][d];
  }
  for (int i = 0; i < 3; i++) {
    dp[i] = 0.0;
    dc[i] = 0.0;
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) {
        dp[i] += (nv[i][a] * nv[i][b]) * S.ep[3 * a + b];
        dc[i] += (nv[i][a] * nv[i][b]) * S.ec[3 * a + b];
      }
  }
  for (int i = 0; i < 3; i++) {
    App[i] = dp[i] / (1.0 + kn[i]);
    Apm[i] = dp[i] / (1.0 - kn[i]);
    Acp[i] = dc[i] / (1.0 + kn[i]);
    Acm[i] = dc[i] / (1.0 - kn[i]);
  }
  Pol P{S.Ap, S.Ac, S.c2p, S.s2p, amp, ph, g.orb_t, norb};
  double M, Mf;
  tdi_channel(P, t, 0, 1, 2, App, Apm, Acp, Acm, kr, L, M, Mf);
  out[0 * norb + m] = M;
  out[3 * norb + m] = Mf;
  tdi_channel(P, t, 1, 2, 0, App, Apm, Acp, Acm, kr, L, M, Mf);
  out[1 * norb + m] = M;
  out[4 * norb + m] = Mf;
  tdi_channel(P, t, 2, 0, 1, App, Apm, Acp, Acm, kr, L, M, Mf);
  out[2 * norb + m] = M;
  out[5 * norb + m] = Mf;
}

// ------------------------------------------------------------ TDI splines
// extract_amplitude_and_phase + unwrap_phase (utils/src/glass_math.c:1244-1308,
// 1034-1052) and the channel's amplitude / phase splines; one thread per
// (source, channel).  The flip and phase-jump arrays live in the slots of
// the spline's c1 and c2 coefficients until the sweeps overwrite them.
// C (source, channel) pairs per CTA of 128 threads, 4 norb doubles of shared
// memory per pair: the per-node work (|M + i Mf|, atan2, remainder, the spline
// right-hand sides and coefficients) over all threads (node-parallel); the
// flip scan, the unwrapping scan and the spline recurrences on one thread per
// pair (per array for the recurrences).  The flip and phase-jump arrays use
// the slots of the two right-hand-side arrays until those are formed.  Every
// value has the same FP64 expression as in one sequential pass.
template <int C>
__global__ void __launch_bounds__(128) wv_tdi_kernel(WvGridDev g, int n, const WvSrc *srcs, const double *resp,
                                                     double *tdi) {
  extern __shared__ __align__(16) double tsm[];
  __shared__ int s_ok[C];
  const int base = blockIdx.x * C;
  const int nch = min(C, 3 * n - base);
  const int N = g.norb;
  if ((int)threadIdx.x < nch) s_ok[threadIdx.x] = srcs[(base + threadIdx.x) / 3].status == 0;
  __syncthreads();
  // per pair c: As (values of the amplitude spline), Q (phase), then za, zp
  // (flip and pj until the right-hand sides overwrite them)
#define WV_TDI_PTRS                                                       \
  const int idx = base + c, s = idx / 3, ch = idx - 3 * (idx / 3);       \
  double *As = tsm + (size_t)c * (4 * N + 1), *Q = As + N, *za = As + 2 * N, *zp = As + 3 * N; \
  const double *M = resp + ((size_t)s * 7 + ch) * N, *Mf = resp + ((size_t)s * 7 + 3 + ch) * N; \
  (void)M;                                                                \
  (void)Mf;                                                               \
  (void)Q;                                                                \
  (void)za;                                                               \
  (void)zp;
  for (int q = threadIdx.x; q < nch * N; q += blockDim.x) {
    const int c = q / N, i = q - c * N;
    if (!s_ok[c]) continue;
    WV_TDI_PTRS
    As[i] = sqrt(M[i] * M[i] + Mf[i] * Mf[i]);
  }
  __syncthreads();
  if ((int)threadIdx.x < nch && s_ok[threadIdx.x]) {
    const int c = threadIdx.x;
    WV_TDI_PTRS
    double *flip = za, *pj = zp;
    flip[0] = 1.0;
    pj[0] = 0.0;
    int i = 1;
    do {
      flip[i] = flip[i - 1];
      pj[i] = pj[i - 1];
      if ((As[i] < As[i - 1]) && (As[i] < As[i + 1])) {
        const double d1 = As[i + 1] + As[i - 1] - 2.0 * As[i];
        const double d2 = -As[i + 1] + As[i - 1] - 2.0 * As[i];
        const double d3 = -As[i + 1] + As[i - 1] + 2.0 * As[i];
        if (fabs(d2 / d1) < 0.1) {
          flip[i + 1] = -1.0 * flip[i];
          pj[i + 1] = pj[i] + kPI;
          i++;
        }
        if (fabs(d3 / d1) < 0.1) {
          flip[i] = -1.0 * flip[i - 1];
          pj[i] = pj[i - 1] + kPI;
        }
      }
      i++;
    } while (i < N - 1);
    flip[N - 1] = flip[N - 2];
    pj[N - 1] = pj[N - 2];
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nch * N; q += blockDim.x) {
    const int c = q / N, i = q - c * N;
    if (!s_ok[c]) continue;
    WV_TDI_PTRS
    const double *phR = resp + ((size_t)s * 7 + 6) * N;
    As[i] = za[i] * As[i];
    const double v = remainder(phR[i], kPI2);
    Q[i] = -atan2(Mf[i], M[i]) + zp[i] - v;
  }
  __syncthreads();
  if ((int)threadIdx.x < nch && s_ok[threadIdx.x]) {
    const int c = threadIdx.x;
    WV_TDI_PTRS
    double v = Q[0];
    for (int i = 0; i < N; i++) {
      double u = Q[i];
      const double qq = rint(fabs(u - v) / (kPI2));
      if (qq > 0.0) {
        if (v > u)
          u += qq * kPI2;
        else
          u -= qq * kPI2;
      }
      v = u;
      Q[i] = u;
    }
  }
  __syncthreads();
  // natural cubic splines of As and Q (utils/src/glass_math.c:101-175)
  const double *h = g.fac_ssb;
  for (int q = threadIdx.x; q < nch * N; q += blockDim.x) {
    const int c = q / N, i = q - c * N;
    if (!s_ok[c] || i == 0 || i == N - 1) continue;
    WV_TDI_PTRS
    za[i] = spline_rhs(As, i, h);
    zp[i] = spline_rhs(Q, i, h);
  }
  __syncthreads();
  if ((int)threadIdx.x < 2 * nch && s_ok[threadIdx.x >> 1]) {
    const int c = threadIdx.x >> 1;
    spline_recurrence(tsm + (size_t)c * (4 * N + 1) + (2 + (threadIdx.x & 1)) * N, N, g.fac_ssb);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nch * N; q += blockDim.x) {
    const int c = q / N, i = q - c * N;
    if (!s_ok[c]) continue;
    WV_TDI_PTRS
    double *ca = tdi + ((size_t)s * 3 + ch) * 8 * N, *cp = ca + 4 * N;
    spline_coeffs(As, za, i, N, h, ca);
    spline_coeffs(Q, zp, i, N, h, cp);
  }
#undef WV_TDI_PTRS
}

// ------------------------------------------------------------ FFTs
// Radices of an in-place decimation-in-time FFT: 3s, then 4s, then a 2.
struct RadixPlan {
  int n;
  int r[24];
  int pre[24];  // R_0 ... R_{s-1}
};

__device__ __forceinline__ void radix_plan(int L, RadixPlan &P) {
  P.n = 0;
  int rem = L, pre = 1;
  while (rem % 3 == 0) {
    P.r[P.n] = 3;
    P.pre[P.n++] = pre;
    pre *= 3;
    rem /= 3;
  }
  while (rem % 4 == 0) {
    P.r[P.n] = 4;
    P.pre[P.n++] = pre;
    pre *= 4;
    rem /= 4;
  }
  while (rem % 2 == 0) {
    P.r[P.n] = 2;
    P.pre[P.n++] = pre;
    pre *= 2;
    rem /= 2;
  }
}

// Input position of element x: its stage digits read in reverse.
__device__ __forceinline__ int digit_rev(int x, const RadixPlan &P) {
  int pos = 0;
  for (int s = P.n - 1; s >= 0; s--) {
    const int d = x % P.r[s];
    x /= P.r[s];
    pos += d * P.pre[s];
  }
  return pos;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C>
__device__ __forceinline__ C mkc(decltype(C::x) x, decltype(C::x) y) {
  C r;
  r.x = x;
  r.y = y;
  return r;
}

// In-place mixed-radix FFT of a[L] held in digit-reversed order; result in
// natural order.  tw[j * twmul] = e^{-2 pi i j / L}; sign -1 forward, +1
// inverse (unnormalised).  Whole CTA.  C = double2 or float2.
template <typename C>
__device__ void dit_fft(C *a, int L, const RadixPlan &P, const C *__restrict__ tw, int twmul, int sign) {
  using R = decltype(C::x);
  int p = 1;
  for (int st = 0; st < P.n; st++) {
    const int Rd = P.r[st], q = p * Rd, nb = L / Rd;
    const int tstep = (L / q) * twmul;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
      const int b = t / p, k = t - b * p;
      C *base = a + (size_t)b * q + k;
      if (Rd == 4) {
        C v0 = base[0], v1 = base[p], v2 = base[2 * p], v3 = base[3 * p];
        C w1 = tw[k * tstep], w2 = tw[2 * k * tstep], w3 = tw[3 * k * tstep];
        if (sign > 0) {
          w1.y = -w1.y;
          w2.y = -w2.y;
          w3.y = -w3.y;
        }
        v1 = cmul(v1, w1);
        v2 = cmul(v2, w2);
        v3 = cmul(v3, w3);
        const C t0 = mkc<C>(v0.x + v2.x, v0.y + v2.y), t1 = mkc<C>(v0.x - v2.x, v0.y - v2.y);
        const C t2 = mkc<C>(v1.x + v3.x, v1.y + v3.y), t3 = mkc<C>(v1.x - v3.x, v1.y - v3.y);
        const C t3r = sign < 0 ? mkc<C>(t3.y, -t3.x) : mkc<C>(-t3.y, t3.x);
        base[0] = mkc<C>(t0.x + t2.x, t0.y + t2.y);
        base[p] = mkc<C>(t1.x + t3r.x, t1.y + t3r.y);
        base[2 * p] = mkc<C>(t0.x - t2.x, t0.y - t2.y);
        base[3 * p] = mkc<C>(t1.x - t3r.x, t1.y - t3r.y);
      } else if (Rd == 2) {
        C v0 = base[0], v1 = base[p];
        C w1 = tw[k * tstep];
        if (sign > 0) w1.y = -w1.y;
        v1 = cmul(v1, w1);
        base[0] = mkc<C>(v0.x + v1.x, v0.y + v1.y);
        base[p] = mkc<C>(v0.x - v1.x, v0.y - v1.y);
      } else {
        C v0 = base[0], v1 = base[p], v2 = base[2 * p];
        C w1 = tw[k * tstep], w2 = tw[2 * k * tstep];
        if (sign > 0) {
          w1.y = -w1.y;
          w2.y = -w2.y;
        }
        v1 = cmul(v1, w1);
        v2 = cmul(v2, w2);
        const R s3 = (R)0.86602540378443864676 * (R)sign;
        const C sm = mkc<C>(v1.x + v2.x, v1.y + v2.y), df = mkc<C>(v1.x - v2.x, v1.y - v2.y);
        const C m1 = mkc<C>(v0.x - (R)0.5 * sm.x, v0.y - (R)0.5 * sm.y);
        const C m2 = mkc<C>(-s3 * df.y, s3 * df.x);
        base[0] = mkc<C>(v0.x + sm.x, v0.y + sm.y);
        base[p] = mkc<C>(m1.x + m2.x, m1.y + m2.y);
        base[2 * p] = mkc<C>(m1.x - m2.x, m1.y - m2.y);
      }
    }
    __syncthreads();
    p = q;
  }
}

// ------------------------------------------------------------ layers
constexpr int kLayerThreads = 256;

__global__ void __launch_bounds__(kLayerThreads) wv_layers_kernel(WvGridDev g, int n, const WvSrc *srcs,
                                                                  const double *ssb, const double *tdi,
                                                                  double *coef, const int *count, const int *list) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  int s = blockIdx.x / 3;
  const int ch = blockIdx.x - 3 * (blockIdx.x / 3);
  if (list) {  // the sources of a re-evaluation list, list[0 .. *count - 1]
    if (s >= *count) return;
    s = list[s];
  }
  const WvSrc &S = srcs[s];
  if (S.status || S.c == 0) return;
  const int nl = S.nl, NT = g.NT, Nds = NT * (nl + 1), M = Nds / 2, norb = g.norb;
  double2 *zb = reinterpret_cast<double2 *>(sm_raw);
  double2 *lb = zb + M;
  RadixPlan PM, PN;
  radix_plan(M, PM);
  radix_plan(NT, PN);
  const double *ph_ssb = ssb + (size_t)s * 8 * norb + 4 * norb;
  const double *ca = tdi + ((size_t)s * 3 + ch) * 8 * norb, *cp = ca + 4 * norb;
  const double k0 = S.k[0], k1 = S.k[1], k2 = S.k[2];
  const double *r0 = g.r0ds[nl];
  const double dtds = g.wdt / (double)(nl + 1);
  // heterodyned samples (build_interpolated_waveform), packed two per complex
  for (int i = threadIdx.x; i < Nds; i += blockDim.x) {
    const double tds = g.t0 + i * dtds;
    const double phhet = kPI2 * S.fhet * tds;
    double kr = 0.0;
    kr += k0 * r0[3 * i + 0];
    kr += k1 * r0[3 * i + 1];
    kr += k2 * r0[3 * i + 2];
    const double tsc = tds - kr;
    const int je = even_index(g.orb_t, norb, tsc);
    const double phds = spl_eval(ph_ssb, norb, je, tsc - g.orb_t[je]);
    const int jb = bin_index(g.tssb, norb, tds);
    const double d = tds - g.tssb[jb];
    const double a = spl_eval(ca, norb, jb, d);
    double p = spl_eval(cp, norb, jb, d);
    p += phds;
    p -= phhet;
    const double w = a * cos(p);
    double *slot = reinterpret_cast<double *>(zb + digit_rev(i >> 1, PM));
    slot[i & 1] = w;
  }
  __syncthreads();
  const double2 *tw = g.tw[nl];
  dit_fft(zb, M, PM, tw, 2, -1);
  const double norm = g.norm_sqrtNF / (nl + 1.0);
  const double *win = g.win[nl];
  double *out = coef + ((size_t)s * 3 + ch) * (kWvMaxLayers * (size_t)NT);
  for (int off = 0; off < nl; off++) {
    const int m = S.jmin + off;
    const int center = (off + 1) * NT / 2;
    for (int t = threadIdx.x; t < NT; t += blockDim.x) {
      const int j = t - NT / 2, idx = center + j;
      double2 val = make_double2(0.0, 0.0);
      if (j > -NT / 2 && idx >= 0 && idx <= M) {
        double wt = win[j < 0 ? -j : j];
        if (j == 0 && (m == 0 || m == g.NF)) wt /= 2.0;
        // bin idx of the real spectrum from the packed spectrum
        const double2 zk = zb[idx % M], zm0 = zb[(M - idx) % M];
        const double2 zm = make_double2(zm0.x, -zm0.y);
        const double2 e = tw[idx];
        const double2 sm = make_double2(zk.x + zm.x, zk.y + zm.y), df = make_double2(zk.x - zm.x, zk.y - zm.y);
        const double2 ed = cmul(e, df);
        const double2 X = make_double2(0.5 * (sm.x + ed.y), 0.5 * (sm.y - ed.x));
        val = make_double2(wt * X.x, wt * X.y);
      }
      lb[digit_rev(t, PN)] = val;
    }
    __syncthreads();
    dit_fft(lb, NT, PN, tw, nl + 1, +1);
    for (int t = threadIdx.x; t < NT; t += blockDim.x) {
      const double re = lb[t].x / NT, im = lb[t].y / NT;
      double v;
      if (m == 0 || m == g.NF) {
        v = (t % 2 == 0) ? re * kSQRT2 * norm : 0.0;
      } else {
        const double sgn = (m % 2 == 0) ? 1.0 : -1.0;
        v = (((t + m) % 2 == 0) ? re : sgn * im) * norm;
      }
      out[(size_t)t * nl + off] = v;
    }
    __syncthreads();
  }
}

// wavelet_transform_timefreq_by_layers (utils/src/glass_wavelet.c:544-610)
// on a caller's series: the real FFT of its N = NT (nl + 1) samples (packed
// two per complex, mixed radix), then per layer the windowed band around its
// centre, an NT-point inverse FFT and the layer's pixels, as the waveform
// kernel above does for its own samples.  One CTA; the output replaces the
// input (zero beyond NT nl).
__global__ void __launch_bounds__(kLayerThreads) wdm_by_layers_kernel(int NF, int NT, int jmin, int nl,
                                                                      const double *win, const double2 *tw,
                                                                      double *data) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  const int Nds = NT * (nl + 1), M = Nds / 2;
  double2 *zb = reinterpret_cast<double2 *>(sm_raw);
  double2 *lb = zb + M;
  RadixPlan PM, PN;
  radix_plan(M, PM);
  radix_plan(NT, PN);
  for (int i = threadIdx.x; i < Nds; i += blockDim.x) {
    double *slot = reinterpret_cast<double *>(zb + digit_rev(i >> 1, PM));
    slot[i & 1] = data[i];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < Nds; i += blockDim.x) data[i] = 0.0;
  dit_fft(zb, M, PM, tw, 2, -1);
  const double norm = sqrt((double)NF) / (nl + 1.0);
  for (int off = 0; off < nl; off++) {
    const int m = jmin + off;
    const int center = (off + 1) * NT / 2;
    for (int t = threadIdx.x; t < NT; t += blockDim.x) {
      const int j = t - NT / 2, idx = center + j;
      double2 val = make_double2(0.0, 0.0);
      if (j > -NT / 2 && idx >= 0 && idx <= M) {
        double wt = win[j < 0 ? -j : j];
        if (j == 0 && (m == 0 || m == NF)) wt /= 2.0;
        const double2 zk = zb[idx % M], zm0 = zb[(M - idx) % M];
        const double2 zm = make_double2(zm0.x, -zm0.y);
        const double2 e = tw[idx];
        const double2 sm = make_double2(zk.x + zm.x, zk.y + zm.y), df = make_double2(zk.x - zm.x, zk.y - zm.y);
        const double2 ed = cmul(e, df);
        const double2 X = make_double2(0.5 * (sm.x + ed.y), 0.5 * (sm.y - ed.x));
        val = make_double2(wt * X.x, wt * X.y);
      }
      lb[digit_rev(t, PN)] = val;
    }
    __syncthreads();
    dit_fft(lb, NT, PN, tw, nl + 1, +1);
    for (int t = threadIdx.x; t < NT; t += blockDim.x) {
      const double re = lb[t].x / NT, im = lb[t].y / NT;
      double v;
      if (m == 0 || m == NF) {
        if (t % 2) continue;  // odd pixels stay zero
        v = re * kSQRT2 * norm;
      } else {
        const double sgn = (m % 2 == 0) ? 1.0 : -1.0;
        v = (((t + m) % 2 == 0) ? re : sgn * im) * norm;
      }
      data[(size_t)t * nl + off] = v;
    }
    __syncthreads();
  }
}


// ------------------------------------------------------------ likelihood
constexpr int kDloglThreads = 256;

__global__ void __launch_bounds__(kDloglThreads) wv_dlogl_kernel(WvGridDev g, int n, const WvSrc *srcs,
                                                                 const double *coef, const double *term_x,
                                                                 double *dlogl, double *term_y, double *hh_out,
                                                                 int *status, const int *count, const int *list) {
  int s = blockIdx.x;
  if (list) {
    if (s >= *count) return;
    s = list[s];
  }
  const WvSrc &S = srcs[s];
  __shared__ double red[2][kDloglThreads / 32];
  if (S.status) {
    if (threadIdx.x == 0) {
      if (dlogl) dlogl[s] = NAN;
      if (term_y) term_y[s] = NAN;
      if (hh_out) hh_out[s] = NAN;
    }
    return;
  }
  const int NT = g.NT, N = g.N, c = S.c, npix = NT * c;
  const double *h0 = coef + (size_t)s * 3 * (kWvMaxLayers * (size_t)NT);
  const double *h1 = h0 + kWvMaxLayers * (size_t)NT, *h2 = h1 + kWvMaxLayers * (size_t)NT;
  const double *r = g.res, *ic = g.invC;
  double dh = 0.0, hh = 0.0;
  for (int q = threadIdx.x; q < npix; q += blockDim.x) {
    const int i = q / c, j = S.jlo + (q - i * c);
    const int k = i + j * NT - g.kmin;
    const double a0 = h0[q], a1 = h1[q], a2 = h2[q];
    const double d0 = r[k], d1 = r[N + k], d2 = r[2 * N + k];
    const double c00 = ic[k], c01 = ic[N + k], c02 = ic[2 * N + k];
    const double c10 = ic[3 * N + k], c11 = ic[4 * N + k], c12 = ic[5 * N + k];
    const double c20 = ic[6 * N + k], c21 = ic[7 * N + k], c22 = ic[8 * N + k];
    dh += d0 * a0 * c00 + d1 * a1 * c11 + d2 * a2 * c22 + d0 * a1 * c01 + d0 * a2 * c02 + d1 * a2 * c12 +
          d1 * a0 * c10 + d2 * a0 * c20 + d2 * a1 * c21;
    hh += a0 * a0 * c00 + a1 * a1 * c11 + a2 * a2 * c22 + a0 * a1 * c01 + a0 * a2 * c02 + a1 * a2 * c12 +
          a1 * a0 * c10 + a2 * a0 * c20 + a2 * a1 * c21;
  }
  for (int o = 16; o > 0; o >>= 1) {
    dh += __shfl_xor_sync(0xffffffffu, dh, o);
    hh += __shfl_xor_sync(0xffffffffu, hh, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = dh;
    red[1][threadIdx.x >> 5] = hh;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    dh = 0.0;
    hh = 0.0;
    for (int w = 0; w < kDloglThreads / 32; w++) {
      dh += red[0][w];
      hh += red[1][w];
    }
    const double term = hh - 2.0 * dh;
    if (term_y) term_y[s] = term;
    if (hh_out) hh_out[s] = hh;
    if (dlogl) {
      const double tx = term_x ? term_x[s] : 0.0;
      dlogl[s] = -0.5 * term - (-0.5 * tx);
    }
    if (status) status[s] = isfinite(term) ? (c == 0 ? 4 : 0) : 1;
  }
}

// ------------------------------------------------------------ mixed precision
// Spline value in FP32 (Horner) from FP64 coefficients (the channel amplitude,
// O(1e-22)).
__device__ __forceinline__ float spl_eval_f(const double *c, int n, int j, float d) {
  return (float)c[j] + d * ((float)c[n + j] + d * ((float)c[2 * n + j] + d * (float)c[3 * n + j]));
}

// Per spline interval j of one (source, channel), the constants the mixed
// sampler needs, built in FP64 and stored as floats / double-floats:
//   carrier (barycentre phase spline on the orbit grid x, heterodyne folded in)
//     pa = (a_j - 2 pi fhet x_j) mod 2 pi, pb = b_j - 2 pi fhet, pc, pd, pt = t0 - x_j
//   channel relative phase (spline on the TDI grid y): ca, cb, cc, cd, ct = t0 - y_j
//   channel amplitude (same grid): aa, ab, ac, ad
struct WvMixInterval {
  float4 p0;  // pa.hi, pa.lo, pb.hi, pb.lo
  float4 p1;  // pc, pd, pt.hi, pt.lo
  float4 c0;  // ca.hi, ca.lo, cb.hi, cb.lo
  float4 c1;  // cc, cd, ct.hi, ct.lo
  float4 a;   // amplitude coefficients
};

// As wv_layers_kernel in mixed precision.  The sample phase — barycentre
// phase at the light-time-shifted time minus the heterodyne, plus the
// channel's relative phase — is evaluated in double-float arithmetic from the
// per-interval constants above (so no FP64 instruction runs per sample), with
// the linear terms and the light-time projection k.r0 in double-float and the
// quadratic and cubic terms (< 0.1 rad) in FP32, then reduced mod 2 pi.  The
// amplitude spline, the cosine, both FFTs and the layer transforms run in
// FP32.  Coefficients are written divided by the segment's noise scale.
__global__ void __launch_bounds__(kLayerThreads) wv_layers_mix_kernel(WvGridDev g, int n, const WvSrc *srcs,
                                                                      const double *ssb, const double *tdi,
                                                                      float *coef) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  const int s = blockIdx.x / 3, ch = blockIdx.x - 3 * (blockIdx.x / 3);
  const WvSrc &S = srcs[s];
  if (S.status || S.c == 0) return;
  const int nl = S.nl, NT = g.NT, Nds = NT * (nl + 1), M = Nds / 2, norb = g.norb;
  float2 *zb = reinterpret_cast<float2 *>(sm_raw);
  float2 *lb = zb + M;
  // interval table: in the layer buffer's place (unused until the samples are in)
  WvMixInterval *tab = reinterpret_cast<WvMixInterval *>((reinterpret_cast<uintptr_t>(lb) + 15) & ~(uintptr_t)15);
  RadixPlan PM, PN;
  radix_plan(M, PM);
  radix_plan(NT, PN);
  const double *ph_ssb = ssb + (size_t)s * 8 * norb + 4 * norb;
  const double *ca = tdi + ((size_t)s * 3 + ch) * 8 * norb, *cp = ca + 4 * norb;
  const double w_het = kPI2 * S.fhet;
  for (int j = threadIdx.x; j < norb; j += blockDim.x) {
    const double x = g.orb_t[j], y = g.tssb[j];
    double pa = ph_ssb[j] - w_het * x;
    pa = pa - kPI2 * rint(pa * (1.0 / kPI2));
    const df dpa = df_from_double(pa), dpb = df_from_double(ph_ssb[norb + j] - w_het);
    const df dpt = df_from_double(g.t0 - x), dca = df_from_double(cp[j]), dcb = df_from_double(cp[norb + j]);
    const df dct = df_from_double(g.t0 - y);
    WvMixInterval I;
    I.p0 = make_float4(dpa.hi, dpa.lo, dpb.hi, dpb.lo);
    I.p1 = make_float4((float)ph_ssb[2 * norb + j], (float)ph_ssb[3 * norb + j], dpt.hi, dpt.lo);
    I.c0 = make_float4(dca.hi, dca.lo, dcb.hi, dcb.lo);
    I.c1 = make_float4((float)cp[2 * norb + j], (float)cp[3 * norb + j], dct.hi, dct.lo);
    I.a = make_float4((float)ca[j], (float)ca[norb + j], (float)ca[2 * norb + j], (float)ca[3 * norb + j]);
    tab[j] = I;
  }
  const df k0 = df_from_double(S.k[0]), k1 = df_from_double(S.k[1]), k2 = df_from_double(S.k[2]);
  const df whet = df_from_double(w_het);
  const df dtds = df_from_double(g.wdt / (double)(nl + 1));
  const float dtds_f = dtds.hi;
  // interval search in FP32: a sample within a few seconds of a node may take
  // the neighbouring interval, whose cubic agrees there to rounding
  const float x0 = (float)(g.t0 - g.orb_t[0]), inv_dx = (float)(1.0 / (g.orb_t[1] - g.orb_t[0]));
  const float y0 = (float)(g.t0 - g.tssb[0]), inv_dy = (float)(1.0 / (g.tssb[1] - g.tssb[0]));
  const float *r0h = g.r0hi[nl], *r0l = g.r0lo[nl];
  __syncthreads();
  for (int i = threadIdx.x; i < Nds; i += blockDim.x) {
    const float fi = (float)i;
    const df idt = df_mul_f(dtds, fi);  // tds - t0
    df kr = df_mul(k0, df{r0h[3 * i + 0], r0l[3 * i + 0]});
    kr = df_add(kr, df_mul(k1, df{r0h[3 * i + 1], r0l[3 * i + 1]}));
    kr = df_add(kr, df_mul(k2, df{r0h[3 * i + 2], r0l[3 * i + 2]}));
    const float tf = fmaf(fi, dtds_f, 0.f);
    const int je = min(max((int)floorf((x0 + tf - kr.hi) * inv_dx), 0), norb - 1);
    const int jb = min(max((int)floorf((y0 + tf) * inv_dy), 0), norb - 2);
    const WvMixInterval &P = tab[je];
    const WvMixInterval &C = tab[jb];
    const float4 p0 = P.p0, p1 = P.p1, c0 = C.c0, c1 = C.c1, am = C.a;
    // u = tsc - x_je = (t0 - x_je) + (tds - t0) - k.r0;  v = tds - y_jb
    const df u = df_add(df_add(df{p1.z, p1.w}, idt), df_neg(kr));
    const df v = df_add(df{c1.z, c1.w}, idt);
    const float uf = u.hi, vf = v.hi;
    df ph = df_add(df{p0.x, p0.y}, df_mul(df{p0.z, p0.w}, u));
    ph = df_add(ph, df_neg(df_mul(whet, kr)));
    ph = df_add(ph, df{c0.x, c0.y});
    ph = df_add(ph, df_mul(df{c0.z, c0.w}, v));
    const float small = fmaf(fmaf(p1.y, uf, p1.x), uf * uf, fmaf(c1.y, vf, c1.x) * (vf * vf));
    ph = df_add(ph, df{small, 0.f});
    const float pr = df_reduce_2pi(ph);
    const float a = fmaf(fmaf(fmaf(am.w, vf, am.z), vf, am.y), vf, am.x);
    float *slot = reinterpret_cast<float *>(zb + digit_rev(i >> 1, PM));
    slot[i & 1] = a * cosf(pr);
  }
  __syncthreads();
  const float2 *tw = g.tw32[nl];
  dit_fft(zb, M, PM, tw, 2, -1);
  const float norm = (float)(g.norm_sqrtNF / (nl + 1.0) / g.scale / NT);
  const float *win = g.win32[nl];
  float *out = coef + ((size_t)s * 3 + ch) * (kWvMaxLayers * (size_t)NT);
  for (int off = 0; off < nl; off++) {
    const int m = S.jmin + off;
    const int center = (off + 1) * NT / 2;
    for (int t = threadIdx.x; t < NT; t += blockDim.x) {
      const int j = t - NT / 2, idx = center + j;
      float2 val = make_float2(0.f, 0.f);
      if (j > -NT / 2 && idx >= 0 && idx <= M) {
        float wt = win[j < 0 ? -j : j];
        if (j == 0 && (m == 0 || m == g.NF)) wt *= 0.5f;
        const float2 zk = zb[idx % M], zm0 = zb[(M - idx) % M];
        const float2 zm = make_float2(zm0.x, -zm0.y);
        const float2 e = tw[idx];
        const float2 sm = make_float2(zk.x + zm.x, zk.y + zm.y), df = make_float2(zk.x - zm.x, zk.y - zm.y);
        const float2 ed = cmul(e, df);
        val = make_float2(wt * 0.5f * (sm.x + ed.y), wt * 0.5f * (sm.y - ed.x));
      }
      lb[digit_rev(t, PN)] = val;
    }
    __syncthreads();
    dit_fft(lb, NT, PN, tw, nl + 1, +1);
    for (int t = threadIdx.x; t < NT; t += blockDim.x) {
      const float re = lb[t].x * norm, im = lb[t].y * norm;
      float v;
      if (m == 0 || m == g.NF) {
        v = (t % 2 == 0) ? re * (float)kSQRT2 : 0.f;
      } else {
        v = ((t + m) % 2 == 0) ? re : ((m % 2 == 0) ? im : -im);
      }
      out[(size_t)t * nl + off] = v;
    }
    __syncthreads();
  }
}

// Sparse delta logL, term = sum over the source's pixels of h^T invC h -
// 2 h^T invC r, in FP32 products (r/s as hi + lo floats, invC s^2, h/s) with
// double-float sums.  Per pixel the form with the smaller rounding error is
// used: the residual form e^T invC e - r^T invC r (e = r - h, the FP64 data
// term subtracted) where the template matches the data, the direct form
// h^T invC (h - 2 r) where the data is much louder than the template.
__global__ void __launch_bounds__(kDloglThreads) wv_dlogl_mix_kernel(WvGridDev g, int n, const WvSrc *srcs,
                                                                     const float *coef, const double *term_x,
                                                                     double *dlogl, double *term_y, double *hh_out,
                                                                     int *status, double kest, int *count, int *list,
                                                                     unsigned long long *total) {
  const int s = blockIdx.x;
  const WvSrc &S = srcs[s];
  __shared__ float2 red[2][kDloglThreads / 32];
  __shared__ double redq[kDloglThreads / 32];
  __shared__ float rede[kDloglThreads / 32];
  if (S.status) {
    if (threadIdx.x == 0) {
      if (dlogl) dlogl[s] = NAN;
      if (term_y) term_y[s] = NAN;
      if (hh_out) hh_out[s] = NAN;
    }
    return;
  }
  const int NT = g.NT, N = g.N, c = S.c, npix = NT * c;
  const float *h0 = coef + (size_t)s * 3 * (kWvMaxLayers * (size_t)NT);
  const float *h1 = h0 + kWvMaxLayers * (size_t)NT, *h2 = h1 + kWvMaxLayers * (size_t)NT;
  const float *rh = g.res_hi, *rl = g.res_lo, *ic = g.invC32;
  df acc = {0.f, 0.f}, hacc = {0.f, 0.f};
  double qacc = 0.0;
  float eacc = 0.f;  // (r - h)^T C (r - h), for the error estimate
  for (int q = threadIdx.x; q < npix; q += blockDim.x) {
    const int i = q / c, j = S.jlo + (q - i * c);
    const int k = i + j * NT - g.kmin;
    const float a0 = h0[q], a1 = h1[q], a2 = h2[q];
    const float r0h = rh[k], r1h = rh[N + k], r2h = rh[2 * N + k];
    const float r0l = rl[k], r1l = rl[N + k], r2l = rl[2 * N + k];
    const float c00 = ic[k], c01 = ic[N + k], c02 = ic[2 * N + k];
    const float c10 = ic[3 * N + k], c11 = ic[4 * N + k], c12 = ic[5 * N + k];
    const float c20 = ic[6 * N + k], c21 = ic[7 * N + k], c22 = ic[8 * N + k];
    const float th = a0 * (a0 * c00 + a1 * c01 + a2 * c02) + a1 * (a0 * c10 + a1 * c11 + a2 * c12) +
                     a2 * (a0 * c20 + a1 * c21 + a2 * c22);
    const float e0 = (r0h - a0) + r0l, e1 = (r1h - a1) + r1l, e2 = (r2h - a2) + r2l;
    const float ee = e0 * e0 + e1 * e1 + e2 * e2;
    const float hn = a0 * a0 + a1 * a1 + a2 * a2, rn = r0h * r0h + r1h * r1h + r2h * r2h;
    const float te = e0 * (e0 * c00 + e1 * c01 + e2 * c02) + e1 * (e0 * c10 + e1 * c11 + e2 * c12) +
                     e2 * (e0 * c20 + e1 * c21 + e2 * c22);
    eacc += te;
    float t;
    if (ee * ee <= hn * (hn + 4.f * rn)) {
      // residual form: rounding ~ |e|^2, the data term exact in FP64
      t = te;
      qacc += g.qpix[k];
    } else {
      // direct form: rounding ~ |h| (|h| + 2 |r|)
      const float u0 = (a0 - 2.f * r0h) - 2.f * r0l, u1 = (a1 - 2.f * r1h) - 2.f * r1l,
                  u2 = (a2 - 2.f * r2h) - 2.f * r2l;
      t = a0 * (c00 * u0 + c01 * u1 + c02 * u2) + a1 * (c10 * u0 + c11 * u1 + c12 * u2) +
          a2 * (c20 * u0 + c21 * u1 + c22 * u2);
    }
    acc = df_add(acc, df{t, 0.f});
    hacc = df_add(hacc, df{th, 0.f});
  }
  for (int o = 16; o > 0; o >>= 1) {
    const df ao = {__shfl_xor_sync(0xffffffffu, acc.hi, o), __shfl_xor_sync(0xffffffffu, acc.lo, o)};
    const df ho = {__shfl_xor_sync(0xffffffffu, hacc.hi, o), __shfl_xor_sync(0xffffffffu, hacc.lo, o)};
    acc = df_add(acc, ao);
    hacc = df_add(hacc, ho);
    qacc += __shfl_xor_sync(0xffffffffu, qacc, o);
    eacc += __shfl_xor_sync(0xffffffffu, eacc, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = make_float2(acc.hi, acc.lo);
    red[1][threadIdx.x >> 5] = make_float2(hacc.hi, hacc.lo);
    redq[threadIdx.x >> 5] = qacc;
    rede[threadIdx.x >> 5] = eacc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sr = 0.0, sh = 0.0, sq = 0.0, se = 0.0;
    for (int w = 0; w < kDloglThreads / 32; w++) {
      sr += (double)red[0][w].x + (double)red[0][w].y;
      sh += (double)red[1][w].x + (double)red[1][w].y;
      sq += redq[w];
      se += (double)rede[w];
    }
    const double term = sr - sq;
    // The template's error delta h gives |delta logL error| ~
    // |delta h^T C (h - r)| <~ kWvMixedErrK sqrt((h|h) (r-h|r-h)); past the
    // tolerance, or not finite, the source is listed for FP64.
    if (kest > 0.0 && c != 0 && (!isfinite(term) || !(kest * sqrt(fmax(sh, 0.0) * fmax(se, 0.0)) <= 1.0))) {
      list[atomicAdd(count, 1)] = s;
      atomicAdd(total, 1ull);
    }
    if (term_y) term_y[s] = term;
    if (hh_out) hh_out[s] = sh;
    if (dlogl) {
      const double tx = term_x ? term_x[s] : 0.0;
      dlogl[s] = -0.5 * term - (-0.5 * tx);
    }
    if (status) status[s] = isfinite(term) ? (c == 0 ? 4 : 0) : 1;
  }
}

__global__ void wv_unscale_kernel(const float *in, double *out, long long n, double scale) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i] * scale;
}

__global__ void wv_info_kernel(int n, const WvSrc *srcs, int *info) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  info[4 * s + 0] = srcs[s].jmin;
  info[4 * s + 1] = srcs[s].nl;
  info[4 * s + 2] = srcs[s].jlo;
  info[4 * s + 3] = srcs[s].status ? -1 : srcs[s].c;
}

}  // namespace

// ================================================================ host side
// initialize_interpolated_analytic_orbits (utils/src/glass_lisa.c:271-380) with
// analytic_orbits (:77-124)
void wv_analytic_orbit(double Tobs, double t0, std::vector<double> &t, std::vector<double> &pos) {
  int n = (int)(kOrbSamplesPerYear * Tobs / kYEAR);
  if (n < 20) n = 20;
  const double buffer = Tobs / (double)(n - 1);
  const double cadence = (Tobs + 2.0 * buffer) / (double)(n - 1);
  const double R = kAU * (kLARM / (2.0 * kSQ3 * kAU));
  static const double sbs[3] = {0.0, 0.866025403784439, -0.866025403784438};
  static const double cbs[3] = {1.0, -0.5, -0.5};
  t.resize(n);
  pos.resize((size_t)9 * n);
  for (int k = 0; k < n; k++) {
    const double tt = t0 + k * cadence - buffer;
    const double alpha = kPI2 * tt / kYEAR;
    const double sa = sin(alpha), ca = cos(alpha);
    const double sa2 = sa * sa, ca2 = ca * ca, saca = sa * ca, AUca = kAU * ca, AUsa = kAU * sa;
    t[k] = tt;
    for (int i = 0; i < 3; i++) {
      const double sb = sbs[i], cb = cbs[i];
      pos[(size_t)(3 * i + 0) * n + k] = AUca + R * (saca * sb - (1. + sa2) * cb);
      pos[(size_t)(3 * i + 1) * n + k] = AUsa + R * (saca * cb - (1. + ca2) * sb);
      pos[(size_t)(3 * i + 2) * n + k] = -kSQ3 * R * (ca * cb + sa * sb);
    }
  }
}

namespace {

// Host copy of the cubic spline (same arithmetic as warp_spline_pair plus the
// grid factors), evaluated with the binary-search lookup.
struct HostSpline {
  int n = 0;
  const double *x = nullptr;
  std::vector<double> c;  // [4][n]
};

static void grid_factors(const double *x, int n, double *fac) {
  double *h = fac, *l = fac + n, *mu = fac + 2 * n;
  for (int i = 0; i < 3 * n; i++) fac[i] = 0.0;
  h[0] = x[1] - x[0];
  for (int i = 1; i < n - 1; i++) h[i] = x[i + 1] - x[i];
  l[0] = l[n - 1] = 1.0;
  for (int i = 1; i < n - 1; i++) {
    l[i] = 2.0 * (x[i + 1] - x[i - 1]) - h[i - 1] * mu[i - 1];
    mu[i] = h[i] / l[i];
  }
}

static void host_spline(HostSpline &sp, const double *x, const double *y, int n, const double *fac) {
  sp.n = n;
  sp.x = x;
  sp.c.assign((size_t)4 * n, 0.0);
  double *c0 = sp.c.data(), *c1 = c0 + n, *c2 = c0 + 2 * n, *c3 = c0 + 3 * n;
  const double *h = fac, *l = fac + n, *mu = fac + 2 * n;
  for (int i = 0; i < n; i++) c0[i] = y[i];
  double z = 0.0;
  c2[0] = 0.0;
  for (int i = 1; i < n - 1; i++) {
    const double al = 3.0 * ((c0[i + 1] - c0[i]) / h[i] - (c0[i] - c0[i - 1]) / h[i - 1]);
    z = (al - h[i - 1] * z) / l[i];
    c2[i] = z;
  }
  c1[n - 1] = c2[n - 1] = c3[n - 1] = 0.0;
  for (int i = n - 2; i >= 0; i--) {
    c2[i] = c2[i] - mu[i] * c2[i + 1];
    c1[i] = (c0[i + 1] - c0[i]) / h[i] - h[i] * (c2[i + 1] + 2.0 * c2[i]) / 3.0;
    c3[i] = (c2[i + 1] - c2[i]) / (3.0 * h[i]);
  }
}

static double host_eval(const HostSpline &sp, double v) {
  const int n = sp.n;
  const double *x = sp.x;
  int j;
  if (!(v > x[0])) {
    j = 0;
  } else if (v >= x[n - 1]) {
    j = v == x[n - 1] ? n - 1 : n - 2;
  } else {
    j = (int)(std::upper_bound(x, x + n, v) - x) - 1;
  }
  const double d = v - x[j];
  const double *c = sp.c.data();
  return c[j] + c[n + j] * d + c[2 * n + j] * d * d + c[3 * n + j] * d * d * d;
}

static void unit_root(long long j, long long P, double *c, double *s) {
  long long r = j % P;
  if (r < 0) r += P;
  double sg = -1.0;
  if (2 * r > P) {
    r = P - r;
    sg = 1.0;
  }
  const double a = 2.0 * M_PI * ((double)r / (double)P);
  *c = cos(a);
  *s = sg * sin(a);
}

}  // namespace

cudaError_t wdm_by_layers_launch(int NF, int NT, int jmin, int nl, const double *d_win, const double2 *d_tw,
                                 double *d_data, cudaStream_t s) {
  const size_t sm = sizeof(double2) * ((size_t)NT * (nl + 1) / 2 + NT);
  cudaError_t e = cudaFuncSetAttribute(wdm_by_layers_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  wdm_by_layers_kernel<<<1, kLayerThreads, sm, s>>>(NF, NT, jmin, nl, d_win, d_tw, d_data);
  return cudaGetLastError();
}

void wdm_unit_roots(int P, double2 *out) {
  for (int k = 0; k < P; k++) {
    double c, sn;
    unit_root(k, P, &c, &sn);
    out[k] = make_double2(c, sn);
  }
}


size_t wv_work_bytes(int cap, int norb, int NT) {
  auto pad = [](size_t b) { return (b + 255) / 256 * 256; };
  return pad(sizeof(WvSrc) * (size_t)cap) + pad(sizeof(double) * (size_t)cap * 8 * norb) +
         pad(sizeof(double) * (size_t)cap * 7 * norb) + pad(sizeof(double) * (size_t)cap * 24 * norb) +
         pad(sizeof(double) * (size_t)cap * 3 * kWvMaxLayers * NT) + pad(sizeof(unsigned long long)) +
         pad(sizeof(int) * ((size_t)cap + 1));
}

void wv_work_carve(WvWorkDev &w, void *base, int cap, int norb, int NT) {
  auto pad = [](size_t b) { return (b + 255) / 256 * 256; };
  char *p = (char *)base;
  w.cap = cap;
  w.src = (WvSrc *)p;
  p += pad(sizeof(WvSrc) * (size_t)cap);
  w.ssb = (double *)p;
  p += pad(sizeof(double) * (size_t)cap * 8 * norb);
  w.resp = (double *)p;
  p += pad(sizeof(double) * (size_t)cap * 7 * norb);
  w.tdi = (double *)p;
  p += pad(sizeof(double) * (size_t)cap * 24 * norb);
  w.coef = (double *)p;
  p += pad(sizeof(double) * (size_t)cap * 3 * kWvMaxLayers * NT);
  w.total = (unsigned long long *)p;
  p += pad(sizeof(unsigned long long));
  w.count = (int *)p;
  w.list = w.count + 1;
}

cudaError_t wv_build_grid(const WvGridHost &h, WvGridDev *g, void **mem, cudaStream_t s) {
  const int norb = (int)h.orb_t.size(), NT = h.NT;
  if (norb < 20 || norb > kWvMaxOrb || NT < 8 || NT > kWvMaxNT) return cudaErrorInvalidValue;
  // orbit position splines on the orbit nodes
  std::vector<double> fac_orb(3 * (size_t)norb), fac_ssb(3 * (size_t)norb), tssb(norb);
  grid_factors(h.orb_t.data(), norb, fac_orb.data());
  HostSpline pos[9];
  for (int q = 0; q < 9; q++) host_spline(pos[q], h.orb_t.data(), h.orb_pos.data() + (size_t)q * norb, norb,
                                          fac_orb.data());
  const double dt = h.Tobs / (double)(norb - 1);
  for (int i = 0; i < norb; i++) tssb[i] = h.t0 + i * dt;
  grid_factors(tssb.data(), norb, fac_ssb.data());
  // S/C positions, unit arm vectors and arm lengths at the TDI nodes
  std::vector<double> geo(21 * (size_t)norb);
  for (int m = 0; m < norb; m++) {
    double x[3][3], nv[3][3], L[3];
    for (int i = 0; i < 3; i++)
      for (int d = 0; d < 3; d++) x[i][d] = host_eval(pos[3 * i + d], tssb[m]) / kCLIGHT;
    for (int d = 0; d < 3; d++) {
      nv[0][d] = x[1][d] - x[2][d];
      nv[1][d] = x[2][d] - x[0][d];
      nv[2][d] = x[0][d] - x[1][d];
    }
    for (int i = 0; i < 3; i++) {
      L[i] = 0.0;
      for (int d = 0; d < 3; d++) L[i] += nv[i][d] * nv[i][d];
      L[i] = sqrt(L[i]);
    }
    for (int i = 0; i < 3; i++)
      for (int d = 0; d < 3; d++) nv[i][d] /= L[i];
    double *G = geo.data() + 21 * (size_t)m;
    for (int i = 0; i < 3; i++)
      for (int d = 0; d < 3; d++) {
        G[3 * i + d] = x[i][d];
        G[9 + 3 * i + d] = nv[i][d];
      }
    for (int i = 0; i < 3; i++) G[18 + i] = L[i];
  }
  // per layer count: S/C 1 at the downsampled times, window, twiddles
  std::vector<double> r0[kWvMaxLayers + 1], win[kWvMaxLayers + 1];
  std::vector<double2> tw[kWvMaxLayers + 1];
  std::vector<float> win32[kWvMaxLayers + 1], r0hi[kWvMaxLayers + 1], r0lo[kWvMaxLayers + 1];
  std::vector<float2> tw32[kWvMaxLayers + 1];
  for (int nl = 1; nl <= kWvMaxLayers; nl++) {
    const int Nds = NT * (nl + 1);
    const double dtds = h.wdt / (double)(nl + 1);
    r0[nl].resize(3 * (size_t)Nds);
    for (int i = 0; i < Nds; i++) {
      const double tds = h.t0 + i * dtds;
      for (int d = 0; d < 3; d++) r0[nl][3 * (size_t)i + d] = host_eval(pos[d], tds) / kCLIGHT;
    }
    win[nl].resize(NT / 2 + 1);
    wdm_window(nl + 1, NT, h.A, h.nx, true, win[nl].data());
    tw[nl].resize(Nds);
    tw32[nl].resize(Nds);
    for (int k = 0; k < Nds; k++) {
      double c, sn;
      unit_root(k, Nds, &c, &sn);
      tw[nl][k] = make_double2(c, sn);
      tw32[nl][k] = make_float2((float)c, (float)sn);
    }
    win32[nl].assign(win[nl].begin(), win[nl].end());
    r0hi[nl].resize(r0[nl].size());
    r0lo[nl].resize(r0[nl].size());
    for (size_t q = 0; q < r0[nl].size(); q++) {
      r0hi[nl][q] = (float)r0[nl][q];
      r0lo[nl][q] = (float)(r0[nl][q] - (double)r0hi[nl][q]);
    }
  }
  // one allocation
  auto pad = [](size_t b) { return (b + 255) / 256 * 256; };
  size_t bytes = pad(8 * (size_t)norb) * 2 + pad(8 * geo.size()) + pad(8 * fac_orb.size()) * 2;
  for (int nl = 1; nl <= kWvMaxLayers; nl++)
    bytes += pad(8 * r0[nl].size()) + pad(8 * win[nl].size()) + pad(16 * tw[nl].size()) + pad(4 * win32[nl].size()) +
             pad(8 * tw32[nl].size()) + 2 * pad(4 * r0hi[nl].size());
  char *base = nullptr;
  cudaError_t e = cudaMalloc((void **)&base, bytes);
  if (e != cudaSuccess) return e;
  *mem = base;
  char *p = base;
  auto put = [&](const void *src, size_t b) -> const void * {
    void *dst = p;
    p += pad(b);
    e = e != cudaSuccess ? e : cudaMemcpyAsync(dst, src, b, cudaMemcpyHostToDevice, s);
    return dst;
  };
  g->orb_t = (const double *)put(h.orb_t.data(), 8 * (size_t)norb);
  g->tssb = (const double *)put(tssb.data(), 8 * (size_t)norb);
  g->geo = (const double *)put(geo.data(), 8 * geo.size());
  g->fac_orb = (const double *)put(fac_orb.data(), 8 * fac_orb.size());
  g->fac_ssb = (const double *)put(fac_ssb.data(), 8 * fac_ssb.size());
  g->r0ds[0] = nullptr;
  g->win[0] = nullptr;
  g->tw[0] = nullptr;
  g->win32[0] = nullptr;
  g->tw32[0] = nullptr;
  g->r0hi[0] = g->r0lo[0] = nullptr;
  for (int nl = 1; nl <= kWvMaxLayers; nl++) {
    g->r0ds[nl] = (const double *)put(r0[nl].data(), 8 * r0[nl].size());
    g->win[nl] = (const double *)put(win[nl].data(), 8 * win[nl].size());
    g->tw[nl] = (const double2 *)put(tw[nl].data(), 16 * tw[nl].size());
    g->win32[nl] = (const float *)put(win32[nl].data(), 4 * win32[nl].size());
    g->tw32[nl] = (const float2 *)put(tw32[nl].data(), 8 * tw32[nl].size());
    g->r0hi[nl] = (const float *)put(r0hi[nl].data(), 4 * r0hi[nl].size());
    g->r0lo[nl] = (const float *)put(r0lo[nl].data(), 4 * r0lo[nl].size());
  }
  if (e != cudaSuccess) return e;
  g->NF = h.NF;
  g->NT = NT;
  g->norb = norb;
  g->kmin = h.kmin;
  g->kmax = h.kmax;
  g->N = h.kmax - h.kmin;
  g->lmin = h.kmin / NT;
  g->lmax = h.kmax / NT;
  g->Tobs = h.Tobs;
  g->t0 = h.t0;
  g->wdt = h.wdt;
  g->wdf = h.wdf;
  g->A = h.A;
  g->norm_sqrtNF = sqrt((double)h.NF);
  return cudaStreamSynchronize(s);  // host vectors go out of scope
}

static size_t layers_smem(int NT) { return sizeof(double2) * (size_t)NT * (kWvMaxLayers + 1) / 2 + sizeof(double2) * NT; }

// ------------------------------------------------------------ Fisher matrix
// ucb_fisher_wavelet (ucb/src/glass_ucb_waveform.c:524-640) for a batch of
// sources: central differences with step 1e-6 (each parameter +-5e-7, the
// cosine parameters clamped to [-1, 1]) of 16 FP64 wavelet waveforms per
// source, on the pixels of each + waveform's list whose time index t has
// imin < t < imax, and the Fisher matrix as the nine XYZ cross terms of invC
// per pixel (wavelet_nwip, utils/src/glass_math.c:382-391).
constexpr double kFisherEps = 1.0e-6;

// Row 16 s + 2 i (+) and 16 s + 2 i + 1 (-) of the perturbed parameters.
__global__ void wv_fisher_params_kernel(int n, const double *params, double *pp) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 16 * n) return;
  const int s = idx >> 4, r = idx & 15, i = r >> 1;
  double *o = pp + 8 * (size_t)idx;
  for (int k = 0; k < 8; k++) o[k] = params[8 * (size_t)s + k];
  if ((r & 1) == 0) {
    o[i] += kFisherEps / 2.;
    if ((i == 1 || i == 4) && o[i] > 1.0) o[i] = 1.0;
  } else {
    o[i] -= kFisherEps / 2.;
    if ((i == 1 || i == 4) && o[i] < -1.0) o[i] = -1.0;
  }
}

constexpr int kFisherThreads = 256;

__global__ void __launch_bounds__(kFisherThreads) wv_fisher_kernel(WvGridDev g, int n, const WvSrc *srcs,
                                                                   const double *coef, int imin, int imax,
                                                                   double *fisher, int *status) {
  const int s = blockIdx.x;
  const WvSrc *S = srcs + 16 * (size_t)s;
  __shared__ double red[kFisherThreads / 32][36];
  int st = 0;
  for (int r = 0; r < 16; r++) st |= S[r].status;
  if (st) {
    if (threadIdx.x < 64 && fisher) fisher[64 * (size_t)s + threadIdx.x] = NAN;
    if (threadIdx.x == 0 && status) status[s] = st;
    return;
  }
  const int NT = g.NT, N = g.N;
  const size_t LNT = (size_t)kWvMaxLayers * NT;
  // union of the + waveforms' kept layers
  int jl = 1 << 30, jh = -(1 << 30);
  for (int i = 0; i < 8; i++)
    if (S[2 * i].c > 0) {
      jl = min(jl, S[2 * i].jlo);
      jh = max(jh, S[2 * i].jlo + S[2 * i].c);
    }
  const int nj = jh > jl ? jh - jl : 0;
  const double inv = 1. / (kFisherEps);
  double acc[36];
#pragma unroll
  for (int q = 0; q < 36; q++) acc[q] = 0.0;
  for (int q = threadIdx.x; q < NT * nj; q += blockDim.x) {
    const int t = q / nj, j = jl + (q - t * nj);
    const int k = t + j * NT - g.kmin;
    if (!(t > imin && t < imax) || k < 0 || k >= N) continue;
    double dh[8][3];
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const WvSrc &P = S[2 * i], &M = S[2 * i + 1];
      dh[i][0] = dh[i][1] = dh[i][2] = 0.0;
      if (P.c > 0 && j >= P.jlo && j < P.jlo + P.c) {
        const double *cp = coef + (16 * (size_t)s + 2 * i) * 3 * LNT + t * P.c + (j - P.jlo);
        double m0 = 0.0, m1 = 0.0, m2 = 0.0;
        if (M.c > 0 && j >= M.jlo && j < M.jlo + M.c) {
          const double *cm = coef + (16 * (size_t)s + 2 * i + 1) * 3 * LNT + t * M.c + (j - M.jlo);
          m0 = cm[0];
          m1 = cm[LNT];
          m2 = cm[2 * LNT];
        }
        dh[i][0] = (cp[0] - m0) * inv;
        dh[i][1] = (cp[LNT] - m1) * inv;
        dh[i][2] = (cp[2 * LNT] - m2) * inv;
      }
    }
    double c[9];
#pragma unroll
    for (int ab = 0; ab < 9; ab++) c[ab] = g.invC[(size_t)ab * N + k];
    int idx = 0;
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
      for (int jj = i; jj < 8; jj++, idx++) {
        double v = 0.0;
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
          for (int b = 0; b < 3; b++) v += dh[i][a] * dh[jj][b] * c[3 * a + b];
        acc[idx] += v;
      }
  }
  // CTA reduction of the 36 sums
#pragma unroll
  for (int q = 0; q < 36; q++)
    for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
  if ((threadIdx.x & 31) == 0)
    for (int q = 0; q < 36; q++) red[threadIdx.x >> 5][q] = acc[q];
  __syncthreads();
  if (threadIdx.x < 36) {
    double v = 0.0;
    for (int w = 0; w < kFisherThreads / 32; w++) v += red[w][threadIdx.x];
    if (v != v) v = 10.0;  // the reference's sentinel for a NaN element
    int i = 0, r = threadIdx.x;
    while (r >= 8 - i) {
      r -= 8 - i;
      i++;
    }
    const int jj = i + r;
    if (fisher) {
      fisher[64 * (size_t)s + 8 * i + jj] = v;
      fisher[64 * (size_t)s + 8 * jj + i] = v;
    }
  }
  if (threadIdx.x == 0 && status) status[s] = 0;
}

// Launches a tile kernel with C = 16, 4 or 1 items per CTA of 128 threads,
// the largest whose shared memory (C x per bytes) fits 200 KB.
template <typename K16, typename K4, typename K1, typename... Args>
static cudaError_t wv_launch_tiles(K16 k16, K4 k4, K1 k1, size_t per, int items, cudaStream_t s, Args... args) {
  const size_t cap = 200 * 1024;
  cudaError_t e;
  if (16 * per <= cap) {
    if ((e = cudaFuncSetAttribute(k16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(16 * per))) != cudaSuccess)
      return e;
    k16<<<(items + 15) / 16, 128, 16 * per, s>>>(args...);
  } else if (4 * per <= cap) {
    if ((e = cudaFuncSetAttribute(k4, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(4 * per))) != cudaSuccess)
      return e;
    k4<<<(items + 3) / 4, 128, 4 * per, s>>>(args...);
  } else {
    if ((e = cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)per)) != cudaSuccess) return e;
    k1<<<items, 128, per, s>>>(args...);
  }
  return cudaGetLastError();
}

cudaError_t wv_waveform_launch(const WvGridDev &g, const WvWorkDev &w, int precision, int n, const double *params,
                               int *status, cudaStream_t s, int *nlaunch) {
  if (n <= 0) return cudaSuccess;
  const int norb = g.norb;
  cudaError_t e;
  {
    // 4 norb doubles of shared memory per source; 16 sources per CTA where
    // they fit, fewer for long observations
    const size_t per = sizeof(double) * (4 * (size_t)norb + 1);
    if ((e = wv_launch_tiles(wv_plan_kernel<16>, wv_plan_kernel<4>, wv_plan_kernel<1>, per, n, s, g, n, params, w.src,
                             w.ssb, status)) != cudaSuccess)
      return e;
  }
  const long long nr = (long long)n * norb;
  wv_resp_kernel<<<(unsigned)((nr + 127) / 128), 128, 0, s>>>(g, n, w.src, w.ssb, w.resp);
  {
    const size_t per = sizeof(double) * (4 * (size_t)norb + 1);
    if ((e = wv_launch_tiles(wv_tdi_kernel<16>, wv_tdi_kernel<4>, wv_tdi_kernel<1>, per, 3 * n, s, g, n, w.src, w.resp,
                             w.tdi)) != cudaSuccess)
      return e;
  }
  if (precision == 1) {
    // float2 samples and layer buffer; the interval table shares the layer
    // buffer's place and may be larger than it
    const size_t sm = sizeof(float2) * (size_t)g.NT * (kWvMaxLayers + 1) / 2 +
                      std::max(sizeof(float2) * (size_t)g.NT, sizeof(WvMixInterval) * (size_t)norb + 16);
    e = cudaFuncSetAttribute(wv_layers_mix_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    wv_layers_mix_kernel<<<3 * n, kLayerThreads, sm, s>>>(g, n, w.src, w.ssb, w.tdi, reinterpret_cast<float *>(w.coef));
  } else {
    const size_t sm = layers_smem(g.NT);
    e = cudaFuncSetAttribute(wv_layers_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    wv_layers_kernel<<<3 * n, kLayerThreads, sm, s>>>(g, n, w.src, w.ssb, w.tdi, w.coef, nullptr, nullptr);
  }
  if (nlaunch) *nlaunch += 4;
  return cudaGetLastError();
}

cudaError_t wv_fisher_launch(const WvGridDev &g, const WvWorkDev &w, int n, const double *params, double *pp,
                             int imin, int imax, double *fisher, int *status, cudaStream_t s, int *nlaunch) {
  if (n <= 0) return cudaSuccess;
  if (16 * n > w.cap) return cudaErrorInvalidValue;
  wv_fisher_params_kernel<<<(16 * n + 127) / 128, 128, 0, s>>>(n, params, pp);
  cudaError_t e = wv_waveform_launch(g, w, 0, 16 * n, pp, nullptr, s, nlaunch);
  if (e != cudaSuccess) return e;
  wv_fisher_kernel<<<n, kFisherThreads, 0, s>>>(g, n, w.src, w.coef, imin, imax, fisher, status);
  if (nlaunch) *nlaunch += 2;
  return cudaGetLastError();
}

cudaError_t wv_dlogl_launch(const WvGridDev &g, const WvWorkDev &w, int precision, int n, const double *term_x,
                            double *dlogl, double *term_y, double *hh, int *status, cudaStream_t s, int *nlaunch,
                            double tol) {
  if (n <= 0) return cudaSuccess;
  if (precision == 1) {
    const double kest = tol > 0.0 ? kWvMixedErrK / tol : 0.0;
    cudaError_t e;
    if (kest > 0.0 && (e = cudaMemsetAsync(w.count, 0, sizeof(int), s)) != cudaSuccess) return e;
    wv_dlogl_mix_kernel<<<n, kDloglThreads, 0, s>>>(g, n, w.src, reinterpret_cast<const float *>(w.coef), term_x,
                                                    dlogl, term_y, hh, status, kest, w.count, w.list, w.total);
    if (nlaunch) *nlaunch += 1;
    if (kest > 0.0) {
      // the listed sources again in FP64: their layers (over the mixed
      // coefficients, which are no longer read) and their likelihood; the
      // grids cover every source and the CTAs past the list return at once
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      const size_t sm = layers_smem(g.NT);
      if ((e = cudaFuncSetAttribute(wv_layers_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) !=
          cudaSuccess)
        return e;
      wv_layers_kernel<<<3 * n, kLayerThreads, sm, s>>>(g, n, w.src, w.ssb, w.tdi, w.coef, w.count, w.list);
      wv_dlogl_kernel<<<n, kDloglThreads, 0, s>>>(g, n, w.src, w.coef, term_x, dlogl, term_y, hh, status, w.count,
                                                  w.list);
      if (nlaunch) *nlaunch += 2;
    }
  } else {
    wv_dlogl_kernel<<<n, kDloglThreads, 0, s>>>(g, n, w.src, w.coef, term_x, dlogl, term_y, hh, status, nullptr,
                                                nullptr);
    if (nlaunch) *nlaunch += 1;
  }
  return cudaGetLastError();
}

cudaError_t wv_export(const WvGridDev &g, const WvWorkDev &w, int precision, int n, int *info, double *xyz,
                      cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (info) wv_info_kernel<<<(n + 127) / 128, 128, 0, s>>>(n, w.src, info);
  if (xyz) {
    const long long cnt = (long long)n * 3 * kWvMaxLayers * g.NT;
    if (precision == 1) {
      wv_unscale_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(reinterpret_cast<const float *>(w.coef), xyz,
                                                                      cnt, g.scale);
    } else {
      cudaError_t e = cudaMemcpyAsync(xyz, w.coef, sizeof(double) * cnt, cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return e;
    }
  }
  return cudaGetLastError();
}

void wv_mixed_data(int N, int NT, const double *rX, const double *rY, const double *rZ, const double *invC,
                   double *scale, std::vector<float> &res_hi, std::vector<float> &res_lo, std::vector<float> &invC32,
                   std::vector<double> &qpix) {
  (void)NT;
  // noise scale: root mean square of the X-channel standard deviation
  double m = 0.0;
  for (int k = 0; k < N; k++) m += invC[k] > 0.0 ? 1.0 / invC[k] : 0.0;
  const double s = m > 0.0 ? sqrt(m / N) : 1.0;
  *scale = s;
  const double *r[3] = {rX, rY, rZ};
  res_hi.resize(3 * (size_t)N);
  res_lo.resize(3 * (size_t)N);
  invC32.resize(9 * (size_t)N);
  for (int c = 0; c < 3; c++)
    for (int k = 0; k < N; k++) {
      const double v = r[c][k] / s;
      const float hi = (float)v;
      res_hi[(size_t)c * N + k] = hi;
      res_lo[(size_t)c * N + k] = (float)(v - (double)hi);
    }
  for (size_t q = 0; q < 9 * (size_t)N; q++) invC32[q] = (float)(invC[q] * s * s);
  qpix.assign((size_t)N, 0.0);
  for (int k = 0; k < N; k++) {
    double acc = 0.0;
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) acc += (r[a][k] / s) * (r[b][k] / s) * (invC[(size_t)(3 * a + b) * N + k] * s * s);
    qpix[k] = acc;
  }
}

}  // namespace glass
