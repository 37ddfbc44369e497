// Noise-model likelihood of XYZ frequency-domain data for sm_103a: the noise
// module's instrument covariance (noise/src/glass_noise_model.c:389-546),
// optionally plus the galactic foreground (:612-654, added as
// generate_full_covariance_matrix does, :894-907), the 3x3 inverse and
// log-determinant (utils/src/glass_math.c:240-289) and my_noise_log_likelihood
// (noise/src/glass_noise_model.c:1243-1273), for a batch of noise models.
//
// The reference regenerates the whole covariance, inverts it and sums the
// likelihood for every proposed noise model (noise_instrument_model_mcmc and
// noise_foreground_model_mcmc, noise/src/glass_noise_sampler.c:395-752), ten
// proposals per chain per sweep.  Everything that depends on frequency alone
// (the TDI and arm transfer functions, f^(-7/3), the data's auto- and
// cross-spectra) is tabulated once per bin when the data are set; a batch then
// costs one pass over the table per model: per bin the link levels enter
// linearly, the foreground takes its exp/pow/tanh, and the inverse and
// log-determinant follow the reference's Cholesky-like elimination.
//
// FP64, compiled without multiply-add contraction.  The inverse's entries are
// the cofactors times 1/det instead of the reference's
// exp(log|cofactor| - log det) (the same numbers to a few ulp).

#include "../../include/glass_gb300.h"
#include "glass_common.cuh"
#include "noise.cuh"

namespace glass {

namespace {

constexpr int kNoiseThreads = 256;
constexpr int kNoiseBinsPerThread = 8;
constexpr int kNoiseChunk = kNoiseThreads * kNoiseBinsPerThread;  // bins per CTA

struct NoiseArgs {
  int N, nchunks, nprop;
  const double *tab;  // kNoiseTabRows rows of N
  const double *inst;  // [nprop][12]
  const double *sgal;  // [nprop][5] or null
  double *partial;     // [nprop][nchunks]
};

__device__ __forceinline__ double block_sum(double v, double *red) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kNoiseThreads / 32; w++) s += red[w];
  return s;
}

// One CTA per (bin chunk, model): per-bin covariance, inverse, likelihood
// terms; the chunk's sum goes to partial[model][chunk].
__global__ void __launch_bounds__(kNoiseThreads) noise_logl_kernel(NoiseArgs a) {
  __shared__ double red[kNoiseThreads / 32];
  const int chunk = blockIdx.x, p = blockIdx.y;
  const double *in = a.inst + 12 * (size_t)p;
  const double s12 = in[0], s21 = in[1], s23 = in[2], s32 = in[3], s13 = in[4], s31 = in[5];
  const double o12 = in[6], o21 = in[7], o23 = in[8], o32 = in[9], o13 = in[10], o31 = in[11];
  const bool gal = a.sgal != nullptr;
  double Amp = 0, f1 = 0, alpha = 0, fk = 0, f2 = 0;
  if (gal) {  // map_array_to_foreground_params (noise/src/glass_noise_model.c:67-74)
    const double *sg = a.sgal + 5 * (size_t)p;
    Amp = exp(sg[0]);
    f1 = exp(sg[1]);
    alpha = sg[2];
    fk = exp(sg[3]);
    f2 = exp(sg[4]);
  }
  const int N = a.N;
  const double *F = a.tab + (size_t)kTabF * N, *COSX = a.tab + (size_t)kTabCosx * N;
  const double *TDI = a.tab + (size_t)kTabTdi * N, *ACC = a.tab + (size_t)kTabAcc * N;
  const double *OMS = a.tab + (size_t)kTabOms * N, *TG = a.tab + (size_t)kTabTgal * N;
  const double *P73 = a.tab + (size_t)kTabFp73 * N;
  const double *XX = a.tab + (size_t)kTabXX * N, *YY = a.tab + (size_t)kTabYY * N;
  const double *ZZ = a.tab + (size_t)kTabZZ * N, *XY = a.tab + (size_t)kTabXY * N;
  const double *XZ = a.tab + (size_t)kTabXZ * N, *YZ = a.tab + (size_t)kTabYZ * N;
  double acc = 0.0;
#pragma unroll 1
  for (int r = 0; r < kNoiseBinsPerThread; r++) {
    const int n = chunk * kNoiseChunk + r * kNoiseThreads + threadIdx.x;
    if (n >= N) break;
    const double f = F[n];
    double cxx = 0.0, cyy = 0.0, czz = 0.0, cxy = 0.0, cxz = 0.0, cyz = 0.0;
    if (f != 0.0) {
      const double cosx = COSX[n], tdi = TDI[n], acc_tf = ACC[n], oms_tf = OMS[n];
      // acc_tf is 0 at f >= 10 mHz, where the reference leaves out the
      // acceleration terms: adding exact zeros changes nothing
      const double A12 = s12 * acc_tf, A21 = s21 * acc_tf, A23 = s23 * acc_tf;
      const double A32 = s32 * acc_tf, A13 = s13 * acc_tf, A31 = s31 * acc_tf;
      const double O12 = o12 * oms_tf, O21 = o21 * oms_tf, O23 = o23 * oms_tf;
      const double O32 = o32 * oms_tf, O13 = o13 * oms_tf, O31 = o31 * oms_tf;
      double c00 = (O12 + O21 + O13 + O31) * .25;
      double c11 = (O23 + O32 + O21 + O12) * .25;
      double c22 = (O31 + O13 + O32 + O23) * .25;
      double c01 = (O12 + O21) * .5;
      double c02 = (O13 + O31) * .5;
      double c12 = (O32 + O23) * .5;
      c00 += ((A12 + A13) + ((A21 + A31)) * cosx * cosx);
      c11 += ((A23 + A21) + ((A32 + A12)) * cosx * cosx);
      c22 += ((A31 + A32) + ((A13 + A23)) * cosx * cosx);
      c01 += 2. * (A12 + A21);
      c02 += 2. * (A13 + A31);
      c12 += 2. * (A32 + A23);
      c00 *= -2. * tdi;
      c11 *= -2. * tdi;
      c22 *= -2. * tdi;
      c01 *= tdi * cosx;
      c02 *= tdi * cosx;
      c12 *= tdi * cosx;
      cxx = c00 / 4.0;
      cyy = c11 / 4.0;
      czz = c22 / 4.0;
      cxy = c01 / 4.0;
      cxz = c02 / 4.0;
      cyz = c12 / 4.0;
      if (gal) {
        // utils/src/glass_galaxy.c:40-44, skipped above 10 f1 as the reference does
        const double t = TG[n];
        const double Sgal =
            (f > f1 * 10) ? 0.0 : Amp * P73[n] * exp(-pow(f / f1, alpha)) * 0.5 * (1. + tanh((fk - f) / f2));
        const double d = t * Sgal / 4.0, o = -0.5 * t * Sgal / 4.0;
        cxx += d;
        cyy += d;
        czz += d;
        cxy += o;
        cxz += o;
        cyz += o;
      }
    }
    const double d1 = cxx;
    const double d2 = cyy - cxy * cxy / d1;
    const double tt = cyz - cxy * cxz / d1;
    const double d3 = (czz - cxz * cxz / d1) - (tt * tt) / d2;
    const double logdetC = log(d1) + log(d2) + log(d3);
    const double idet = 1.0 / (d1 * d2 * d3);
    const double ixx = (cyy * czz - cyz * cyz) * idet;
    const double iyy = (czz * cxx - cxz * cxz) * idet;
    const double izz = (cxx * cyy - cxy * cxy) * idet;
    const double ixy = (cxz * cyz - czz * cxy) * idet;
    const double ixz = (cxy * cyz - cxz * cyy) * idet;
    const double iyz = (cxy * cxz - cxx * cyz) * idet;
    double l = 0.0;
    l -= 0.5 * XX[n] * ixx * 2;
    l -= 0.5 * YY[n] * iyy * 2;
    l -= 0.5 * ZZ[n] * izz * 2;
    l -= XY[n] * ixy * 2;
    l -= XZ[n] * ixz * 2;
    l -= YZ[n] * iyz * 2;
    l -= logdetC;
    acc += l;
  }
  const double s = block_sum(acc, red);
  if (threadIdx.x == 0) a.partial[(size_t)p * a.nchunks + chunk] = s;
}

// Per model: the chunks' sums in order, and the constant -3 N log(2 pi).
__global__ void noise_finish_kernel(const double *partial, int nchunks, int nprop, double cst, double *logl) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nprop) return;
  double s = 0.0;
  for (int c = 0; c < nchunks; c++) s += partial[(size_t)p * nchunks + c];
  logl[p] = s - cst;
}

}  // namespace

// ------------------------------------------------------------------- host
// The per-bin table, with the reference's own expressions (host libm): the
// grid f_n = fmin + n/T (noise/src/glass_noise_model.c:1384-1385), the
// transfer functions of :415-446 and :620-624, and the data's auto- and
// cross-spectra of :1251-1263.
void noise_build_table(double T, double fmin, int N, const double *X, const double *Y, const double *Z,
                       double *tab) {
  const double fstar = kCLIGHT / (2.0 * M_PI * kLARM);
  const double acc_units = 2.81837551648e-19;  // 1/(2 pi c)^2
  const double oms_units = 4.39256635604e-16;  // (2 pi / c)^2
  const double acc_fmax = 0.01;
  for (int n = 0; n < N; n++) {
    const double f = fmin + (double)n / T;
    double *col[kNoiseTabRows];
    for (int r = 0; r < kNoiseTabRows; r++) col[r] = tab + (size_t)r * N + n;
    *col[kTabF] = f;
    if (f != 0.0) {
      const double x = f / fstar, f2 = f * f;
      const double sx = sin(x);
      *col[kTabCosx] = cos(x);
      *col[kTabTdi] = -8.0 * (sx * sx);
      *col[kTabAcc] = (f < acc_fmax) ? acc_units / f2 * (1.0 + pow(0.4e-3 / f, 2)) * (1.0 + pow(f / 8.0e-3, 4)) : 0.0;
      *col[kTabOms] = oms_units * f2 * (1.0 + pow(2.0e-3 / f, 4));
      const double xg = f / (kCLIGHT / (kPI2 * kLARM));
      *col[kTabTgal] = 4. * xg * xg * sin(xg) * sin(xg);
      *col[kTabFp73] = pow(f, -7. / 3.);
    } else {
      *col[kTabCosx] = *col[kTabTdi] = *col[kTabAcc] = *col[kTabOms] = *col[kTabTgal] = *col[kTabFp73] = 0.0;
    }
    const double rex = X[2 * n], imx = X[2 * n + 1];
    const double rey = Y[2 * n], imy = Y[2 * n + 1];
    const double rez = Z[2 * n], imz = Z[2 * n + 1];
    *col[kTabXX] = rex * rex + imx * imx;
    *col[kTabYY] = rey * rey + imy * imy;
    *col[kTabZZ] = rez * rez + imz * imz;
    *col[kTabXY] = rex * rey + imx * imy;
    *col[kTabXZ] = rex * rez + imx * imz;
    *col[kTabYZ] = rey * rez + imy * imz;
  }
}

int noise_chunks(int N) { return (N + kNoiseChunk - 1) / kNoiseChunk; }

cudaError_t noise_logl_launch(const NoiseDev &nd, int nprop, const double *inst, const double *sgal, double *logl,
                              cudaStream_t stream, int *nlaunch) {
  NoiseArgs a;
  a.N = nd.N;
  a.nchunks = noise_chunks(nd.N);
  a.nprop = nprop;
  a.tab = nd.tab;
  a.inst = inst;
  a.sgal = sgal;
  a.partial = nd.partial;
  int launches = 0;
  // models in slices of at most 65535 (the grid's y extent)
  for (int p0 = 0; p0 < nprop; p0 += 65535) {
    const int np = nprop - p0 < 65535 ? nprop - p0 : 65535;
    NoiseArgs s = a;
    s.nprop = np;
    s.inst = inst + 12 * (size_t)p0;
    s.sgal = sgal ? sgal + 5 * (size_t)p0 : nullptr;
    s.partial = nd.partial + (size_t)p0 * a.nchunks;
    noise_logl_kernel<<<dim3(a.nchunks, np), kNoiseThreads, 0, stream>>>(s);
    launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  const double cst = 3 * nd.N * log(2 * M_PI);
  noise_finish_kernel<<<(nprop + 255) / 256, 256, 0, stream>>>(nd.partial, a.nchunks, nprop, cst, logl);
  launches++;
  if (nlaunch) *nlaunch = launches;
  return cudaGetLastError();
}

}  // namespace glass
