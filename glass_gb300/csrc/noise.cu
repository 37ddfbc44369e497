// Noise-model likelihood of XYZ frequency-domain data for sm_103a: the noise
// module's instrument covariance (noise/src/glass_noise_model.c:389-546),
// optionally plus the galactic foreground (:612-654, added as
// generate_full_covariance_matrix does, :894-907), the 3x3 inverse and
// log-determinant (utils/src/glass_math.c:240-289) and my_noise_log_likelihood
// (noise/src/glass_noise_model.c:1243-1273), for a batch of noise models,
// optionally with a stochastic background (SGWB) of one of the reference's
// three spectral templates times the instrument's response
// (generate_sgwb_model, :778-842; the wavelet form :843-892).
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

#include <math.h>

#include <vector>

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
  int sg_type;         // SGWB template
  const double *sgwb;  // [nprop][4] or null
  const double *rsg;   // SGWB response, 6 rows of N
  double *partial;     // [nprop][nchunks]
};

// Instrument covariance of one bin at link levels in[12] (sacc[6], soms[6]),
// from the bin's cos(f/f*), -8 sin^2(f/f*) and transfer functions
// (noise/src/glass_noise_model.c:445-546; acc_tf is 0 at f >= 10 mHz, where the
// reference leaves out the acceleration terms: adding exact zeros changes
// nothing), normalised by 4.
__device__ __forceinline__ void noise_inst_cov(double cosx, double tdi, double acc_tf, double oms_tf,
                                               const double *in, double &cxx, double &cyy, double &czz, double &cxy,
                                               double &cxz, double &cyz) {
  const double A12 = in[0] * acc_tf, A21 = in[1] * acc_tf, A23 = in[2] * acc_tf;
  const double A32 = in[3] * acc_tf, A13 = in[4] * acc_tf, A31 = in[5] * acc_tf;
  const double O12 = in[6] * oms_tf, O21 = in[7] * oms_tf, O23 = in[8] * oms_tf;
  const double O32 = in[9] * oms_tf, O13 = in[10] * oms_tf, O31 = in[11] * oms_tf;
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
}

// The galactic foreground's PSD at f (utils/src/glass_galaxy.c:40-44), zero
// above 10 f1 as in noise/src/glass_noise_model.c:627-631; fp73 = f^(-7/3).
__device__ __forceinline__ double noise_sgal(double f, double fp73, double Amp, double f1, double alpha, double fk,
                                             double f2) {
  return (f > f1 * 10) ? 0.0 : Amp * fp73 * exp(-pow(f / f1, alpha)) * 0.5 * (1. + tanh((fk - f) / f2));
}

// ------------------------------------------------------------------ SGWB
// Cosmological constants of the templates (utils/src/glass_constants.h:81-86):
// H0 = 70 km/s/Mpc in 1/s, the f^-3 prefactor 3 H0^2 / (4 pi^2) that turns
// an energy-density spectrum into a strain PSD, and the radiation-era
// transfer factor of the lognormal template.
constexpr double kSgH0 = 70 * 3.24078e-20;
constexpr double kSgHscale = 3 * kSgH0 * kSgH0 / (4 * M_PI * M_PI);
constexpr double kSgCgOr0 = 1.6e-5 / (0.7 * 0.7);

// erfc by Abramowitz & Stegun 7.1.26 (|error| < 1.5e-7), the rational
// approximation the reference's glass_erfc uses (utils/src/glass_math.c:1310),
// evaluated on |x| and reflected (erfc(-x) = 2 - erfc(x)).
__device__ __forceinline__ double sgwb_erfc(double x) {
  const double ax = fabs(x);
  const double t = 1.0 / (1.0 + 0.3275911 * ax);
  const double poly = ((((1.061405429 * t - 1.453152027) * t + 1.421413741) * t - 0.284496736) * t + 0.254829592) * t;
  const double y = poly * exp(-ax * ax);
  return x < 0.0 ? 2.0 - y : y;
}

// The background's strain PSD at f > 0 (noise/src/glass_noise_model.c:725-776):
//  powerlaw          p = log10 A, alpha: A (f / 25 Hz)^alpha
//  lognormal         p = log10 A, log10 f*, log10 Delta: the wide-Delta
//                    lognormal-peak spectrum of Pi & Sasaki (JCAP 2020,
//                    eq. 3.29), its asymptote 0.783e-3 A^2 for Delta >= 9
//  phase transition  p = rb, b, log10 Ap, log10 fp: Ap times the broken power
//                    law in s = f / fp with slopes 9 and b
// each times Hscale / f^3.
__device__ double sgwb_psd(int type, double f, const double *p) {
  const double pre = kSgHscale / (f * f * f);
  if (type == kSgwbPowerlaw) {
    const double A = pow(10.0, p[0]);
    return pre * A * pow(f / 25.0, p[1]);
  }
  if (type == kSgwbLognormal) {
    const double A = pow(10.0, p[0]), fst = pow(10.0, p[1]), D = pow(10.0, p[2]);
    const double scale = pre * kSgCgOr0 * A * A;
    if (!(D < 9.0)) return scale * 0.783 / 1e3;
    const double ft = f / fst, lft = log(ft), D2 = D * D;
    const double rpi = sqrt(M_PI);
    const double h32 = 0.5 * log(1.5);
    const double lK = lft + 1.5 * D2;
    const double u = lK + h32;
    const double t1 = 4.0 / 5.0 / rpi * ft * ft * ft * exp(9.0 * D2 / 4.0) / D *
                      ((lK * lK + 0.5 * D2) * sgwb_erfc(u / D) - D / rpi * exp(-u * u / D2) * (lK - h32));
    const double v = lft + D2 - 0.5 * log(4.0 / 3.0);
    const double t2 = 0.0659 / D2 * ft * ft * exp(D2) * exp(-v * v / D2);
    const double t3 = (1.0 / 3.0) * sqrt(2.0) / rpi * pow(ft, -4) * exp(8.0 * D2) / D * exp(-lft * lft / (2.0 * D2)) *
                      sgwb_erfc((4.0 * D2 - lft + log(4.0)) / (D * sqrt(2.0)));
    return scale * (t1 + t2 + t3);
  }
  // phase transition
  const double rb = p[0], b = p[1], Ap = pow(10.0, p[2]), fp = pow(10.0, p[3]);
  const double rb4 = rb * rb * rb * rb;
  const double m = (9 * rb4 + b) / (rb4 + 1);
  const double sr = f / fp, s4 = sr * sr * sr * sr, s9 = s4 * s4 * sr;
  const double M = s9 * pow((1 + rb4) / (rb4 + s4), (9 - b) / 4) * pow((b + 4) / (b + 4 - m + m * sr * sr), (b + 4) / 2);
  return Ap * M * pre;
}

// Inverse and log-determinant of a symmetric 3x3 covariance by the
// reference's elimination (utils/src/glass_math.c:261-274), the entries as
// cofactor / det: iv = xx, yy, zz, xy, xz, yz.
__device__ __forceinline__ void noise_inv3(double cxx, double cyy, double czz, double cxy, double cxz, double cyz,
                                           double *iv, double &logdetC) {
  const double d1 = cxx;
  const double d2 = cyy - cxy * cxy / d1;
  const double tt = cyz - cxy * cxz / d1;
  const double d3 = (czz - cxz * cxz / d1) - (tt * tt) / d2;
  logdetC = log(d1) + log(d2) + log(d3);
  const double idet = 1.0 / (d1 * d2 * d3);
  iv[0] = (cyy * czz - cyz * cyz) * idet;
  iv[1] = (czz * cxx - cxz * cxz) * idet;
  iv[2] = (cxx * cyy - cxy * cxy) * idet;
  iv[3] = (cxz * cyz - czz * cxy) * idet;
  iv[4] = (cxy * cyz - cxz * cyy) * idet;
  iv[5] = (cxy * cxz - cxx * cyz) * idet;
}

__device__ __forceinline__ void noise_gal_params(const double *sg, double &Amp, double &f1, double &alpha,
                                                 double &fk, double &f2) {
  // map_array_to_foreground_params (noise/src/glass_noise_model.c:67-74)
  Amp = exp(sg[0]);
  f1 = exp(sg[1]);
  alpha = sg[2];
  fk = exp(sg[3]);
  f2 = exp(sg[4]);
}

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
  const bool gal = a.sgal != nullptr;
  double Amp = 0, f1 = 0, alpha = 0, fk = 0, f2 = 0;
  if (gal) noise_gal_params(a.sgal + 5 * (size_t)p, Amp, f1, alpha, fk, f2);
  const double *sgp = a.sgwb ? a.sgwb + 4 * (size_t)p : nullptr;
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
      noise_inst_cov(COSX[n], TDI[n], ACC[n], OMS[n], in, cxx, cyy, czz, cxy, cxz, cyz);
      if (gal) {
        // utils/src/glass_galaxy.c:40-44, skipped above 10 f1 as the reference does
        const double t = TG[n];
        const double Sgal = noise_sgal(f, P73[n], Amp, f1, alpha, fk, f2);
        const double d = t * Sgal / 4.0, o = -0.5 * t * Sgal / 4.0;
        cxx += d;
        cyy += d;
        czz += d;
        cxy += o;
        cxz += o;
        cyz += o;
      }
      if (sgp) {
        // added last, as the instrument sampler combines the three
        // (noise/src/glass_noise_sampler.c:559-568)
        const double S = sgwb_psd(a.sg_type, f, sgp);
        const double *R = a.rsg;
        cxx += R[n] * S;
        cyy += R[(size_t)N + n] * S;
        czz += R[2 * (size_t)N + n] * S;
        cxy += R[3 * (size_t)N + n] * S;
        cxz += R[4 * (size_t)N + n] * S;
        cyz += R[5 * (size_t)N + n] * S;
      }
    }
    double iv[6], logdetC;
    noise_inv3(cxx, cyy, czz, cxy, cxz, cyz, iv, logdetC);
    double l = 0.0;
    l -= 0.5 * XX[n] * iv[0] * 2;
    l -= 0.5 * YY[n] * iv[1] * 2;
    l -= 0.5 * ZZ[n] * iv[2] * 2;
    l -= XY[n] * iv[3] * 2;
    l -= XZ[n] * iv[4] * 2;
    l -= YZ[n] * iv[5] * 2;
    l -= logdetC;
    acc += l;
  }
  const double s = block_sum(acc, red);
  if (threadIdx.x == 0) a.partial[(size_t)p * a.nchunks + chunk] = s;
}

// The one- and two-channel forms: the instrument covariance of
// generate_instrument_noise_model's case 1 (Michelson X, XYZnoise_FF) and
// case 2 (A and E, AEnoise_FF; utils/src/glass_lisa.c:1121-1145) on the link
// levels sacc12 = in[0], soms12 = in[6] (noise/src/glass_noise_model.c:450-461),
// normalised by 4, plus the foreground's case 1 (Sgal / 4) or case 2
// (1.5 t Sgal / 4, :635-641), the diagonal inverse and log-determinant
// (utils/src/glass_math.c:248-258) and noise_log_likelihood's sum
// (noise/src/glass_noise_model.c:1104-1134).  sin^2(f/f*) is the table's
// -8 sin^2 times -1/8 (exact).
__global__ void __launch_bounds__(kNoiseThreads) noise_ch12_kernel(NoiseArgs a, int nch) {
  __shared__ double red[kNoiseThreads / 32];
  const int chunk = blockIdx.x, p = blockIdx.y;
  const double *in = a.inst + 12 * (size_t)p;
  const bool gal = a.sgal != nullptr;
  double Amp = 0, f1 = 0, alpha = 0, fk = 0, f2 = 0;
  if (gal) noise_gal_params(a.sgal + 5 * (size_t)p, Amp, f1, alpha, fk, f2);
  const double sacc12 = in[0], soms12 = in[6];
  const int N = a.N;
  const double *F = a.tab + (size_t)kTabF * N, *COSX = a.tab + (size_t)kTabCosx * N;
  const double *TDI = a.tab + (size_t)kTabTdi * N, *ACC = a.tab + (size_t)kTabAcc * N;
  const double *OMS = a.tab + (size_t)kTabOms * N, *TG = a.tab + (size_t)kTabTgal * N;
  const double *P73 = a.tab + (size_t)kTabFp73 * N, *C2X = a.tab + (size_t)kTabCos2x * N;
  const double *P0 = a.tab + (size_t)kTabP0 * N, *P1 = a.tab + (size_t)kTabP1 * N;
  double acc = 0.0;
#pragma unroll 1
  for (int r = 0; r < kNoiseBinsPerThread; r++) {
    const int n = chunk * kNoiseChunk + r * kNoiseThreads + threadIdx.x;
    if (n >= N) break;
    const double f = F[n];
    double c = 0.0;
    if (f != 0.0) {
      const double cosx = COSX[n], sx2 = TDI[n] * -0.125;
      const double Spm = sacc12 * ACC[n], Sop = soms12 * OMS[n];
      c = (nch == 1) ? 16. * sx2 * (2. * (1.0 + cosx * cosx) * Spm + Sop)
                     : 8. * sx2 * (2. * Spm * (3. + 2. * cosx + C2X[n]) + Sop * (2. + cosx));
      c = c / 4.0;
      if (gal) {
        const double Sgal = noise_sgal(f, P73[n], Amp, f1, alpha, fk, f2);
        c += (nch == 1 ? Sgal : 1.5 * TG[n] * Sgal) / 4.0;
      }
    }
    const double ic = 1. / c;
    double l = -0.5 * (2.0 * (P0[n] * ic));
    double ld = log(c);
    if (nch == 2) {
      l -= 0.5 * (2.0 * (P1[n] * ic));
      ld += log(c);
    }
    acc += l - ld;
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


// ------------------------------------------------------- wavelet domain
struct NoiseWvArgs {
  int Nlayer, Ncoarse, Q, LJ, nchunks, mode;
  double inv_ND;
  const double *tab, *P, *mod;
  const double *inst, *sgal;
  int sg_type;
  const double *sgwb, *rsg;  // [nprop][4] or null; 6 rows of Nlayer
  double *out;  // logl (modes 0/1) or partial (mode 2)
};

// The background's variance in layer j (generate_sgwb_model_wavelet
// :843-892: the Fourier model at the layer centre over ND, zero in the DC
// layer): sg6 = xx, yy, zz, xy, xz, yz.
__device__ __forceinline__ void noise_wv_sgwb(const NoiseWvArgs &a, int j, const double *sgp, double *sg6) {
  const int NL = a.Nlayer;
  const double f = a.tab[(size_t)kTabF * NL + j];
  const double S = f != 0.0 ? sgwb_psd(a.sg_type, f, sgp) : 0.0;
#pragma unroll
  for (int e = 0; e < 6; e++) sg6[e] = f != 0.0 ? a.rsg[(size_t)e * NL + j] * S * a.inv_ND : 0.0;
}

// Instrument (and foreground) variance of one layer in the wavelet domain:
// the Fourier model at the layer centre over ND (generate_instrument_noise_
// model_wavelet :561-610, generate_galactic_foreground_model_wavelet :656-722,
// whose off-diagonals have the isotropic -1/2 undone).  inst6, conf6: xx, yy,
// zz, xy, xz, yz.
__device__ __forceinline__ void noise_wv_layer(const NoiseWvArgs &a, int j, const double *in, bool gal, double Amp,
                                               double f1, double alpha, double fk, double f2, double *inst6,
                                               double *conf6) {
  const int NL = a.Nlayer;
  const double f = a.tab[(size_t)kTabF * NL + j];
  double cxx = 0, cyy = 0, czz = 0, cxy = 0, cxz = 0, cyz = 0;
  if (f != 0.0)
    noise_inst_cov(a.tab[(size_t)kTabCosx * NL + j], a.tab[(size_t)kTabTdi * NL + j], a.tab[(size_t)kTabAcc * NL + j],
                   a.tab[(size_t)kTabOms * NL + j], in, cxx, cyy, czz, cxy, cxz, cyz);
  inst6[0] = cxx * a.inv_ND;
  inst6[1] = cyy * a.inv_ND;
  inst6[2] = czz * a.inv_ND;
  inst6[3] = cxy * a.inv_ND;
  inst6[4] = cxz * a.inv_ND;
  inst6[5] = cyz * a.inv_ND;
  double dg = 0.0, og = 0.0;
  if (gal && f != 0.0) {
    const double t = a.tab[(size_t)kTabTgal * NL + j];
    const double Sgal = noise_sgal(f, a.tab[(size_t)kTabFp73 * NL + j], Amp, f1, alpha, fk, f2);
    dg = t * Sgal / 4.0;
    og = -0.5 * t * Sgal / 4.0;
    og *= -2.0;
  }
  conf6[0] = conf6[1] = conf6[2] = dg * a.inv_ND;
  conf6[3] = conf6[4] = conf6[5] = og * a.inv_ND;
}

// Modes 0/1: the covariance is the same for every cell of a layer, so a
// layer's cells contribute -Q/2 (ixx Sxx + ... + 2 ixy Sxy ...) - Q/2 Ncoarse
// log det with S the layer's sums of the cell statistics.  One CTA per model.
__global__ void __launch_bounds__(kNoiseThreads) noise_wv_stationary_kernel(NoiseWvArgs a) {
  __shared__ double red[kNoiseThreads / 32];
  const int p = blockIdx.x;
  const double *in = a.inst + 12 * (size_t)p;
  const bool gal = a.mode == 1;
  double Amp = 0, f1 = 0, alpha = 0, fk = 0, f2 = 0;
  if (gal) noise_gal_params(a.sgal + 5 * (size_t)p, Amp, f1, alpha, fk, f2);
  const int NL = a.Nlayer;
  const double Qd = (double)a.Q;
  const double *sgp = a.sgwb ? a.sgwb + 4 * (size_t)p : nullptr;
  double acc = 0.0;
  for (int j = threadIdx.x; j < NL; j += blockDim.x) {
    double c6[6], g6[6];
    noise_wv_layer(a, j, in, gal, Amp, f1, alpha, fk, f2, c6, g6);
    if (gal) {  // generate_full_stationary_covariance_matrix_coarse (:1003-1010)
      c6[0] += g6[0];
      c6[1] += g6[1];
      c6[2] += g6[2];
      c6[3] -= g6[3] / 2.;
      c6[4] -= g6[4] / 2.;
      c6[5] -= g6[5] / 2.;
    }
    if (sgp) {  // added last (:1012-1019)
      double s6[6];
      noise_wv_sgwb(a, j, sgp, s6);
#pragma unroll
      for (int e = 0; e < 6; e++) c6[e] += s6[e];
    }
    double iv[6], ld;
    noise_inv3(c6[0], c6[1], c6[2], c6[3], c6[4], c6[5], iv, ld);
    double s = 0.0;
    s -= 0.5 * Qd * iv[0] * a.tab[(size_t)kTabXX * NL + j];
    s -= 0.5 * Qd * iv[1] * a.tab[(size_t)kTabYY * NL + j];
    s -= 0.5 * Qd * iv[2] * a.tab[(size_t)kTabZZ * NL + j];
    s -= Qd * iv[3] * a.tab[(size_t)kTabXY * NL + j];
    s -= Qd * iv[4] * a.tab[(size_t)kTabXZ * NL + j];
    s -= Qd * iv[5] * a.tab[(size_t)kTabYZ * NL + j];
    s -= 0.5 * Qd * ld * (double)a.Ncoarse;
    acc += s;
  }
  const double s = block_sum(acc, red);
  if (threadIdx.x == 0) a.out[p] = s;
}

// Mode 2: the foreground modulated per cell (generate_full_dynamic_covariance_
// matrix_coarse :923-981).  One CTA per (chunk of LJ layers, model); the
// chunk's layer covariances go to shared memory, then every cell is inverted
// and summed with its statistics (my_noise_log_likelihood_wavelet_coarse
// :1211-1241).
constexpr int kNoiseWvMaxLJ = 64;
__global__ void __launch_bounds__(kNoiseThreads) noise_wv_dynamic_kernel(NoiseWvArgs a) {
  __shared__ double red[kNoiseThreads / 32];
  __shared__ double lay[kNoiseWvMaxLJ][18];
  const int chunk = blockIdx.x, p = blockIdx.y;
  const double *in = a.inst + 12 * (size_t)p;
  double Amp, f1, alpha, fk, f2;
  noise_gal_params(a.sgal + 5 * (size_t)p, Amp, f1, alpha, fk, f2);
  const double *sgp = a.sgwb ? a.sgwb + 4 * (size_t)p : nullptr;
  const int j0 = chunk * a.LJ;
  const int nl = min(a.LJ, a.Nlayer - j0);
  for (int t = threadIdx.x; t < nl; t += blockDim.x) {
    noise_wv_layer(a, j0 + t, in, true, Amp, f1, alpha, fk, f2, &lay[t][0], &lay[t][6]);
    if (sgp)
      noise_wv_sgwb(a, j0 + t, sgp, &lay[t][12]);
    else
      for (int e = 12; e < 18; e++) lay[t][e] = 0.0;
  }
  __syncthreads();
  const int Nc = a.Ncoarse;
  const size_t Npix = (size_t)a.Nlayer * Nc;
  const double Qd = (double)a.Q;
  double acc = 0.0;
  for (int idx = threadIdx.x; idx < nl * Nc; idx += blockDim.x) {
    const int jj = idx / Nc, q = idx - jj * Nc;
    double c6[6];
#pragma unroll
    for (int e = 0; e < 6; e++) c6[e] = lay[jj][e] + lay[jj][6 + e] * a.mod[(size_t)e * Nc + q];
    if (sgp) {  // the stationary background last (:964-971)
#pragma unroll
      for (int e = 0; e < 6; e++) c6[e] += lay[jj][12 + e];
    }
    double iv[6], ld;
    noise_inv3(c6[0], c6[1], c6[2], c6[3], c6[4], c6[5], iv, ld);
    const size_t k = (size_t)(j0 + jj) * Nc + q;
    double s = 0.0;
    s -= 0.5 * Qd * iv[0] * a.P[k];
    s -= 0.5 * Qd * iv[1] * a.P[Npix + k];
    s -= 0.5 * Qd * iv[2] * a.P[2 * Npix + k];
    s -= Qd * iv[3] * a.P[3 * Npix + k];
    s -= Qd * iv[4] * a.P[4 * Npix + k];
    s -= Qd * iv[5] * a.P[5 * Npix + k];
    s -= 0.5 * Qd * ld;
    acc += s;
  }
  const double s = block_sum(acc, red);
  if (threadIdx.x == 0) a.out[(size_t)p * a.nchunks + chunk] = s;
}

__global__ void noise_wv_const_kernel(double *logl, int nprop, double cst) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < nprop) logl[p] -= cst;
}

// ------------------------------------------------ spline noise model
// One CTA per model (noise_spline_model_mcmc / _rjmcmc,
// noise/src/glass_noise_sampler.c:133, :232): one thread per channel solves
// the natural cubic spline through the model's control points
// (spline_coefficients, utils/src/glass_math.c:98-178: the tridiagonal
// system's forward elimination and back substitution, sequential), then all
// threads evaluate it over the bins with the binary-search lookup (the largest
// knot <= f: binary_search, :443-473, on distinct knots), add the transfer
// floor (generate_spline_noise_model, noise/src/glass_noise_model.c:366-387),
// and sum noise_log_likelihood's terms (:1104-1134): -|d|^2 / C per channel
// and -log C.
struct SplineNoiseArgs {
  int nch, N, kmax;
  const double *tab;  // f, transfer, P0[, P1]
  const int *nknots;
  const double *knot_f, *knot_C;
  double *logl;
};

__device__ __forceinline__ int spline_knot_below(int K, const double *x, double v) {
  if (v <= x[0]) return 0;
  if (v >= x[K - 1]) return K - 1;
  int lo = 0, hi = K - 1;  // x[lo] <= v < x[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (x[mid] <= v)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(kNoiseThreads) spline_noise_kernel(SplineNoiseArgs a) {
  extern __shared__ double sm[];
  __shared__ double red[kNoiseThreads / 32];
  const int p = blockIdx.x, K = a.nknots[p], KM = a.kmax;
  if (K < 2 || K > KM) {  // the whole CTA leaves before any barrier
    if (threadIdx.x == 0) a.logl[p] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  // x[KM], then per channel c0, c1, c2, c3, mu, z (each KM)
  double *x = sm;
  for (int k = threadIdx.x; k < K; k += blockDim.x) x[k] = a.knot_f[(size_t)p * KM + k];
  __syncthreads();
  if (threadIdx.x < a.nch) {
    const int c = threadIdx.x;
    double *c0 = sm + KM * (1 + 6 * c), *c1 = c0 + KM, *c2 = c1 + KM, *c3 = c2 + KM, *mu = c3 + KM, *z = mu + KM;
    const double *y = a.knot_C + ((size_t)p * a.nch + c) * KM;
    mu[0] = z[0] = 0.0;
    for (int i = 1; i < K - 1; i++) {
      const double hm = x[i] - x[i - 1], hi = x[i + 1] - x[i];
      const double al = 3.0 * ((y[i + 1] - y[i]) / hi - (y[i] - y[i - 1]) / hm);
      const double l = 2.0 * (x[i + 1] - x[i - 1]) - hm * mu[i - 1];
      mu[i] = hi / l;
      z[i] = (al - hm * z[i - 1]) / l;
    }
    c0[K - 1] = y[K - 1];
    c1[K - 1] = c2[K - 1] = c3[K - 1] = 0.0;
    for (int i = K - 2; i >= 0; i--) {
      const double h = x[i + 1] - x[i];
      c0[i] = y[i];
      c2[i] = z[i] - mu[i] * c2[i + 1];
      c1[i] = (c0[i + 1] - c0[i]) / h - h * (c2[i + 1] + 2.0 * c2[i]) / 3.0;
      c3[i] = (c2[i + 1] - c2[i]) / (3.0 * h);
    }
  }
  __syncthreads();
  const int N = a.N;
  const double *F = a.tab, *TR = a.tab + N;
  double acc = 0.0;
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    const double f = F[n];
    const int j = spline_knot_below(K, x, f);
    const double d = f - x[j];
    double ld = 0.0;
    for (int c = 0; c < a.nch; c++) {
      const double *c0 = sm + KM * (1 + 6 * c), *c1 = c0 + KM, *c2 = c1 + KM, *c3 = c2 + KM;
      const double C = (c0[j] + c1[j] * d + c2[j] * d * d + c3[j] * d * d * d) + TR[n];
      acc -= 0.5 * (2.0 * (a.tab[(size_t)(2 + c) * N + n] * (1. / C)));
      ld += log(C);
    }
    acc -= ld;
  }
  const double s = block_sum(acc, red);
  if (threadIdx.x == 0) a.logl[p] = s;
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

static void noise_freq_rows(double f, double *tab, int N, int n) {
  const double fstar = kCLIGHT / (2.0 * M_PI * kLARM);
  const double acc_units = 2.81837551648e-19;  // 1/(2 pi c)^2
  const double oms_units = 4.39256635604e-16;  // (2 pi / c)^2
  const double acc_fmax = 0.01;
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
}

void noise_build_table_ch(double T, double fmin, int N, int nch, const double *d0, const double *d1, double *tab) {
  const double fstar = kCLIGHT / (2.0 * M_PI * kLARM);
  for (int n = 0; n < N; n++) {
    const double f = fmin + (double)n / T;
    noise_freq_rows(f, tab, N, n);
    tab[(size_t)kTabCos2x * N + n] = cos(2. * (f / fstar));  // AEnoise_FF's cos 2x
    tab[(size_t)kTabP0 * N + n] = d0[2 * n] * d0[2 * n] + d0[2 * n + 1] * d0[2 * n + 1];
    tab[(size_t)kTabP1 * N + n] = nch == 2 ? d1[2 * n] * d1[2 * n] + d1[2 * n + 1] * d1[2 * n + 1] : 0.0;
    for (int r = kTabXY; r <= kTabYZ; r++) tab[(size_t)r * N + n] = 0.0;
  }
}

void noise_wv_build(int NT, double df, int lmin, int Nlayer, int Q, const double *X, const double *Y, const double *Z,
                    double *tab, double *P) {
  const int Nc = NT / Q;
  const size_t Npix = (size_t)Nlayer * Nc;
  const double invQ = 1.0 / (double)Q;
  for (int j = 0; j < Nlayer; j++) {
    noise_freq_rows((double)(lmin + j) * df, tab, Nlayer, j);
    double S[6] = {0, 0, 0, 0, 0, 0};
    for (int q = 0; q < Nc; q++) {
      double sxx = 0, syy = 0, szz = 0, sxy = 0, sxz = 0, syz = 0;
      for (int i = q * Q; i < (q + 1) * Q; i++) {
        const size_t k = (size_t)i + (size_t)j * NT;
        const double wx = X[k], wy = Y[k], wz = Z[k];
        sxx += wx * wx;
        syy += wy * wy;
        szz += wz * wz;
        sxy += wx * wy;
        sxz += wx * wz;
        syz += wy * wz;
      }
      const size_t kc = (size_t)q + (size_t)j * Nc;
      const double v[6] = {sxx * invQ, syy * invQ, szz * invQ, sxy * invQ, sxz * invQ, syz * invQ};
      for (int e = 0; e < 6; e++) {
        P[(size_t)e * Npix + kc] = v[e];
        S[e] += v[e];
      }
    }
    for (int e = 0; e < 6; e++) tab[(size_t)(kTabXX + e) * Nlayer + j] = S[e];
  }
}

// Natural cubic spline through (x[i], y[i]) in the coefficient form
// y0 + y1 d + y2 d^2 + y3 d^3 on interval i (the tridiagonal solve of
// spline_coefficients, utils/src/glass_math.c:98-178), evaluated with the
// even-spacing lookup of even_sampled_search (:393-402: floor of the offset
// over x[1] - x[0], clamped to [0, n - 1]; the last node's polynomial is the
// constant y[n - 1]).
namespace {
struct SgSpline {
  std::vector<double> x, c0, c1, c2, c3;
  void fit(const std::vector<double> &xs, const std::vector<double> &ys) {
    const int n = (int)xs.size();
    x = xs;
    c0.assign(n, 0.0);
    c1.assign(n, 0.0);
    c2.assign(n, 0.0);
    c3.assign(n, 0.0);
    std::vector<double> h(n, 0.0), rhs(n, 0.0), diag(n, 1.0), up(n, 0.0), z(n, 0.0);
    h[0] = xs[1] - xs[0];
    for (int i = 1; i < n - 1; i++) {
      h[i] = xs[i + 1] - xs[i];
      rhs[i] = 3.0 * ((ys[i + 1] - ys[i]) / h[i] - (ys[i] - ys[i - 1]) / h[i - 1]);
    }
    for (int i = 1; i < n - 1; i++) {  // forward elimination, natural ends
      diag[i] = 2.0 * (xs[i + 1] - xs[i - 1]) - h[i - 1] * up[i - 1];
      up[i] = h[i] / diag[i];
      z[i] = (rhs[i] - h[i - 1] * z[i - 1]) / diag[i];
    }
    c0[n - 1] = ys[n - 1];
    for (int i = n - 2; i >= 0; i--) {  // back substitution
      c0[i] = ys[i];
      c2[i] = z[i] - up[i] * c2[i + 1];
      c1[i] = (c0[i + 1] - c0[i]) / h[i] - h[i] * (c2[i + 1] + 2.0 * c2[i]) / 3.0;
      c3[i] = (c2[i + 1] - c2[i]) / (3.0 * h[i]);
    }
  }
  double at(double v) const {
    const int n = (int)x.size();
    int j = (int)floor((v - x[0]) / (x[1] - x[0]));
    if (j < 0) j = 0;
    if (j > n - 1) j = n - 1;
    const double d = v - x[j];
    return c0[j] + c1[j] * d + c2[j] * d * d + c3[j] * d * d * d;
  }
};
}  // namespace

int noise_sgwb_rows(int nresp, const double *resp, int N, const double *f, double *R6) {
  // alloc_pop_sgwb_response (noise/src/glass_noise_model.c:134-189): 10 to
  // 3000 rows; log of f and of the auto-responses, asinh of the
  // cross-responses over 1e-7
  if (nresp < 10 || nresp > 3000) return -1;
  const double ascale = 1e-7;
  std::vector<double> lf(nresp), col[6];
  for (int e = 0; e < 6; e++) col[e].resize(nresp);
  for (int i = 0; i < nresp; i++) {
    const double *r = resp + 7 * (size_t)i;
    if (!(r[0] > 0) || !(r[1] > 0) || !(r[2] > 0) || !(r[3] > 0)) return -1;
    lf[i] = log(r[0]);
    for (int e = 0; e < 3; e++) col[e][i] = log(r[1 + e]);
    for (int e = 3; e < 6; e++) col[e][i] = asinh(r[1 + e] / ascale);
  }
  SgSpline sp[6];
  for (int e = 0; e < 6; e++) sp[e].fit(lf, col[e]);
  for (int n = 0; n < N; n++) {
    if (f[n] == 0.0) {
      for (int e = 0; e < 6; e++) R6[(size_t)e * N + n] = 0.0;
      continue;
    }
    const double l = log(f[n]);  // generate_sgwb_model (:808-820)
    for (int e = 0; e < 3; e++) R6[(size_t)e * N + n] = exp(sp[e].at(l));
    for (int e = 3; e < 6; e++) R6[(size_t)e * N + n] = ascale * sinh(sp[e].at(l));
  }
  return 0;
}

static int noise_wv_lj(const NoiseWvDev &w) {
  int lj = 4096 / (w.Ncoarse > 0 ? w.Ncoarse : 1);
  if (lj < 1) lj = 1;
  if (lj > kNoiseWvMaxLJ) lj = kNoiseWvMaxLJ;
  return lj;
}

int noise_wv_chunks(const NoiseWvDev &w) {
  const int lj = noise_wv_lj(w);
  return (w.Nlayer + lj - 1) / lj;
}

cudaError_t noise_wv_logl_launch(const NoiseWvDev &w, int mode, int nprop, const double *inst, const double *sgal,
                                 int sg_type, const double *sgwb, double *logl, cudaStream_t stream, int *nlaunch) {
  NoiseWvArgs a;
  a.Nlayer = w.Nlayer;
  a.Ncoarse = w.Ncoarse;
  a.Q = w.Q;
  a.LJ = noise_wv_lj(w);
  a.nchunks = noise_wv_chunks(w);
  a.mode = mode;
  a.inv_ND = 1.0 / (double)((long long)w.NF * w.NT);
  a.tab = w.tab;
  a.P = w.P;
  a.mod = w.mod;
  a.inst = inst;
  a.sgal = sgal;
  a.sg_type = sg_type;
  a.sgwb = sgwb;
  a.rsg = w.rsg;
  int launches = 0;
  cudaError_t e;
  if (mode != 2) {
    for (int p0 = 0; p0 < nprop; p0 += 65535 * 16) {
      const int np = nprop - p0 < 65535 * 16 ? nprop - p0 : 65535 * 16;
      NoiseWvArgs s = a;
      s.inst = inst + 12 * (size_t)p0;
      s.sgal = sgal ? sgal + 5 * (size_t)p0 : nullptr;
      s.sgwb = sgwb ? sgwb + 4 * (size_t)p0 : nullptr;
      s.out = logl + p0;
      noise_wv_stationary_kernel<<<np, kNoiseThreads, 0, stream>>>(s);
      launches++;
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
  } else {
    for (int p0 = 0; p0 < nprop; p0 += 65535) {
      const int np = nprop - p0 < 65535 ? nprop - p0 : 65535;
      NoiseWvArgs s = a;
      s.inst = inst + 12 * (size_t)p0;
      s.sgal = sgal + 5 * (size_t)p0;
      s.sgwb = sgwb ? sgwb + 4 * (size_t)p0 : nullptr;
      s.out = w.partial + (size_t)p0 * a.nchunks;
      noise_wv_dynamic_kernel<<<dim3(a.nchunks, np), kNoiseThreads, 0, stream>>>(s);
      launches++;
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
  }
  // my_noise_log_likelihood_wavelet_coarse's constant over the full pixel count (:1238-1240)
  const double cst = 0.5 * 3 * ((double)w.Nlayer * w.NT) * log(2 * M_PI);
  if (mode == 2) {
    noise_finish_kernel<<<(nprop + 255) / 256, 256, 0, stream>>>(w.partial, a.nchunks, nprop, cst, logl);
  } else {
    noise_wv_const_kernel<<<(nprop + 255) / 256, 256, 0, stream>>>(logl, nprop, cst);
  }
  launches++;
  if (nlaunch) *nlaunch = launches;
  return cudaGetLastError();
}

int noise_chunks(int N) { return (N + kNoiseChunk - 1) / kNoiseChunk; }

static size_t spline_smem(int nch, int kmax) { return sizeof(double) * (size_t)kmax * (1 + 6 * nch); }

cudaError_t spline_noise_launch(const SplineNoiseDev &s, int nprop, int kmax, const int *nknots, const double *knot_f,
                                const double *knot_C, double *logl, cudaStream_t stream, int *nlaunch) {
  static LaunchSetup setup;
  int dummy = 0;
  cudaError_t e = launch_setup(setup, [&](int *o) {
    *o = 1;
    return cudaFuncSetAttribute(spline_noise_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)spline_smem(2, kSplineMaxKnots));
  }, &dummy);
  if (e != cudaSuccess) return e;
  SplineNoiseArgs a;
  a.nch = s.nch;
  a.N = s.N;
  a.kmax = kmax;
  a.tab = s.tab;
  a.nknots = nknots;
  a.knot_f = knot_f;
  a.knot_C = knot_C;
  a.logl = logl;
  spline_noise_kernel<<<nprop, kNoiseThreads, spline_smem(s.nch, kmax), stream>>>(a);
  if (nlaunch) *nlaunch = 1;
  return cudaGetLastError();
}

cudaError_t noise_logl_launch(const NoiseDev &nd, int nprop, const double *inst, const double *sgal, int sg_type,
                              const double *sgwb, double *logl, cudaStream_t stream, int *nlaunch) {
  NoiseArgs a;
  a.N = nd.N;
  a.nchunks = noise_chunks(nd.N);
  a.nprop = nprop;
  a.tab = nd.tab;
  a.inst = inst;
  a.sgal = sgal;
  a.sg_type = sg_type;
  a.sgwb = sgwb;
  a.rsg = nd.rsg;
  a.partial = nd.partial;
  int launches = 0;
  // models in slices of at most 65535 (the grid's y extent)
  for (int p0 = 0; p0 < nprop; p0 += 65535) {
    const int np = nprop - p0 < 65535 ? nprop - p0 : 65535;
    NoiseArgs s = a;
    s.nprop = np;
    s.inst = inst + 12 * (size_t)p0;
    s.sgal = sgal ? sgal + 5 * (size_t)p0 : nullptr;
    s.sgwb = sgwb ? sgwb + 4 * (size_t)p0 : nullptr;
    s.partial = nd.partial + (size_t)p0 * a.nchunks;
    if (nd.nch == 3)
      noise_logl_kernel<<<dim3(a.nchunks, np), kNoiseThreads, 0, stream>>>(s);
    else
      noise_ch12_kernel<<<dim3(a.nchunks, np), kNoiseThreads, 0, stream>>>(s, nd.nch);
    launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  const double cst = nd.nch == 3 ? 3 * nd.N * log(2 * M_PI) : 0.0;
  noise_finish_kernel<<<(nprop + 255) / 256, 256, 0, stream>>>(nd.partial, a.nchunks, nprop, cst, logl);
  launches++;
  if (nlaunch) *nlaunch = launches;
  return cudaGetLastError();
}

}  // namespace glass
