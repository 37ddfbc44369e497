// Gradient of delta logL and Fisher matrix of UCB proposals, by tangent
// (forward-mode) propagation through the mixed-precision waveform, replacing
// the reference's finite-difference ucb_fisher (ucb/src/glass_ucb_waveform.c:364-522),
// which costs eight extra waveforms per source.
//
// Structure of the template used here (ucb/src/glass_ucb_waveform.c:822-922):
// every arm series is  d = S P e^{-i theta}  with S = sinc(arg1) aevol / 4,
// P = DP dplus + DC dcross (DP, DC complex polarisation factors) and
// theta = arg1 - arg2.  Hence
//   * ln A and phi0 act as  dh/dlnA = h,  dh/dphi0 = -i h  (exact);
//   * cos(iota) and psi enter only through DP, DC: h = DP H+ + DC Hx with H+,
//     Hx the responses to unit factors, so two basis templates give both;
//   * f0, fdot and the sky angles need tangent templates
//       dd = d (d ln S - i d theta) + S dP e^{-i theta}
//     propagated sample by sample (FP32: a derivative needs relative, not
//     absolute, phase accuracy).
// Six templates (H+, Hx, T_f0, T_fdot, T_costheta, T_phi) x four A/E series are
// FFT'd; per bin the eight derivatives are assembled and
//   grad_k = (r - h | dh/dp_k),   F_kl = (dh/dp_k | dh/dp_l)
// accumulated (inner product of utils/src/glass_math.c:362-380).
#include <cooperative_groups.h>

#include "ucb_fd_device.cuh"

namespace glass {

constexpr int kGradTemplates = 6;
constexpr int kGradSeries = 4 * kGradTemplates;

// sinc'(x) = (x cos x - sin x)/x^2: Taylor series through x^11 for |x| <= 1.
__device__ __forceinline__ float dsinc_f(float x) {
  if (fabsf(x) > 1.0f) {
    float s, c;
    sincosf(x, &s, &c);
    return (x * c - s) / (x * x);
  }
  const float x2 = x * x;
  float p = 1.9270852604024e-09f;      // 12/13!
  p = fmaf(p, x2, -2.505210838544172e-07f);  // -10/11!
  p = fmaf(p, x2, 2.2045855379188714e-05f);  // 8/9!
  p = fmaf(p, x2, -1.1904761904761906e-03f); // -6/7!
  p = fmaf(p, x2, 3.3333333333333333e-02f);  // 4/5!
  p = fmaf(p, x2, -0.33333333333333333f);    // -2/3!
  return p * x;
}

struct GradPlanArgs {
  PlanArgs base;
  int N_fixed;
  ItemGrad *items;
  double *grad, *fisher;
};

__global__ void __launch_bounds__(256) fd_plangrad_kernel(GradPlanArgs ga) {
  const PlanArgs &a = ga.base;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int b = -1;
  if (i < a.nitems) {
    ItemMix c;
    int st = planmix_item(a, i, ga.N_fixed, c);
    if (st) {
      plan_write_skipped(a, i, st);
      const double v = (st & 3) ? __longlong_as_double(0x7ff8000000000000ULL) : 0.0;
      for (int k = 0; k < 8; k++) ga.grad[8 * (size_t)i + k] = v;
      if (ga.fisher)
        for (int k = 0; k < 64; k++) ga.fisher[64 * (size_t)i + k] = v;
    } else {
      ItemGrad g;
      g.m = c;
      const double *p = a.params + 8 * (size_t)i;
      const double T = a.T;
      const double cth = p[1];
      double sth = sqrt(1.0 - cth * cth);
      if (sth < 1e-9) sth = 1e-9;  // d/dcos(theta) is singular at the poles
      double sph, cph;
      sincos(p[2], &sph, &cph);
      const double u[3] = {cth * cph, cth * sph, -sth}, v[3] = {sph, -cph, 0.};
      const double du_c[3] = {cph, sph, cth / sth}, dv_c[3] = {0., 0., 0.};
      const double du_p[3] = {-cth * sph, cth * cph, 0.}, dv_p[3] = {cph, sph, 0.};
      g.dk_c[0] = (float)(cth / sth * cph);
      g.dk_c[1] = (float)(cth / sth * sph);
      g.dk_c[2] = -1.f;
      g.dk_c[3] = 0.f;
      g.dk_p[0] = (float)(sth * sph);
      g.dk_p[1] = (float)(-sth * cph);
      g.dk_p[2] = 0.f;
      g.dk_p[3] = 0.f;
      int idx = 0;
      for (int r = 0; r < 3; r++)
        for (int s = r; s < 3; s++, idx++) {
          g.ep[idx] = (float)(v[r] * v[s] - u[r] * u[s]);
          g.ec[idx] = (float)(u[r] * v[s] + v[r] * u[s]);
          g.dep_c[idx] = (float)(dv_c[r] * v[s] + v[r] * dv_c[s] - du_c[r] * u[s] - u[r] * du_c[s]);
          g.dec_c[idx] = (float)(du_c[r] * v[s] + u[r] * dv_c[s] + dv_c[r] * u[s] + v[r] * du_c[s]);
          g.dep_p[idx] = (float)(dv_p[r] * v[s] + v[r] * dv_p[s] - du_p[r] * u[s] - u[r] * du_p[s]);
          g.dec_p[idx] = (float)(du_p[r] * v[s] + u[r] * dv_p[s] + dv_p[r] * u[s] + v[r] * du_p[s]);
        }
      const double ci = p[4];
      double s2, c2;
      sincos(2.0 * p[5], &s2, &c2);
      const double Ap = 0.5 * (1.0 + ci * ci);
      g.DP[0] = (float)(Ap * c2);
      g.DP[1] = (float)(ci * s2);
      g.DC[0] = (float)(-Ap * s2);
      g.DC[1] = (float)(ci * c2);
      g.dDP_i[0] = (float)(ci * c2);
      g.dDP_i[1] = (float)s2;
      g.dDC_i[0] = (float)(-ci * s2);
      g.dDC_i[1] = (float)c2;
      g.dDP_s[0] = (float)(-2.0 * Ap * s2);
      g.dDP_s[1] = (float)(2.0 * ci * c2);
      g.dDC_s[0] = (float)(-2.0 * Ap * c2);
      g.dDC_s[1] = (float)(-2.0 * ci * s2);
      g.f0 = (float)(p[0] / T);
      g.fdot = (float)(p[7] / (T * T));
      g.invT = (float)(1.0 / T);
      g.fstar = (float)a.fstar;
      ga.items[i] = g;
      b = fd_bin_of(c.N);
    }
  }
  plan_bin(a, i, b);
}

struct GradConsts {
  float Rf, invLf, AUcf, invTf, AUf, Tf;
};

// One sample n of one proposal: the 6 templates' arm values combined into
// their 4 A/E series each (the slow part of the waveform and its tangents).
__device__ __forceinline__ void grad_sample(const GradConsts &K, const ItemGrad &g, const OrbitSampleMix &o,
                                            const GeoSampleMix &gm, float2 (&accs)[kGradSeries]) {
  const ItemMix &c = g.m;
  // ---- geometry (as slow_sample_mix: offsets and arm monomials from the
  // per-size table), plus absolute positions for d tau/dk
  const float ca = o.ca_hi, sa = o.sa_hi;
  float f[28];
  {
    const float4 *g4 = reinterpret_cast<const float4 *>(gm.f);
#pragma unroll
    for (int q = 0; q < 7; q++) {
      const float4 v = g4[q];
      f[4 * q] = v.x;
      f[4 * q + 1] = v.y;
      f[4 * q + 2] = v.z;
      f[4 * q + 3] = v.w;
    }
  }
  float dx[3], dy[3], dz[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    dx[i] = f[3 * i];
    dy[i] = f[3 * i + 1];
    dz[i] = f[3 * i + 2];
  }
  // carrier phase (double-float) common to the three spacecraft
  const float psi0 = carrier_phase_mix(c, o).hi;
  const float uf = o.u_hi;
  const float tgc = K.AUcf * (c.k[0] * ca + c.k[1] * sa);
  const float gx = K.AUf * ca, gy = K.AUf * sa;  // guiding centre (m)
  float fon[3], arg2[3], aev[3], vv[3], wxi[3], dtc[3], dtp[3], kd[3], kcd[3], kpd[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float kdx = c.k[0] * dx[i] + c.k[1] * dy[i] + c.k[2] * dz[i];
    kd[i] = kdx;
    kcd[i] = g.dk_c[0] * dx[i] + g.dk_c[1] * dy[i] + g.dk_c[2] * dz[i];
    kpd[i] = g.dk_p[0] * dx[i] + g.dk_p[1] * dy[i] + g.dk_p[2] * dz[i];
    const float taui = tgc + kdx * (float)(1.0 / kCLIGHT);
    const float tT = taui * K.invTf;
    const float v = uf - tT;  // xi / T
    vv[i] = v;
    fon[i] = fmaf(c.fdfs, v, c.fonfs0);
    aev[i] = fmaf(c.aef, v, 1.0f);
    arg2[i] = psi0 - c.w0c * kdx + c.p7pi * tT * (tT - 2.0f * uf);
    // d arg2 / d xi and d tau / d(cos theta), d tau / d phi
    wxi[i] = 6.2831853f * fmaf(g.fdot, v * K.Tf, g.f0);
    const float X = gx + dx[i], Y = gy + dy[i], Z = dz[i];
    dtc[i] = (g.dk_c[0] * X + g.dk_c[1] * Y + g.dk_c[2] * Z) * (float)(1.0 / kCLIGHT);
    dtp[i] = (g.dk_p[0] * X + g.dk_p[1] * Y + g.dk_p[2] * Z) * (float)(1.0 / kCLIGHT);
  }
  // unique arms 12, 13, 23: the six quadratic forms share the monomials of the
  // arm's unit vector; the two directions of an arm differ only in k.r's sign
  float qf[3][6], krq[3], dkcq[3], dkpq[3];
#pragma unroll
  for (int q = 0; q < 3; q++) {
    const int i0 = q == 2 ? 1 : 0, i1 = q == 0 ? 1 : 2;
    const float *m = f + 9 + 6 * q;  // x^2, 2xy, 2xz, y^2, 2yz, z^2 of the unit arm
    const float *E[6] = {g.ep, g.ec, g.dep_c, g.dec_c, g.dep_p, g.dec_p};
#pragma unroll
    for (int t = 0; t < 6; t++)
      qf[q][t] = fmaf(E[t][0], m[0], fmaf(E[t][3], m[3], fmaf(E[t][5], m[5], fmaf(E[t][1], m[1], fmaf(E[t][2], m[2], E[t][4] * m[4])))));
    krq[q] = (kd[i1] - kd[i0]) * K.invLf;
    dkcq[q] = (kcd[i1] - kcd[i0]) * K.invLf;
    dkpq[q] = (kpd[i1] - kpd[i0]) * K.invLf;
  }
#pragma unroll
  for (int s = 0; s < kGradSeries; s++) accs[s] = make_float2(0.f, 0.f);

  // combination coefficients of the four A/E series per directed arm
  // (12, 13, 21, 23, 31, 32): a2, a1, e2, e1 (as ae_combos); compile-time
  // constants, so the zero terms vanish
  constexpr float kC[4][6] = {
      {-1.f, 1.f, 0.f, 0.f, 1.f, -1.f},   // a2 = d31 - d32 - d12 + d13
      {0.f, 1.f, -1.f, -1.f, 1.f, 0.f},   // a1 = d13 - d23 - d21 + d31
      {1.f, -1.f, 2.f, -2.f, 1.f, -1.f},  // e2 = d12 - d13 + 2 d21 - 2 d23 + d31 - d32
      {2.f, 1.f, 1.f, -1.f, -1.f, -2.f},  // e1 = 2 d12 + d13 + d21 - d23 - d31 - 2 d32
  };
  const float invfsT = __fdividef(K.invTf, g.fstar);
  const float f0T = g.f0 * K.Tf;  // f0 T
  // 1 / (f0 T aevol_i) per spacecraft, for the amplitude-evolution derivatives
  float rfa[3];
#pragma unroll
  for (int i = 0; i < 3; i++) rfa[i] = __frcp_rn(f0T * aev[i]);
#pragma unroll
  for (int arm = 0; arm < 6; arm++) {
    // directed arm -> (spacecraft i, unique arm q, orientation sign)
    const int i = arm >> 1;
    const int q = (arm == 0 || arm == 2) ? 0 : (arm == 1 || arm == 4) ? 1 : 2;
    const float sg = (arm == 2 || arm == 4 || arm == 5) ? -1.f : 1.f;
    const float dp = qf[q][0], dc = qf[q][1];
    const float kr = sg * krq[q];
    const float dkr_c = sg * dkcq[q];
    const float dkr_p = sg * dkpq[q];
    const float arg1 = 0.5f * fon[i] * (1.0f + kr);
    const float sn = sinc_f(arg1);
    const float gS = __fdividef(dsinc_f(arg1), sn);
    const float S = 0.25f * sn * aev[i];
    float sth, cth;
    fast_sincos(arg1 - arg2[i], &sth, &cth);
    const float2 E = make_float2(cth, -sth);
    const float2 SE = make_float2(S * E.x, S * E.y);
    const float2 Pc = make_float2(g.DP[0] * dp + g.DC[0] * dc, g.DP[1] * dp + g.DC[1] * dc);
    const float2 d = cmul(Pc, SE);
    const float2 Bp = make_float2(dp * SE.x, dp * SE.y);
    const float2 Bx = make_float2(dc * SE.x, dc * SE.y);
    // f0 (params[0] = f0 T)
    const float dA1_0 = 0.5f * (1.0f + kr) * invfsT;
    const float dth_0 = dA1_0 - 6.2831853f * vv[i];
    const float dlS_0 = gS * dA1_0 - c.aef * vv[i] * rfa[i];
    const float2 T0 = cmul(d, make_float2(dlS_0, -dth_0));
    // fdot (params[7] = fdot T^2)
    const float dA1_7 = dA1_0 * vv[i];
    const float dth_7 = dA1_7 - 3.14159265f * vv[i] * vv[i];
    const float dlS_7 = gS * dA1_7 + 0.6666667f * vv[i] * rfa[i];
    const float2 T7 = cmul(d, make_float2(dlS_7, -dth_7));
    // cos(theta)
    const float dA1_c = 0.5f * fon[i] * dkr_c;
    const float dth_c = dA1_c + wxi[i] * dtc[i];
    const float dpc = qf[q][2], dcc = qf[q][3];
    const float2 dPc = make_float2(g.DP[0] * dpc + g.DC[0] * dcc, g.DP[1] * dpc + g.DC[1] * dcc);
    const float2 Tc = cadd(cmul(d, make_float2(gS * dA1_c, -dth_c)), cmul(dPc, SE));
    // phi
    const float dA1_p = 0.5f * fon[i] * dkr_p;
    const float dth_p = dA1_p + wxi[i] * dtp[i];
    const float dpp = qf[q][4], dcp = qf[q][5];
    const float2 dPp = make_float2(g.DP[0] * dpp + g.DC[0] * dcp, g.DP[1] * dpp + g.DC[1] * dcp);
    const float2 Tp = cadd(cmul(d, make_float2(gS * dA1_p, -dth_p)), cmul(dPp, SE));
    const float2 vals[kGradTemplates] = {Bp, Bx, T0, T7, Tc, Tp};
#pragma unroll
    for (int t = 0; t < kGradTemplates; t++)
#pragma unroll
      for (int s = 0; s < 4; s++) {
        const float cf = kC[s][arm];
        if (cf == 1.f) {
          accs[4 * t + s].x += vals[t].x;
          accs[4 * t + s].y += vals[t].y;
        } else if (cf == -1.f) {
          accs[4 * t + s].x -= vals[t].x;
          accs[4 * t + s].y -= vals[t].y;
        } else if (cf != 0.f) {
          accs[4 * t + s].x = fmaf(cf, vals[t].x, accs[4 * t + s].x);
          accs[4 * t + s].y = fmaf(cf, vals[t].y, accs[4 * t + s].y);
        }
      }
  }
}

struct GradSpecArgs {
  int NFFT, cap, bin, fisher_mode;
  GradConsts K;
  const int *bin_count;
  const int *bin_list;
  const ItemGrad *items;
  const OrbitSampleMix *mix;  // this size's orbit table
  const GeoSampleMix *geo;    // this size's sample geometry
  const float2 *tw;
  const float4 *w32, *w32lo, *g32;
  const float2 *invc;  // invC_A, invC_E per segment bin (reference-indexed Fisher)
  const double *Q;
  double *term_y, *grad, *fisher;
  int *status;
};

template <int N>
struct GradCfg {
  // N = 256: two samples and two bins per thread, at most 168 registers (three
  // 128-thread groups per SM instead of four 64-thread ones, which the 205
  // registers of the four-sample form allowed); other sizes four per thread
  static constexpr int GT = N == 256 ? N / 2 : N / 4;
  static constexpr int MINB = N == 256 ? 3 : 1;
  static constexpr int CTA = GT >= 64 ? GT : 128;
  static constexpr int GPC = CTA / GT;
  static constexpr int NACC = 8 + 36;  // gradient, Fisher upper triangle
  // 24 series of N per group in padded rows (pad16), twiddles likewise
  static constexpr int SN = pad16(N);
  static constexpr size_t group_floats2 = (size_t)kGradSeries * SN;
  static constexpr size_t bytes = sizeof(float2) * (SN + GPC * group_floats2) + sizeof(float2) * 32 * GPC;
};

// One group of N/4 threads per proposal: the 24 series are computed sample by
// sample straight into shared memory, FFT'd template by template, whitened,
// and reduced to the gradient and the Fisher matrix.  Nothing of size N
// leaves the SM.
template <int N>
__global__ void __launch_bounds__(GradCfg<N>::CTA, GradCfg<N>::MINB) fd_gradspec_kernel(GradSpecArgs a) {
  using Cfg = GradCfg<N>;
  constexpr int GT = Cfg::GT, GPC = Cfg::GPC, NACC = Cfg::NACC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int SN = Cfg::SN;
  float2 *tw = reinterpret_cast<float2 *>(smem_raw);
  float2 *groups = tw + SN;
  float2 *redall = groups + GPC * Cfg::group_floats2;
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[pad16(i)] = a.tw[i];
  __syncthreads();
  const int g = threadIdx.x / GT, lane = threadIdx.x % GT;
  float2 *sbuf = groups + g * Cfg::group_floats2;  // [s SN + pad16(n)], s = 4 t + combo
  float *part = reinterpret_cast<float *>(sbuf);   // reduction scratch after use
  float2 *red = redall + 32 * g;
  const int count = a.bin_count[a.bin];
  const int NFFT = a.NFFT;

  for (int base = blockIdx.x * GPC; base < count; base += gridDim.x * GPC) {
    const int slot = base + g;
    const bool valid = slot < count;
    const int sl = valid ? slot : count - 1;
    const int item = a.bin_list[sl];
    const ItemGrad &it = a.items[item];
    const int seg = it.m.seg, imin = it.m.imin;
    // the 24 series, N/GT samples per thread
#pragma unroll 1
    for (int r = 0; r < N / GT; r++) {
      const int n = lane + GT * r;
      float2 accs[kGradSeries];
      grad_sample(a.K, it, a.mix[n], a.geo[n], accs);
#pragma unroll
      for (int s = 0; s < kGradSeries; s++) sbuf[(size_t)s * SN + pad16(n)] = accs[s];
    }
    group_sync<GT>();
    // FFT all 24 series (whitening is applied per bin below, with the
    // segment's TDI/whitening table loaded once per bin for all templates)
    fft_reg_smem<N, GT, kGradSeries>(sbuf, tw, lane);
    // assemble the eight derivatives per bin and accumulate
    float accg[NACC];
#pragma unroll
    for (int q = 0; q < NACC; q++) accg[q] = 0.f;
    float racc = 0.f;
    const float s = it.m.amp_hi;
    const float2 DP = make_float2(it.DP[0], it.DP[1]), DC = make_float2(it.DC[0], it.DC[1]);
    const float2 dDPi = make_float2(it.dDP_i[0], it.dDP_i[1]), dDCi = make_float2(it.dDC_i[0], it.dDC_i[1]);
    const float2 dDPs = make_float2(it.dDP_s[0], it.dDP_s[1]), dDCs = make_float2(it.dDC_s[0], it.dDC_s[1]);
    // whitened template t, channel ch (0 A, 1 E) at bin k: the channel's two
    // arm-combination spectra times the bin's table entries
    auto W = [&](int t, int ch, int k, float4 gt) {
      const float2 *f = sbuf + (size_t)(4 * t + 2 * ch) * SN + pad16(k);
      return cadd(cmul(f[0], make_float2(gt.x, gt.y)), cmul(f[SN], make_float2(gt.z, gt.w)));
    };
#pragma unroll 1
    for (int r = 0; r < N / GT; r++) {
      const int k = lane + GT * r;
      const int m = (k + N / 2) & (N - 1);
      const int j = imin + m;
      if (j < 0 || j >= NFFT) continue;
      const size_t sj = (size_t)seg * NFFT + j;
      const float4 w = a.w32[sj], wl = a.w32lo[sj];
      const float4 gAE[2] = {a.g32[2 * sj], a.g32[2 * sj + 1]};
      float qw[2] = {1.f, 1.f};
      if (a.fisher_mode == 1) {
        const float2 ic_t = a.invc[(size_t)seg * NFFT + m], ic_j = a.invc[sj];
        qw[0] = ic_t.x / ic_j.x;
        qw[1] = ic_t.y / ic_j.y;
      }
#pragma unroll
      for (int ch = 0; ch < 2; ch++) {
        const float4 gt = gAE[ch];
        const float2 Hp = cscale(W(0, ch, k, gt), s), Hx = cscale(W(1, ch, k, gt), s);
        const float2 h = cadd(cmul(DP, Hp), cmul(DC, Hx));
        float2 D[8];
        D[0] = cscale(W(2, ch, k, gt), s);
        D[1] = cscale(W(4, ch, k, gt), s);
        D[2] = cscale(W(5, ch, k, gt), s);
        D[3] = h;
        D[4] = cadd(cmul(dDPi, Hp), cmul(dDCi, Hx));
        D[5] = cadd(cmul(dDPs, Hp), cmul(dDCs, Hx));
        D[6] = cmi(h);
        D[7] = cscale(W(3, ch, k, gt), s);
        const float wr = ch ? w.z : w.x, wi = ch ? w.w : w.y;
        const float lr = ch ? wl.z : wl.x, li = ch ? wl.w : wl.y;
        const float rr = (wr - h.x) + lr, ri = (wi - h.y) + li;
        racc += fmaf(rr, rr, ri * ri);
        // half of every sum (the factor 2 of (a|b) = 2 sum Re(a b*) is applied
        // once at the end, where it is exact)
#pragma unroll
        for (int p = 0; p < 8; p++) accg[p] = fmaf(rr, D[p].x, fmaf(ri, D[p].y, accg[p]));
        int q = 8;
#pragma unroll
        for (int p = 0; p < 8; p++)
#pragma unroll
          for (int l = p; l < 8; l++, q++) accg[q] = fmaf(qw[ch], fmaf(D[p].x, D[l].x, D[p].y * D[l].y), accg[q]);
      }
    }
    // reduce over the group: per-thread partials in shared memory (reusing the
    // series buffer once every thread is done with it)
    // rows of GT + 1 floats: lane q summing row q reads bank (q + t) mod 32
    constexpr int PS = GT + 1;
    group_sync<GT>();
#pragma unroll
    for (int q = 0; q < NACC; q++) part[q * PS + lane] = accg[q];
    const df rs = group_sum_df<GT>(racc, red, lane);
    group_sync<GT>();
    for (int q = lane; q < NACC; q += GT) {
      float sum = 0.f;
      for (int t = 0; t < GT; t++) sum += part[q * PS + t];
      part[q * PS] = sum;  // row head
    }
    group_sync<GT>();
    if (valid) {
      for (int q = lane; q < NACC; q += GT) {
        const double v = 2.0 * (double)part[q * PS];
        if (q < 8) {
          a.grad[8 * (size_t)item + q] = v;
        } else if (a.fisher) {
          int qq = q - 8, p = 0;
          while (qq >= 8 - p) {
            qq -= 8 - p;
            p++;
          }
          const int l = p + qq;
          a.fisher[64 * (size_t)item + 8 * p + l] = v;
          a.fisher[64 * (size_t)item + 8 * l + p] = v;
        }
      }
      if (lane == 0) {
        const int jlo = imin < 0 ? 0 : imin;
        const int jhi = imin + N > NFFT ? NFFT : imin + N;
        const double *Qs = a.Q + (size_t)seg * (NFFT + 1);
        const double term = (Qs[jhi] - Qs[jlo]) - ((double)rs.hi + (double)rs.lo);
        a.term_y[item] = term;
        if (a.status) a.status[item] = isfinite(term) ? 0 : 1;
      }
    }
    group_sync<GT>();
  }
}

// Sizes 2048 and 4096: the 24 series of a proposal (384 KB at N = 4096 with
// a work buffer) do not fit one SM, so a cluster of 8 CTAs takes each
// proposal and keeps them in its distributed shared memory: CTA r computes
// samples [r N/8, (r+1) N/8) of all 24 series (the per-sample work shares its
// geometry across the series) and stores each value in the CTA that owns the
// series (3 per CTA); each CTA transforms its three series; CTA r then
// assembles the derivatives over bins [r N/8, (r+1) N/8), reading the 24
// spectra of a bin from the CTAs that hold them, and CTA 0 sums the eight
// CTAs' partial sums.
constexpr int kGradCluster = 8;
constexpr int kGradBigThreads = 256;

template <int N>
struct GradBigCfg {
  static constexpr int SPC = kGradSeries / kGradCluster;  // series per CTA
  static constexpr size_t bytes = sizeof(float2) * (size_t)N * (SPC + 2);  // series, work buffer, twiddles
};

// Stockham FFT of N complex floats by the CTA, out of place between x and y:
// radix-4 stages (butterfly i < N/4, k = i mod p, reads x[i + m N/4], writes
// y[(i - k) 4 + k + m p] after the twiddles exp(-2 pi i m k / (4p))) and a
// radix-2 stage when log2 N is odd.  tw[j] = exp(-2 pi i j / N).  Sizes
// 2048 and 4096 take an even number of passes: the result is back in x.
template <int N>
__device__ __forceinline__ void cta_fft_f32(float2 *x, float2 *y, const float2 *tw) {
  constexpr int L2 = N == 4096 ? 12 : 11;
  static_assert((N == 2048 || N == 4096) && (L2 / 2 + L2 % 2) % 2 == 0, "even number of passes");
  int p = 1;
#pragma unroll 1
  for (; 4 * p <= N; p <<= 2) {
    const int step = N / (4 * p), q = N / 4;
    for (int i = threadIdx.x; i < q; i += blockDim.x) {
      const int k = i & (p - 1);
      float2 u0 = x[i], u1 = x[i + q], u2 = x[i + 2 * q], u3 = x[i + 3 * q];
      if (p > 1) {
        u1 = cmul(u1, tw[k * step]);
        u2 = cmul(u2, tw[2 * k * step]);
        u3 = cmul(u3, tw[3 * k * step]);
      }
      const float2 a = cadd(u0, u2), b = csub(u0, u2), c = cadd(u1, u3), d = cmi(csub(u1, u3));
      const int j = (i - k) * 4 + k;
      y[j] = cadd(a, c);
      y[j + p] = cadd(b, d);
      y[j + 2 * p] = csub(a, c);
      y[j + 3 * p] = csub(b, d);
    }
    __syncthreads();
    float2 *t = x;
    x = y;
    y = t;
  }
  if (p < N) {  // log2 N odd: p = N/2
    for (int i = threadIdx.x; i < N / 2; i += blockDim.x) {
      const int k = i & (p - 1);
      const float2 a = x[i], b = cmul(x[i + N / 2], tw[k]);
      const int j = (i - k) * 2 + k;
      y[j] = cadd(a, b);
      y[j + p] = csub(a, b);
    }
    __syncthreads();
  }
}

template <int N>
__global__ void __launch_bounds__(kGradBigThreads, 1) fd_gradspec_big_kernel(GradSpecArgs a) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  constexpr int SPC = GradBigCfg<N>::SPC, CL = kGradCluster, NB = N / CL, NACC = 8 + 36;
  constexpr int NW = kGradBigThreads / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *ser = reinterpret_cast<float2 *>(smem_raw);  // [SPC][N]: this CTA's series, then spectra
  float2 *work = ser + SPC * N;
  float2 *tw = work + N;
  __shared__ float s_warp[NW][NACC];
  __shared__ float2 s_warp_rr[NW];
  __shared__ float s_tot[NACC];
  __shared__ float2 s_rr;
  const int r = (int)cluster.block_rank(), lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = a.tw[i];
  float2 *sers[CL];
#pragma unroll
  for (int q = 0; q < CL; q++) sers[q] = cluster.map_shared_rank(ser, q);
  const int count = a.bin_count[a.bin];
  const int NFFT = a.NFFT;
  for (int slot = (int)(blockIdx.x / CL); slot < count; slot += (int)(gridDim.x / CL)) {
    const int item = a.bin_list[slot];
    const ItemGrad &it = a.items[item];
    const int seg = it.m.seg, imin = it.m.imin;
    // 1. this CTA's samples of the 24 series, to the CTAs that own them
    for (int n = r * NB + threadIdx.x; n < (r + 1) * NB; n += blockDim.x) {
      float2 accs[kGradSeries];
      grad_sample(a.K, it, a.mix[n], a.geo[n], accs);
#pragma unroll
      for (int sidx = 0; sidx < kGradSeries; sidx++) sers[sidx / SPC][(sidx % SPC) * N + n] = accs[sidx];
    }
    cluster.sync();
    // 2. this CTA's three series
#pragma unroll 1
    for (int sidx = 0; sidx < SPC; sidx++) cta_fft_f32<N>(ser + sidx * N, work, tw);
    cluster.sync();
    // 3. derivatives over this CTA's bins (as fd_gradspec_kernel)
    float accg[NACC];
#pragma unroll
    for (int q = 0; q < NACC; q++) accg[q] = 0.f;
    float racc = 0.f;
    const float sc = it.m.amp_hi;
    const float2 DP = make_float2(it.DP[0], it.DP[1]), DC = make_float2(it.DC[0], it.DC[1]);
    const float2 dDPi = make_float2(it.dDP_i[0], it.dDP_i[1]), dDCi = make_float2(it.dDC_i[0], it.dDC_i[1]);
    const float2 dDPs = make_float2(it.dDP_s[0], it.dDP_s[1]), dDCs = make_float2(it.dDC_s[0], it.dDC_s[1]);
    auto W = [&](int t, int ch, int k, float4 gt) {
      const int s0 = 4 * t + 2 * ch, s1 = s0 + 1;
      const float2 f0 = sers[s0 / SPC][(s0 % SPC) * N + k], f1 = sers[s1 / SPC][(s1 % SPC) * N + k];
      return cadd(cmul(f0, make_float2(gt.x, gt.y)), cmul(f1, make_float2(gt.z, gt.w)));
    };
#pragma unroll 1
    for (int k = r * NB + threadIdx.x; k < (r + 1) * NB; k += blockDim.x) {
      const int m = (k + N / 2) & (N - 1);
      const int j = imin + m;
      if (j < 0 || j >= NFFT) continue;
      const size_t sj = (size_t)seg * NFFT + j;
      const float4 w = a.w32[sj], wl = a.w32lo[sj];
      const float4 gAE[2] = {a.g32[2 * sj], a.g32[2 * sj + 1]};
      float qw[2] = {1.f, 1.f};
      if (a.fisher_mode == 1) {
        const float2 ic_t = a.invc[(size_t)seg * NFFT + m], ic_j = a.invc[sj];
        qw[0] = ic_t.x / ic_j.x;
        qw[1] = ic_t.y / ic_j.y;
      }
#pragma unroll
      for (int ch = 0; ch < 2; ch++) {
        const float4 gt = gAE[ch];
        const float2 Hp = cscale(W(0, ch, k, gt), sc), Hx = cscale(W(1, ch, k, gt), sc);
        const float2 h = cadd(cmul(DP, Hp), cmul(DC, Hx));
        float2 D[8];
        D[0] = cscale(W(2, ch, k, gt), sc);
        D[1] = cscale(W(4, ch, k, gt), sc);
        D[2] = cscale(W(5, ch, k, gt), sc);
        D[3] = h;
        D[4] = cadd(cmul(dDPi, Hp), cmul(dDCi, Hx));
        D[5] = cadd(cmul(dDPs, Hp), cmul(dDCs, Hx));
        D[6] = cmi(h);
        D[7] = cscale(W(3, ch, k, gt), sc);
        const float wr = ch ? w.z : w.x, wi = ch ? w.w : w.y;
        const float lr = ch ? wl.z : wl.x, li = ch ? wl.w : wl.y;
        const float rr = (wr - h.x) + lr, ri = (wi - h.y) + li;
        racc += fmaf(rr, rr, ri * ri);
#pragma unroll
        for (int p = 0; p < 8; p++) accg[p] = fmaf(rr, D[p].x, fmaf(ri, D[p].y, accg[p]));
        int q = 8;
#pragma unroll
        for (int p = 0; p < 8; p++)
#pragma unroll
          for (int l = p; l < 8; l++, q++) accg[q] = fmaf(qw[ch], fmaf(D[p].x, D[l].x, D[p].y * D[l].y), accg[q]);
      }
    }
    // 4. sums over the CTA (the residual power in double-float), then over the cluster
    df rs = {racc, 0.f};
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
      for (int q = 0; q < NACC; q++) accg[q] += __shfl_xor_sync(0xffffffffu, accg[q], off);
      rs = df_add(rs, df{__shfl_xor_sync(0xffffffffu, rs.hi, off), __shfl_xor_sync(0xffffffffu, rs.lo, off)});
    }
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < NACC; q++) s_warp[wid][q] = accg[q];
      s_warp_rr[wid] = make_float2(rs.hi, rs.lo);
    }
    __syncthreads();
    if (threadIdx.x < NACC) {
      float v = 0.f;
      for (int w2 = 0; w2 < NW; w2++) v += s_warp[w2][threadIdx.x];
      s_tot[threadIdx.x] = v;
    } else if (threadIdx.x == NACC) {
      df t = {0.f, 0.f};
      for (int w2 = 0; w2 < NW; w2++) t = df_add(t, df{s_warp_rr[w2].x, s_warp_rr[w2].y});
      s_rr = make_float2(t.hi, t.lo);
    }
    cluster.sync();  // every CTA's sums are published; the spectra are no longer read
    if (r == 0) {
      if (threadIdx.x < NACC) {
        const int q = threadIdx.x;
        float v = 0.f;
        for (int c = 0; c < CL; c++) v += *cluster.map_shared_rank(&s_tot[q], c);
        const double dv = 2.0 * (double)v;
        if (q < 8) {
          a.grad[8 * (size_t)item + q] = dv;
        } else if (a.fisher) {
          int qq = q - 8, p = 0;
          while (qq >= 8 - p) {
            qq -= 8 - p;
            p++;
          }
          const int l = p + qq;
          a.fisher[64 * (size_t)item + 8 * p + l] = dv;
          a.fisher[64 * (size_t)item + 8 * l + p] = dv;
        }
      } else if (threadIdx.x == NACC) {
        df t = {0.f, 0.f};
        for (int c = 0; c < CL; c++) {
          const float2 o = *cluster.map_shared_rank(&s_rr, c);
          t = df_add(t, df{o.x, o.y});
        }
        const int jlo = imin < 0 ? 0 : imin;
        const int jhi = imin + N > NFFT ? NFFT : imin + N;
        const double *Qs = a.Q + (size_t)seg * (NFFT + 1);
        const double term = (Qs[jhi] - Qs[jlo]) - ((double)t.hi + (double)t.lo);
        a.term_y[item] = term;
        if (a.status) a.status[item] = isfinite(term) ? 0 : 1;
      }
    }
    cluster.sync();  // CTA 0 has read the sums before the next proposal overwrites them
  }
}

template <int N>
static cudaError_t launch_gradspec_big(const GradSpecArgs &a, int nitems_bound, int num_sms, cudaStream_t stream) {
  const size_t smem = GradBigCfg<N>::bytes;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kGradCluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(kGradBigThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  static LaunchSetup setup;
  int ncl = 0;
  cudaError_t e = launch_setup(setup, [&](int *o) {
    cudaError_t r = cudaFuncSetAttribute(fd_gradspec_big_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (r != cudaSuccess) return r;
    cudaLaunchConfig_t q = cfg;
    q.gridDim = dim3(kGradCluster * num_sms);
    return cudaOccupancyMaxActiveClusters(o, fd_gradspec_big_kernel<N>, &q);
  }, &ncl);
  if (e != cudaSuccess) return e;
  if (ncl < 1) ncl = 1;
  if (ncl > nitems_bound) ncl = nitems_bound > 0 ? nitems_bound : 1;
  cfg.gridDim = dim3(kGradCluster * ncl);
  return cudaLaunchKernelEx(&cfg, fd_gradspec_big_kernel<N>, a);
}

template <int N>
static cudaError_t launch_gradspec(const GradSpecArgs &a, int nitems_bound, int num_sms, cudaStream_t stream) {
  using Cfg = GradCfg<N>;
  size_t smem = Cfg::bytes;
  static LaunchSetup setup;
  int occ = 0;
  cudaError_t e = launch_setup(setup, [&](int *o) {
    cudaError_t r = cudaFuncSetAttribute(fd_gradspec_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (r != cudaSuccess) return r;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, fd_gradspec_kernel<N>, Cfg::CTA, smem);
  }, &occ);
  if (e != cudaSuccess) return e;
  int need = (nitems_bound + Cfg::GPC - 1) / Cfg::GPC;
  int grid = occ * num_sms;
  if (need < grid) grid = need;
  if (grid < 1) grid = 1;
  fd_gradspec_kernel<N><<<grid, Cfg::CTA, smem, stream>>>(a);
  return cudaGetLastError();
}

size_t fd_grad_series_bytes(int, int) { return 0; }  // the series never leave shared memory

cudaError_t fd_grad_launch(const FdBankDev &bank, const FdTablesDev &tab, FdWorkDev &work, int nitems,
                           const int *item_seg, const double *params, int N_fixed, int fisher_mode, double *term_y,
                           double *grad, double *fisher, int *status, int num_sms, cudaStream_t stream,
                           int *nlaunch) {
  cudaError_t e;
  int launches = 0;
  if (!work.counts_zero && (e = cudaMemsetAsync(work.bin_count, 0, sizeof(int) * (kNumBins + 1), stream)) != cudaSuccess)
    return e;
  work.counts_zero = false;
  GradPlanArgs ga;
  PlanArgs &pa = ga.base;
  pa.nitems = nitems;
  pa.nseg = bank.nseg;
  pa.NFFT = bank.NFFT;
  pa.cap = work.cap;
  pa.precision = 1;
  pa.n_fixed = N_fixed;
  pa.T = bank.T;
  pa.fstar = bank.fstar;
  pa.L = kLARM;
  pa.item_seg = item_seg;
  pa.params = params;
  pa.term_x = nullptr;
  pa.seg_qmin = bank.qmin;
  pa.items64 = nullptr;
  pa.itemsmix = nullptr;
  pa.bin_count = work.bin_count;
  pa.bin_list = work.bin_list;
  pa.dlogl = term_y;
  pa.term_y = nullptr;
  pa.hh = nullptr;
  pa.status = status;
  ga.N_fixed = N_fixed;
  ga.items = work.itemsgrad;
  ga.grad = grad;
  ga.fisher = fisher;
  {
    // one thread per proposal in CTAs of 64..256 threads, as few CTAs as
    // SMs where the batch allows (the kernel is a latency-bound FP64 chain: a
    // second CTA on some SMs doubles their time)
    int per = (nitems + num_sms - 1) / (num_sms > 0 ? num_sms : 1);
    per = (per + 31) / 32 * 32;
    per = per < 64 ? 64 : (per > 256 ? 256 : per);
    fd_plangrad_kernel<<<(nitems + per - 1) / per, per, 0, stream>>>(ga);
  }
  launches++;
  if ((e = cudaGetLastError()) != cudaSuccess) return e;

  GradSpecArgs a;
  a.NFFT = bank.NFFT;
  a.cap = work.cap;
  a.fisher_mode = fisher_mode;
  a.bin_count = work.bin_count;
  a.items = work.itemsgrad;
  a.K.Rf = (float)(kAU * (kLARM / (2.0 * kSQ3 * kAU)));
  a.K.invLf = (float)(1.0 / kLARM);
  a.K.AUcf = (float)(kAU / kCLIGHT);
  a.K.invTf = (float)(1.0 / bank.T);
  a.K.AUf = (float)kAU;
  a.K.Tf = (float)bank.T;
  a.w32 = bank.w32;
  a.w32lo = bank.w32lo;
  a.g32 = bank.g32;
  a.invc = bank.invc;
  a.Q = bank.Q;
  a.term_y = term_y;
  a.grad = grad;
  a.fisher = fisher;
  a.status = status;
  if ((e = cudaEventRecord(work.fork, stream)) != cudaSuccess) return e;
  int nb = 0;
  for (int b = 0; b < kNumBins; b++) {
    const int N = 32 << b;
    if (N > pa.NFFT) break;
    cudaStream_t sb = work.side[b];
    if ((e = cudaStreamWaitEvent(sb, work.fork, 0)) != cudaSuccess) return e;
    a.bin = b;
    a.bin_list = work.bin_list + (size_t)b * work.cap;
    a.tw = tab.tw32[b];
    a.mix = tab.mix[b];
    a.geo = tab.geo[b];
    switch (N) {
      case 32: e = launch_gradspec<32>(a, nitems, num_sms, sb); break;
      case 64: e = launch_gradspec<64>(a, nitems, num_sms, sb); break;
      case 128: e = launch_gradspec<128>(a, nitems, num_sms, sb); break;
      case 256: e = launch_gradspec<256>(a, nitems, num_sms, sb); break;
      case 512: e = launch_gradspec<512>(a, nitems, num_sms, sb); break;
      case 1024: e = launch_gradspec<1024>(a, nitems, num_sms, sb); break;
      case 2048: e = launch_gradspec_big<2048>(a, nitems, num_sms, sb); break;
      default: e = launch_gradspec_big<4096>(a, nitems, num_sms, sb); break;
    }
    launches++;
    // the branch is joined to the caller's stream even when its launch failed
    const cudaError_t ej = cudaEventRecord(work.join[b], sb);
    nb++;
    if (e == cudaSuccess) e = ej;
    if (e != cudaSuccess) {
      for (int q = 0; q < nb; q++) cudaStreamWaitEvent(stream, work.join[q], 0);
      return e;
    }
  }
  for (int b = 0; b < nb; b++)
    if ((e = cudaStreamWaitEvent(stream, work.join[b], 0)) != cudaSuccess) return e;
  // leave the counts at zero for the next launch sequence
  if ((e = cudaMemsetAsync(work.bin_count, 0, sizeof(int) * (kNumBins + 1), stream)) != cudaSuccess) return e;
  work.counts_zero = true;
  if (nlaunch) *nlaunch = launches;
  return cudaSuccess;
}

}  // namespace glass
