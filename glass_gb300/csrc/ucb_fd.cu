// Fourier-domain UCB waveform and delta-logL kernels for sm_103a: plan,
// tables, orchestration and the drop-in single-waveform path.
//
// The reference computes one template at a time on the CPU: ucb_waveform
// (ucb/src/glass_ucb_waveform.c:738-1001) evaluates the slowly varying part of
// the response of the six LISA arms at N sample times, takes six N-point FFTs,
// and synthesises the TDI channels bin by bin (utils/src/glass_lisa.c:645-710);
// gaussian_log_likelihood (utils/src/glass_model.c:726-774) then sums the
// noise-weighted residual power over the whole segment.
//
// Here a batch of proposals of mixed sizes N (32..4096) is evaluated in three
// steps on one stream:
//   1. plan (one thread per proposal, FP64): the reference's bandwidth rule
//      gives N, the alignment gives the template's first segment bin, and the
//      per-proposal constants are prepared; proposals are binned by N;
//   2. slow part (one thread per (proposal, sample), all sizes in one launch):
//      the six arm responses, combined in the time domain into the four series
//      whose FFTs make the A and E channels (the TDI sums are linear, so
//      FFT(a - b) replaces FFT(a) - FFT(b)); written to an L2-resident scratch;
//   3. per size, concurrently: four N-point radix-4/2 Stockham FFTs in shared
//      memory, the per-segment-bin table folding TDI transfer factors, the A/E
//      combination and noise whitening, and the residual power over the
//      template support reduced to one number per proposal.
// Only the template support is visited: logL(r - h) - logL(r) differs from zero
// only there.
//
// Two precisions share the structure: plain FP64 (this file and
// ucb_fd_fp64.cu; the delay and carrier phase round each operation on its
// own, as the reference's C does), and a mixed form
// (ucb_fd_mixed.cu) in which the carrier phase is carried in double-float
// arithmetic and everything else is FP32.
#include "ucb_fd_device.cuh"

namespace glass {

cudaError_t fd_launch_slow_mixed(const SlowArgs &a, int num_sms, cudaStream_t stream, int block, int cap);
cudaError_t fd_launch_slow_fp64(const SlowArgs &a, int num_sms, cudaStream_t stream);
cudaError_t fd_launch_spec_mixed(int N, const SpecArgs &a, int nitems, int num_sms, cudaStream_t stream, bool perch);
cudaError_t fd_launch_spec_fp64(int N, const SpecArgs &a, int nitems, int num_sms, cudaStream_t stream, bool perch);
cudaError_t fd_launch_spec_all_mixed(const SpecAllArgs &A, int num_sms, cudaStream_t stream, bool perch, int cap);
cudaError_t fd_launch_spec_all_fp64(const SpecAllArgs &A, int num_sms, cudaStream_t stream, bool perch);

// ------------------------------------------------------------- plan kernels
// Plain-FP64 plan: ucb_bandwidth, ucb_alignment and the per-proposal constants
// entirely in FP64, one thread per proposal.
__global__ void __launch_bounds__(64) fd_plan64_kernel(PlanArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int b = -1;
  if (i < a.nitems) {
    double p[8];
    int seg;
    int st = plan_validate(a, i, p, seg);
    const double T = a.T, f0 = p[0] / T;
    int N = 0;
    if (!st) {
      N = a.n_fixed > 0 ? a.n_fixed : 2 * bandwidth_dev(a.L, a.fstar, f0, p[7] / (T * T), p[1], exp(p[3]), T, a.NFFT);
      if (N < kMinN || N > kMaxN) st |= 1;
    }
    int imin = 0;
    if (!st) {
      imin = (int)((long long)(f0 * T) - N / 2) - a.seg_qmin[seg];
      if (imin >= a.NFFT || imin + N <= 0) st = 4;
    }
    if (st) {
      plan_write_skipped(a, i, st);
    } else {
      SourceGeom g;
      source_geometry(p, 8, T, g);
      ItemF64 c;
      make_item_f64(g, N, c);
      c.seg = seg;
      c.N = N;
      c.imin = imin;
      c.pad = 0;
      a.items64[i] = c;
      b = fd_bin_of(N);
    }
  }
  plan_bin(a, i, b);
}

// Sets a CUDA-graph conditional node's value to (*count > 0).
__global__ void fd_cond_kernel(const int *count, cudaGraphConditionalHandle h) {
  if (threadIdx.x == 0) cudaGraphSetConditional(h, *(volatile const int *)count > 0 ? 1u : 0u);
}

// Mixed-precision plan, warp-specialised: GB300's FP64 pipe issues a warp
// instruction only every few tens of cycles, so the FP64 work of a proposal is
// split over four warps that run in parallel on different SM sub-partitions,
// each writing its share of the ItemMix record directly: warp 0 the bandwidth
// rule (FP32, FP64 only near a size boundary) and placement, warp 1 the sky
// direction, polarisation tensors and Doppler constants, warp 2 the
// polarisation factors and the FP32 frequency constants, warp 3 the amplitude
// and the double-float carrier constants.  The antenna tensors Mr, Mi are then
// assembled in FP64 by all 128 threads; only the N-dependent fields wait for
// the barrier.  Same results as planmix_item (the FP32 constants to rounding).
// Proposals per CTA: ceil(n / SMs) lanes of each role warp, at least 16, so
// that a batch of a few thousand proposals is one wave over every SM (the
// kernel is latency-bound; a second CTA on some SMs doubles their time).

__global__ void __launch_bounds__(128) fd_planmix_kernel(PlanArgs a) {
  __shared__ double s_ep[32][6], s_ec[32][6], s_dp[32][4], s_amp[32];
  __shared__ int s_st[32], s_N[32], s_imin[32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const int i = blockIdx.x * a.per_cta + l;
  const bool in = l < a.per_cta && i < a.nitems;
  double p[8];
  int seg = 0, st = 1;
  if (in) st = plan_validate(a, i, p, seg);
  const double T = a.T;
  ItemMix *c = a.itemsmix + (in ? i : 0);
  if (in && !st) {
    const double f0 = p[0] / T;
    if (w == 0) {
      int N;
      if (a.n_fixed > 0) {
        N = a.n_fixed;
      } else {
        const float Tf = (float)T, f0f = (float)f0, costhf = (float)p[1];
        const float fdotf = (float)(p[7] / (T * T));
        const float ampf = expf((float)p[3]);
        const float sinthf = sqrtf(fmaxf(0.f, (1.f - costhf) * (1.f + costhf)));
        const int Nmin = 16;
        const int half = a.NFFT / 2;
        const int Nmax = half >= 1 ? (1 << (31 - __clz(half))) : 0;
        float bw = 2.f * Tf * ((4.f + 6.2831853f * f0f * (float)(kAU / kCLIGHT) * sinthf) / (float)kYEAR +
                               fabsf(fdotf) * Tf);
        int DS = pow2_above_f32(bw - 1.f);
        if (DS < 0) DS = doppler_spread_fp64(T, f0, p[7] / (T * T), p[1]);
        if (DS > Nmax) DS = Nmax;
        if (DS < Nmin) DS = Nmin;
        const float x = f0f / (float)a.fstar;
        float sx, cx;
        sincosf(x, &sx, &cx);
        const float c2x = 2.f * cx * cx - 1.f;
        const float wf = 6.2831853f * f0f, w2 = wf * wf;
        const float q1 = 2.0e-5f / f0f, q2 = q1 * q1, q4 = q2 * q2, r1 = 1.0e-4f / f0f;
        const float red = 1.f + 16.f * (q4 * q4 * q2 + r1 * r1);
        const float twoL = 2.f * (float)a.L;
        const float sn4L2 = (16.f / 3.f) * sx * sx *
                            ((2.f + cx) * (float)(kSPS + kSLOC) +
                             2.f * (3.f + 2.f * cx + c2x) * ((float)(kSLOC / 2.0) + (float)kSACC / (w2 * w2) * red));
        const float snrm = ampf * sqrtf(Tf) * sx * twoL / sqrtf(sn4L2);
        int SS = pow2_above_f32(snrm - 1.f);
        if (SS < 0) SS = snr_spread_fp64(T, f0, p[3], a.L, a.fstar);
        if (SS > Nmax) SS = Nmax;
        if (SS < Nmin) SS = Nmin;
        N = 2 * ((DS > SS) ? DS : SS);
      }
      int stw = 0, imin = 0;
      if (N < kMinN || N > kMaxN) {
        stw = 1;
      } else {
        imin = (int)((long long)(f0 * T) - N / 2) - a.seg_qmin[seg];
        if (imin >= a.NFFT || imin + N <= 0) stw = 4;
      }
      s_st[l] = stw;
      s_N[l] = N;
      s_imin[l] = imin;
    } else if (w == 1) {
      const double cth = p[1], sth = sqrt(1.0 - cth * cth);
      double sph, cph;
      sincos(p[2], &sph, &cph);
      const double u[3] = {cth * cph, cth * sph, -sth}, v[3] = {sph, -cph, 0.};
      const double kx = -sth * cph, ky = -sth * sph;
      c->k[0] = (float)kx;
      c->k[1] = (float)ky;
      c->k[2] = (float)(-cth);
      c->k[3] = 0.f;
      c->kl[0] = (float)(kx - (double)c->k[0]);
      c->kl[1] = (float)(ky - (double)c->k[1]);
      c->kl[2] = (float)(-cth - (double)c->k[2]);
      int idx = 0;
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int q = r; q < 3; q++, idx++) {
          s_ep[l][idx] = v[r] * v[q] - u[r] * u[q];
          s_ec[l][idx] = u[r] * v[q] + v[r] * u[q];
        }
      const double bscale = kPI2 * f0 * (kAU / kCLIGHT);
      c->beta1 = df_from_double(bscale * kx);
      c->beta2 = df_from_double(bscale * ky);
    } else if (w == 2) {
      const double cosi = p[4];
      double sinps, cosps;
      sincos(2. * p[5], &sinps, &cosps);
      const double Aplus = (1. + cosi * cosi) * 0.5, Across = -cosi;
      s_dp[l][0] = Aplus * cosps;
      s_dp[l][1] = -Across * sinps;
      s_dp[l][2] = -Aplus * sinps;
      s_dp[l][3] = -Across * cosps;
      const double fdotT = p[7] / T;  // fdot T
      c->fonfs0 = (float)(f0 / a.fstar);
      c->fonfs0l = (float)(f0 / a.fstar - (double)c->fonfs0);
      c->fdfs = (float)(fdotT / a.fstar);
      c->fdfsl = (float)(fdotT / a.fstar - (double)c->fdfs);
      c->aef = (float)(0.66666666666666666666 * fdotT / f0);
      c->aefl = (float)(0.66666666666666666666 * fdotT / f0 - (double)c->aef);
      c->w0c = (float)(kPI2 * f0 / kCLIGHT);
      c->w0cl = (float)(kPI2 * f0 / kCLIGHT - (double)c->w0c);
      c->p7pi = (float)(kPI * p[7]);
    } else {
      s_amp[l] = exp(p[3]);
      const double fT = f0 * T;
      const long long q = (long long)fT;
      c->eps2pi = df_from_double(kPI2 * (fT - (double)q));
      c->phi0 = df_from_double(p[6]);
      c->p7pi_d = df_from_double(kPI * p[7]);
    }
  } else if (w == 0) {
    s_st[l] = st;
    s_N[l] = 0;
    s_imin[l] = 0;
  }
  __syncthreads();
  const int stt = in ? (st | s_st[l]) : 1;
  // amp/(2N) = m 2^e, m in [1, 2): the power of two scales the template
  // exactly in the likelihood kernels, m goes into the antenna tensors
  double msc = 1.0;
  if (in && !stt) {
    const double sc = scalbn(s_amp[l], -(32 - __clz(s_N[l])));  // amp / (2N), N a power of two
    const int ex = ilogb(sc);
    msc = scalbn(sc, -ex);
    if (w == 0) c->amp_p2 = (float)scalbn(1.0, ex);
  }
  // antenna tensors: warp w assembles elements 3w/2 .. of the 12 (Mr, Mi) x 6
  if (in && !stt) {
#pragma unroll
    for (int q = 0; q < 3; q++) {
      const int e = 3 * w + q;  // 0..11: (tensor element, real/imag)
      const int el = e >> 1;
      const double DPx = s_dp[l][(e & 1) ? 1 : 0], DCx = s_dp[l][(e & 1) ? 3 : 2];
      const double md = msc * (DPx * s_ep[l][el] + DCx * s_ec[l][el]);
      const float m = (float)md, ml = (float)(md - (double)m);
      if (e & 1) {
        c->Mi[el] = m;
        c->Mil[el] = ml;
      } else {
        c->Mr[el] = m;
        c->Mrl[el] = ml;
      }
    }
  }
  int b = -1;
  if (w == 0) {
    if (in && stt) {
      plan_write_skipped(a, i, stt);
    } else if (in) {
      const int N = s_N[l];
      c->seg = seg;
      c->N = N;
      c->imin = s_imin[l];
      c->pad = 0;
      const double sc = scalbn(s_amp[l], -(32 - __clz(N)));  // amp / (2N), N a power of two
      c->amp_hi = (float)sc;
      c->amp_lo = (float)(sc - (double)c->amp_hi);
      b = fd_bin_of(N);
    }
    plan_bin(a, i, b);
  }
}

// ------------------------------------------------------------ orbit tables
// One thread per (size, sample): analytic orbits of utils/src/glass_lisa.c:77-124
// at t = t0 + T (n-1)/N (ucb/src/glass_ucb_waveform.c:843), and the FFT
// twiddles exp(-2 pi i k / N).
__global__ void fd_orbit_table_kernel(FdTablesDev tab, double T, double t0) {
  int gid = blockIdx.x * blockDim.x + threadIdx.x;
  // sizes 32..4096 laid out back to back: offset of size b is 32 (2^b - 1)
  int b = 0;
  while (b < kNumBins && gid >= 32 * ((1 << (b + 1)) - 1)) b++;
  if (b >= kNumBins) return;
  int N = 32 << b;
  int n = gid - 32 * ((1 << b) - 1);
  double t = t0 + T * (double)n / (double)N;
  double alpha = kPI2 * t / kYEAR;
  double sa, ca;
  sincos(alpha, &sa, &ca);
  double ecc = kLARM / (2.0 * kSQ3 * kAU);
  double R = kAU * ecc;
  double sa2 = sa * sa, ca2 = ca * ca, saca = sa * ca, AUca = kAU * ca, AUsa = kAU * sa;
  const double sbs[3] = {0.0, 0.866025403784439, -0.866025403784438};
  const double cbs[3] = {1.0, -0.5, -0.5};
  OrbitSample64 o;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    double sb = sbs[i], cb = cbs[i];
    o.x[i] = AUca + R * (saca * sb - (1. + sa2) * cb);
    o.y[i] = AUsa + R * (saca * cb - (1. + ca2) * sb);
    o.z[i] = -kSQ3 * R * (ca * cb + sa * sb);
  }
  o.t = t;
  tab.pos64[b][n] = o;
  OrbitSampleMix m;
  df u = df_from_double(t / T), cd = df_from_double(ca), sd = df_from_double(sa);
  m.u_hi = u.hi;
  m.u_lo = u.lo;
  m.ca_hi = cd.hi;
  m.ca_lo = cd.lo;
  m.sa_hi = sd.hi;
  m.sa_lo = sd.lo;
  m.pad0 = m.pad1 = 0.f;
  tab.mix[b][n] = m;
  // mixed slow-part geometry: offsets from the guiding centre and arm monomials
  // (absent from tables built for the FP64 path alone)
  if (tab.geo[b]) {
    double v[28];
    double d[3][3];
    for (int i = 0; i < 3; i++) {
      d[i][0] = R * (saca * sbs[i] - (1. + sa2) * cbs[i]);
      d[i][1] = R * (saca * cbs[i] - (1. + ca2) * sbs[i]);
      d[i][2] = -kSQ3 * R * (ca * cbs[i] + sa * sbs[i]);
      for (int q = 0; q < 3; q++) v[3 * i + q] = d[i][q];
    }
    const int arm[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int a = 0; a < 3; a++) {
      double r[3];
      for (int q = 0; q < 3; q++) r[q] = (d[arm[a][1]][q] - d[arm[a][0]][q]) / kLARM;
      double *mo = v + 9 + 6 * a;
      mo[0] = r[0] * r[0];
      mo[1] = 2.0 * r[0] * r[1];
      mo[2] = 2.0 * r[0] * r[2];
      mo[3] = r[1] * r[1];
      mo[4] = 2.0 * r[1] * r[2];
      mo[5] = r[2] * r[2];
    }
    v[27] = 0.0;
    GeoSampleMix gm, gl;
    for (int q = 0; q < 28; q++) {
      gm.f[q] = (float)v[q];
      gl.f[q] = (float)(v[q] - (double)gm.f[q]);
    }
    tab.geo[b][n] = gm;
    if (tab.geolo[b]) tab.geolo[b][n] = gl;
  }
  double s, cth;
  sincospi(-2.0 * (double)n / (double)N, &s, &cth);
  tab.tw64[b][n] = make_double2(cth, s);
  tab.tw32[b][n] = make_float2((float)cth, (float)s);
  if (tab.tw32x[b]) {
    const float ch = (float)cth, sh = (float)s;
    tab.tw32x[b][n] = make_float4(ch, sh, (float)(cth - (double)ch), (float)(s - (double)sh));
  }
}

cudaError_t fd_build_orbit_tables(FdTablesDev &tab, double T, double t0, cudaStream_t stream) {
  if (!tab.base) {
    size_t total = 0;
    for (int b = 0; b < kNumBins; b++) {
      int N = 32 << b;
      total += (size_t)N * (sizeof(OrbitSample64) + sizeof(OrbitSampleMix) + 2 * sizeof(GeoSampleMix) +
                            sizeof(float2) + sizeof(double2) + sizeof(float4));
    }
    cudaError_t e = cudaMalloc(&tab.base, total);
    if (e != cudaSuccess) return e;
    char *p = (char *)tab.base;
    for (int b = 0; b < kNumBins; b++) {
      int N = 32 << b;
      tab.pos64[b] = (OrbitSample64 *)p;
      p += (size_t)N * sizeof(OrbitSample64);
      tab.mix[b] = (OrbitSampleMix *)p;
      p += (size_t)N * sizeof(OrbitSampleMix);
      tab.geo[b] = (GeoSampleMix *)p;
      p += (size_t)N * sizeof(GeoSampleMix);
      tab.geolo[b] = (GeoSampleMix *)p;
      p += (size_t)N * sizeof(GeoSampleMix);
      tab.tw64[b] = (double2 *)p;
      p += (size_t)N * sizeof(double2);
      tab.tw32[b] = (float2 *)p;
      p += (size_t)N * sizeof(float2);
      tab.tw32x[b] = (float4 *)p;
      p += (size_t)N * sizeof(float4);
    }
  }
  int total = 32 * ((1 << kNumBins) - 1);
  fd_orbit_table_kernel<<<(total + 255) / 256, 256, 0, stream>>>(tab, T, t0);
  return cudaGetLastError();
}

// ---------------------------------------------------------- host: bank tables
void fd_build_bank_tables(int format, double T, double fstar, int NFFT, int nseg, const int *qmin, const double *rA,
                          const double *rE, const double *invCA, const double *invCE, float4 *w32, float4 *w32lo,
                          float4 *g32, double *Q, double2 *w64, double2 *g64, double *QA, float4 *g32lo) {
  const double sqT = sqrt(T);
  for (int s = 0; s < nseg; s++) {
    double q = 0.0, qa = 0.0;
    Q[(size_t)s * (NFFT + 1)] = 0.0;
    if (QA) QA[(size_t)s * (NFFT + 1)] = 0.0;
    for (int j = 0; j < NFFT; j++) {
      size_t sj = (size_t)s * NFFT + j;
      double f = (double)(qmin[s] + j) / T;
      double x = f / fstar;
      double c1 = cos(x), s1 = sin(x);
      double c2 = 2. * c1 * c1 - 1.0, s2 = 2. * s1 * c1;
      double c3 = 2. * c1 * c2 - c1, s3 = 2. * s1 * c2 + s1;
      double pref, w2r, w2i, w1r, w1i;
      if (format == 0) {  // sangria: utils/src/glass_lisa.c:685-700
        pref = f * (4.0 / fstar * sqT) * s1;
        w2r = c2; w2i = -s2;
        w1r = c1; w1i = -s1;
      } else {  // phase (:480-530) / frequency (:574-630)
        pref = (format == 1) ? sqT : sqT * 2. * x;
        w2r = c3 - c1; w2i = -s3 + s1;
        w1r = c2 - 1.0; w1i = -s2;
      }
      double sA = sqrt(invCA[sj]), sE = sqrt(invCE[sj]);
      double ka = sA * kSQRT1_2 * pref, ke = sE * kINVSQ6 * pref;
      double GA2r = ka * w2r, GA2i = ka * w2i, GA1r = ka * w1r, GA1i = ka * w1i;
      double GE2r = ke * w2r, GE2i = ke * w2i, GE1r = ke * w1r, GE1i = ke * w1i;
      double conj = (format == 1) ? -1.0 : 1.0;  // "phase" conjugates A and E (:545-546)
      double wAr = rA[2 * sj] * sA, wAi = conj * rA[2 * sj + 1] * sA;
      double wEr = rE[2 * sj] * sE, wEi = conj * rE[2 * sj + 1] * sE;
      w64[2 * sj] = make_double2(wAr, wAi);
      w64[2 * sj + 1] = make_double2(wEr, wEi);
      g64[4 * sj + 0] = make_double2(GA2r, GA2i);
      g64[4 * sj + 1] = make_double2(GA1r, GA1i);
      g64[4 * sj + 2] = make_double2(GE2r, GE2i);
      g64[4 * sj + 3] = make_double2(GE1r, GE1i);
      // The whitened data of a loud source reach |w| ~ 50 in its bins; rounded
      // to float, their cross term with the template would carry ~1e-3 of
      // error into delta logL, so the residual is kept as a double-float pair.
      float4 wf = make_float4((float)wAr, (float)wAi, (float)wEr, (float)wEi);
      w32[sj] = wf;
      w32lo[sj] = make_float4((float)(wAr - (double)wf.x), (float)(wAi - (double)wf.y), (float)(wEr - (double)wf.z),
                              (float)(wEi - (double)wf.w));
      const float4 ga = make_float4((float)GA2r, (float)GA2i, (float)GA1r, (float)GA1i);
      const float4 ge = make_float4((float)GE2r, (float)GE2i, (float)GE1r, (float)GE1i);
      g32[2 * sj] = ga;
      g32[2 * sj + 1] = ge;
      // a template's power sits in a few bins, so the rounding of these
      // entries would not average out over its support: kept as hi + lo
      if (g32lo) {
        g32lo[2 * sj] = make_float4((float)(GA2r - (double)ga.x), (float)(GA2i - (double)ga.y),
                                    (float)(GA1r - (double)ga.z), (float)(GA1i - (double)ga.w));
        g32lo[2 * sj + 1] = make_float4((float)(GE2r - (double)ge.x), (float)(GE2i - (double)ge.y),
                                        (float)(GE1r - (double)ge.z), (float)(GE1i - (double)ge.w));
      }
      q += wAr * wAr + wAi * wAi + wEr * wEr + wEi * wEi;
      Q[(size_t)s * (NFFT + 1) + j + 1] = q;
      if (QA) {
        qa += wAr * wAr + wAi * wAi;
        QA[(size_t)s * (NFFT + 1) + j + 1] = qa;
      }
    }
  }
}

// --------------------------------------------------------------- launchers
cudaError_t fd_dlogl_launch(const FdBankDev &bank, const FdTablesDev &tab, FdWorkDev &work, int precision,
                            int nitems, const int *item_seg, const double *params, const double *term_x,
                            double *dlogl, double *term_y, double *hh, int *status, int n_fixed, int num_sms,
                            cudaStream_t stream, int *nlaunch, double *term_ch) {
  cudaError_t e;
  int launches = 0;
  const bool mix = precision == 1;
  if (!work.counts_zero) {
    e = cudaMemsetAsync(work.bin_count, 0, sizeof(int) * kFdCounts, stream);
    if (e != cudaSuccess) return e;
  }
  const bool fallback = mix && (work.fb_e1 > 0.f || work.fb_e2 > 0.f) && work.series2 != nullptr;
  work.counts_zero = false;  // until this sequence has been enqueued in full
  PlanArgs pa;
  pa.nitems = nitems;
  pa.nseg = bank.nseg;
  pa.NFFT = bank.NFFT;
  pa.cap = work.cap;
  pa.precision = precision;
  pa.n_fixed = n_fixed;
  pa.T = bank.T;
  pa.fstar = bank.fstar;
  pa.L = kLARM;
  pa.item_seg = item_seg;
  pa.params = params;
  pa.term_x = term_x;
  pa.seg_qmin = bank.qmin;
  pa.items64 = work.items64;
  pa.itemsmix = work.itemsmix;
  pa.bin_count = work.bin_count;
  pa.bin_list = work.bin_list;
  pa.dlogl = dlogl;
  pa.term_y = term_y;
  pa.hh = hh;
  pa.status = status;
  const bool timing = work.phase_timing;
  work.phase_recorded = false;
  if (timing && (e = cudaEventRecord(work.phase[0], stream)) != cudaSuccess) return e;
  {
    int per = (nitems + num_sms - 1) / (num_sms > 0 ? num_sms : 1);
    pa.per_cta = per < 16 ? 16 : (per > 32 ? 32 : per);
    if (work.tune.plan_per_cta >= 8 && work.tune.plan_per_cta <= 32) pa.per_cta = work.tune.plan_per_cta;
  }
  if (mix)
    fd_planmix_kernel<<<(nitems + pa.per_cta - 1) / pa.per_cta, 128, 0, stream>>>(pa);
  else
    fd_plan64_kernel<<<(nitems + 63) / 64, 64, 0, stream>>>(pa);
  launches++;
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (timing && (e = cudaEventRecord(work.phase[1], stream)) != cudaSuccess) return e;

  SlowArgs sa;
  sa.cap = work.cap;
  sa.NFFT = bank.NFFT;
  sa.fstar = bank.fstar;
  sa.L = kLARM;
  sa.Rf = (float)(kAU * (kLARM / (2.0 * kSQ3 * kAU)));
  sa.invLf = (float)(1.0 / kLARM);
  sa.AUcf = (float)(kAU / kCLIGHT);
  sa.invTf = (float)(1.0 / bank.T);
  sa.bin_count = work.bin_count;
  sa.bin_list = work.bin_list;
  sa.items64 = work.items64;
  sa.itemsmix = work.itemsmix;
  for (int b = 0; b < kNumBins; b++) {
    sa.pos64[b] = tab.pos64[b];
    sa.mix[b] = tab.mix[b];
    sa.geo[b] = tab.geo[b];
  }
  sa.series = work.series;
  sa.nitems = nitems;
  sa.series_len = (long long)(work.series_bytes / (mix ? sizeof(float2) : sizeof(double2)));
  e = mix ? fd_launch_slow_mixed(sa, num_sms, stream, work.tune.slow_block, work.tune.slow_ctas_per_sm)
          : fd_launch_slow_fp64(sa, num_sms, stream);
  launches++;
  if (e != cudaSuccess) return e;
  if (timing && (e = cudaEventRecord(work.phase[2], stream)) != cudaSuccess) return e;

  SpecArgs a;
  a.NFFT = bank.NFFT;
  a.cap = work.cap;
  a.bin_count = work.bin_count;
  a.items64 = work.items64;
  a.itemsmix = work.itemsmix;
  a.series = work.series;
  a.nitems = nitems;
  a.nseg = bank.nseg;
  a.series_len = sa.series_len;
  a.w32 = bank.w32;
  a.w32lo = bank.w32lo;
  a.g32 = bank.g32;
  a.g32lo = bank.g32lo;
  a.Q = bank.Q;
  a.w64 = bank.w64;
  a.g64 = bank.g64;
  a.term_x = term_x;
  a.dlogl = dlogl;
  a.term_y = term_y;
  a.hh = hh;
  a.status = status;
  a.term_ch = term_ch;
  a.QA = bank.QA;
  if (fallback) {
    a.fb_count = work.fb_count;
    a.hp_count = work.hp_count;
    a.hp_list = work.hp_list;
    a.fb_total = work.fb_total;
    a.fb_e1 = work.fb_e1;
    a.fb_e2 = work.fb_e2;
    a.fb_inv_scale = work.fb_inv_scale;
    a.fb_nscale = work.fb_nscale;
  }
  const bool perch = term_ch != nullptr;
  // Inside a CUDA-graph capture, the re-evaluation (three launches, idle in
  // batches with nothing listed) sits behind a conditional node that a
  // one-thread kernel sets when something is listed; outside capture, or
  // where the graph API refuses, it is launched unconditionally.
  bool cond = false;
  cudaGraphConditionalHandle cond_h = 0;
  cudaGraph_t cap_graph = nullptr;
  if (fallback) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamGetCaptureInfo(stream, &cs, nullptr, &cap_graph) == cudaSuccess &&
        cs == cudaStreamCaptureStatusActive &&
        cudaGraphConditionalHandleCreate(&cond_h, cap_graph, 0, cudaGraphCondAssignDefault) == cudaSuccess)
      cond = true;
    (void)cudaGetLastError();
  }
  // sizes up to 1024 (every size a segment of NFFT bins can produce, up to
  // NFFT: ucb_bandwidth caps N there) in one launch on the main stream; 2048
  // and 4096 as their own kernels on side streams running beside it
  int nall = 0;
  while (nall < kSpecAllBins && (32 << nall) <= bank.NFFT) nall++;
  int nb = 0;
  if (bank.NFFT > 1024) {
    if ((e = cudaEventRecord(work.fork, stream)) != cudaSuccess) return e;
    for (int b = kSpecAllBins; b < kNumBins; b++) {
      int N = 32 << b;
      if (N > bank.NFFT) break;
      cudaStream_t sb = work.side[b];
      if ((e = cudaStreamWaitEvent(sb, work.fork, 0)) != cudaSuccess) return e;
      a.bin = b;
      a.bin_list = work.bin_list + (size_t)b * work.cap;
      a.tw = mix ? (const void *)tab.tw32x[b] : (const void *)tab.tw64[b];
      e = mix ? fd_launch_spec_mixed(N, a, nitems, num_sms, sb, perch)
              : fd_launch_spec_fp64(N, a, nitems, num_sms, sb, perch);
      launches++;
      if (e != cudaSuccess) return e;
      if ((e = cudaEventRecord(work.join[b], sb)) != cudaSuccess) return e;
      nb++;
    }
  }
  if (nall > 0) {
    SpecAllArgs A;
    A.a = a;
    A.a.bin = 0;
    A.a.bin_list = work.bin_list;
    A.a.tw = nullptr;
    A.nbins = nall;
    A.zero_counts = nb == 0 ? work.bin_count : nullptr;  // side kernels would still be reading them
    A.done = work.bin_count + kNumBins + 1;  // fb_count is at kNumBins
    for (int b = 0; b < kSpecAllBins; b++) A.tw[b] = mix ? (const void *)tab.tw32x[b] : (const void *)tab.tw64[b];
    e = mix ? fd_launch_spec_all_mixed(A, num_sms, stream, perch, work.tune.spec_ctas_per_sm)
            : fd_launch_spec_all_fp64(A, num_sms, stream, perch);
    launches++;
    if (e != cudaSuccess) return e;
  }
  for (int b = kSpecAllBins; b < kSpecAllBins + nb; b++)
    if ((e = cudaStreamWaitEvent(stream, work.join[b], 0)) != cudaSuccess) return e;
  if (nb > 0 || nall == 0) {  // the size counts only: fb_count follows them
    if ((e = cudaMemsetAsync(work.bin_count, 0, sizeof(int) * kNumBins, stream)) != cudaSuccess) return e;
  }
  if (timing && (e = cudaEventRecord(work.phase[3], stream)) != cudaSuccess) return e;

  // Re-evaluation of the listed mixed proposals in double-float: series
  // (into series2), spectral stage, results written over the mixed ones; the
  // re-evaluation's counts and fb_count end at zero.
  if (fallback) {
    int nmax = kMaxN;
    while (nmax > bank.NFFT) nmax >>= 1;
    SlowArgs sh = sa;
    sh.bin_count = work.hp_count;
    sh.bin_list = work.hp_list;
    sh.series = work.series2;
    sh.series_len = (long long)(work.series_bytes / sizeof(float4));
    for (int b = 0; b < kNumBins; b++) sh.geolo[b] = tab.geolo[b];
    sh.invLd = df_from_double(1.0 / kLARM);
    sh.AUcd = df_from_double(kAU / kCLIGHT);
    sh.invTd = df_from_double(1.0 / bank.T);
    sh.invcd = df_from_double(1.0 / kCLIGHT);
    HpArgs h;
    h.NFFT = bank.NFFT;
    h.cap = work.cap;
    h.nitems = nitems;
    h.nseg = bank.nseg;
    h.series_len = sh.series_len;
    h.nmax = nmax;
    h.bin_count = work.hp_count;
    h.bin_list = work.hp_list;
    h.itemsmix = work.itemsmix;
    h.series = reinterpret_cast<const float4 *>(work.series2);
    h.zero_at = work.fb_count;  // fb_count, the done counters, the spares and hp_count
    h.nzero = kFdCounts - kNumBins;
    h.done = work.bin_count + kNumBins + 2;
    h.w32 = bank.w32;
    h.w32lo = bank.w32lo;
    h.g32 = bank.g32;
    h.g32lo = bank.g32lo;
    h.Q = bank.Q;
    h.QA = bank.QA;
    for (int b = 0; b < kNumBins; b++) h.tw32x[b] = tab.tw32x[b];
    h.term_x = term_x;
    h.dlogl = dlogl;
    h.term_y = term_y;
    h.hh = hh;
    h.term_ch = term_ch;
    h.status = status;
    cudaStream_t ts = stream;
    cudaGraphNode_t cnode = nullptr;
    if (cond) {
      fd_cond_kernel<<<1, 32, 0, stream>>>(work.fb_count, cond_h);
      launches++;
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      const cudaGraphNode_t *deps = nullptr;
      size_t nd = 0;
      cudaStreamCaptureStatus cs;
      cudaGraphNodeParams np = {};
      np.type = cudaGraphNodeTypeConditional;
      np.conditional.handle = cond_h;
      np.conditional.type = cudaGraphCondTypeIf;
      np.conditional.size = 1;
      if ((e = cudaStreamGetCaptureInfo(stream, &cs, nullptr, nullptr, &deps, nullptr, &nd)) != cudaSuccess) return e;
      if ((e = cudaGraphAddNode(&cnode, cap_graph, deps, nullptr, nd, &np)) != cudaSuccess) return e;
      ts = work.side[0];
      if ((e = cudaStreamBeginCaptureToGraph(ts, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                             cudaStreamCaptureModeRelaxed)) != cudaSuccess)
        return e;
    }
    e = fd_launch_reeval(sh, h, perch, num_sms, ts, &launches);
    if (e != cudaSuccess) return e;
    if (cond) {
      cudaGraph_t body = nullptr;
      if ((e = cudaStreamEndCapture(ts, &body)) != cudaSuccess) return e;
      if ((e = cudaStreamUpdateCaptureDependencies(stream, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies)) !=
          cudaSuccess)
        return e;
    }
  }
  work.counts_zero = true;
  if (timing) {
    if ((e = cudaEventRecord(work.phase[4], stream)) != cudaSuccess) return e;
    work.phase_recorded = true;
  }
  if (nlaunch) *nlaunch = launches;
  return cudaSuccess;
}

cudaError_t fd_launch_plan64(const PlanArgs &a, cudaStream_t stream) {
  fd_plan64_kernel<<<(a.nitems + 63) / 64, 64, 0, stream>>>(a);
  return cudaGetLastError();
}

size_t fd_series_bytes(int nitems, int NFFT, int precision) {
  size_t elem = precision == 1 ? sizeof(float2) : sizeof(double2);
  return (size_t)nitems * (size_t)NFFT * 4 * elem;
}

// ------------------------------------------------------- legacy single waveform
// The drop-in ucb_waveform for one source: the per-source constants come from
// the host (source_geometry / make_item_f64, the same FP64 code); the six arm
// responses are computed one thread per sample spread over N/32 CTAs (the
// FP64 pipe of many SMs, not one); then one CTA per Michelson channel (X, Y,
// Z) FFTs its two series and applies the format's TDI weights per bin.  A and
// E follow in fd_ae_kernel from the stored X, Y, Z (utils/src/glass_lisa.c:429-441).
__global__ void fd_single_slow_kernel(const OrbitSample64 *pos, const ItemF64 *item, int N, double fstar, double L,
                                      double2 *d6) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  double2 d[6];
  slow_sample64(*item, pos[n], fstar, L, d);
#pragma unroll
  for (int a = 0; a < 6; a++) d6[(size_t)a * N + n] = d[a];
}

template <int N>
struct LegacyCfg {
  static constexpr int R = (N <= 128) ? 4 : 8;  // bins per thread
  static constexpr int GT = N / R;              // threads (one CTA per channel)
};

template <int N>
__global__ void __launch_bounds__(LegacyCfg<N>::GT) fd_waveform_kernel(const ItemF64 *item, const double2 *d6,
                                                                    int format, double T, double fstar,
                                                                    double *out, const double2 *twg) {
  constexpr int GT = LegacyCfg<N>::GT, R = LegacyCfg<N>::R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *tw = reinterpret_cast<double2 *>(smem_raw);
  double2 *buf = tw + N;
  const int lane = threadIdx.x, ch = blockIdx.x;
  for (int i = lane; i < N; i += GT) tw[i] = twg[i];
  // d: 12, 13, 21, 23, 31, 32 ; X: (12-13, 21-31), Y: (23-21, 32-12), Z: (31-32, 13-23)
  const int ua = ch == 0 ? 0 : ch == 1 ? 3 : 4, ub = ch == 0 ? 1 : ch == 1 ? 2 : 5;
  const int va = ch == 0 ? 2 : ch == 1 ? 5 : 1, vb = ch == 0 ? 4 : ch == 1 ? 0 : 3;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int n = lane + GT * r;
    buf[n] = csub(d6[(size_t)ua * N + n], d6[(size_t)ub * N + n]);
    buf[N + n] = csub(d6[(size_t)va * N + n], d6[(size_t)vb * N + n]);
  }
  __syncthreads();
  group_fft<N, GT, 2, 1, double2, 64>(buf, tw, lane);  // CTA barrier: the CTA may be a partial warp
  const double sqT = sqrt(T);
  const long long q = (long long)(item->f0 * T);
  const double amp_s = item->amp_s;
  double *X = out + (size_t)ch * 2 * N;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int k = lane + GT * r;
    const int m = (k + N / 2) & (N - 1);
    double f = (double)(q + m - N / 2) / T;
    double x = f / fstar;
    double s1, c1;
    sincos(x, &s1, &c1);
    double c2 = 2. * c1 * c1 - 1.0, s2 = 2. * s1 * c1;
    double2 W2, W1;
    double pref;
    if (format == 0) {
      pref = f * (4.0 / fstar * sqT) * s1;
      W2 = make_double2(c2, -s2);
      W1 = make_double2(c1, -s1);
    } else {
      double c3 = 2. * c1 * c2 - c1, s3 = 2. * s1 * c2 + s1;
      pref = (format == 1) ? sqT : sqT * 2. * x;
      W2 = make_double2(c3 - c1, -s3 + s1);
      W1 = make_double2(c2 - 1.0, -s2);
    }
    double2 h = cadd(cmul(buf[k], W2), cmul(buf[N + k], W1));
    double sc = amp_s * pref;
    X[2 * m] = h.x * sc;
    X[2 * m + 1] = h.y * sc;
  }
}

__global__ void fd_ae_kernel(double *out, int N, int format) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= 2 * N) return;
  const double *X = out, *Y = out + 2 * N, *Z = out + 4 * N;
  double *A = out + 6 * N, *E = out + 8 * N;
  double a = (Z[m] - X[m]) * kSQRT1_2;
  double e = (X[m] - 2 * Y[m] + Z[m]) * kINVSQ6;
  if (format == 1 && (m & 1)) {
    a = -a;
    e = -e;
  }
  A[m] = a;
  E[m] = e;
}

template <int N>
static cudaError_t launch_waveform(const ItemF64 *item, const double2 *d6, int format, int nch, double T, double fstar,
                                   double *out, const double2 *tw, cudaStream_t stream) {
  size_t smem = sizeof(double2) * 3 * N;
  static LaunchSetup setup;
  int occ = 0;
  cudaError_t e = launch_setup(setup, [&](int *o) {
    *o = 1;
    return cudaFuncSetAttribute(fd_waveform_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }, &occ);
  if (e != cudaSuccess) return e;
  fd_waveform_kernel<N><<<nch, LegacyCfg<N>::GT, smem, stream>>>(item, d6, format, T, fstar, out, tw);
  return cudaGetLastError();
}

cudaError_t fd_waveform_launch(const OrbitSample64 *pos, const ItemF64 *item, int N, int format, int NI, double T,
                               double fstar, double2 *d6, double *out, const double2 *tw, cudaStream_t stream) {
  int nch = (format != 0 && NI <= 1) ? 1 : 3;
  fd_single_slow_kernel<<<(N + 31) / 32, 32, 0, stream>>>(pos, item, N, fstar, kLARM, d6);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaErrorInvalidValue;
  switch (N) {
#define GLASS_WCASE(NN) \
  case NN:              \
    e = launch_waveform<NN>(item, d6, format, nch, T, fstar, out, tw, stream); \
    break;
    GLASS_WCASE(32)
    GLASS_WCASE(64)
    GLASS_WCASE(128)
    GLASS_WCASE(256)
    GLASS_WCASE(512)
    GLASS_WCASE(1024)
    GLASS_WCASE(2048)
    GLASS_WCASE(4096)
#undef GLASS_WCASE
  }
  if (e != cudaSuccess) return e;
  if (nch == 3) {
    fd_ae_kernel<<<(2 * N + 127) / 128, 128, 0, stream>>>(out, N, format);
    e = cudaGetLastError();
  }
  return e;
}

}  // namespace glass
