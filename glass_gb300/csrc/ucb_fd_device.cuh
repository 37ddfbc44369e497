// Device building blocks of the Fourier-domain UCB kernels (included by the
// ucb_fd*.cu translation units).
#pragma once
#include <math.h>
#include <stdio.h>

#include <type_traits>

#include "ucb_fd.cuh"

namespace glass {

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

__host__ __device__ constexpr int fd_bin_of(int N) {
  return N == 32 ? 0 : N == 64 ? 1 : N == 128 ? 2 : N == 256 ? 3 : N == 512 ? 4 : N == 1024 ? 5 : N == 2048 ? 6 : 7;
}

// --------------------------------------------------------------- complex helpers
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
// multiply by -i
__device__ __forceinline__ float2 cmi(float2 a) { return make_float2(a.y, -a.x); }
__device__ __forceinline__ double2 cmi(double2 a) { return make_double2(a.y, -a.x); }
template <typename C>
__device__ __forceinline__ C cscale(C a, decltype(a.x) s) {
  C r;
  r.x = a.x * s;
  r.y = a.y * s;
  return r;
}

// ------------------------------------------------------------- group barrier
// Groups of at most 32 threads live inside full warps of a larger CTA and
// synchronise with __syncwarp; larger groups are the whole CTA.
template <int GT>
__device__ __forceinline__ void group_sync() {
  if constexpr (GT <= 32) {
    __syncwarp();
  } else {
    __syncthreads();
  }
}

// ----------------------------------------------------------------------- FFT
// In-place forward DFT (exp(-2 pi i k n / N), unnormalised) of NSER series of
// length N held series-major in shared memory, by a group of GT threads.
// Radix-4 Stockham stages (plus one radix-2 stage when log2 N is odd): stage
// with sub-transform size p reads x[i + m N/R], applies exp(-2 pi i m k/(pR)),
// k = i mod p, and writes y[(i-k)R + k + m p].  Every thread holds its
// butterflies' inputs in registers between the two barriers of a stage, which
// lets the stage overwrite its own input.  CH series are processed per round to
// bound register use; rounds touch disjoint series, so a round's loads need no
// barrier after the previous round's stores, only one at the end of the stage.
template <int N, int GT, int NSER, int CH, typename C, int SYNC_GT = GT>
__device__ __forceinline__ void group_fft(C *buf, const C *tw, int lane) {
  constexpr int LOG = ilog2c(N);
  constexpr int NR4 = LOG / 2;
  constexpr int B4 = N / 4 / GT;
  static_assert(B4 >= 1, "group too large for radix-4 stages");
  int p = 1;
#pragma unroll
  for (int st = 0; st < NR4; ++st) {
    const int step = N / (4 * p);
    // the thread's butterfly twiddles, shared by every series (all 1 in the
    // first stage)
    C w[B4][3];
    if (st > 0) {
#pragma unroll
      for (int b = 0; b < B4; ++b) {
        const int k = (lane + GT * b) & (p - 1);
        w[b][0] = tw[k * step];
        w[b][1] = tw[2 * k * step];
        w[b][2] = tw[3 * k * step];
      }
    }
#pragma unroll
    for (int c0 = 0; c0 < NSER; c0 += CH) {
      C v[CH][B4][4];
#pragma unroll
      for (int s = 0; s < CH; ++s)
#pragma unroll
        for (int b = 0; b < B4; ++b) {
          int i = lane + GT * b;
#pragma unroll
          for (int m = 0; m < 4; ++m) v[s][b][m] = buf[(c0 + s) * N + i + m * (N / 4)];
        }
      group_sync<SYNC_GT>();
#pragma unroll
      for (int s = 0; s < CH; ++s)
#pragma unroll
        for (int b = 0; b < B4; ++b) {
          int i = lane + GT * b;
          int k = i & (p - 1);
          C u0 = v[s][b][0];
          C u1 = st > 0 ? cmul(v[s][b][1], w[b][0]) : v[s][b][1];
          C u2 = st > 0 ? cmul(v[s][b][2], w[b][1]) : v[s][b][2];
          C u3 = st > 0 ? cmul(v[s][b][3], w[b][2]) : v[s][b][3];
          C a = cadd(u0, u2), bb = csub(u0, u2), c = cadd(u1, u3), d = cmi(csub(u1, u3));
          int j = (i - k) * 4 + k;
          C *o = buf + (c0 + s) * N + j;
          o[0] = cadd(a, c);
          o[p] = cadd(bb, d);
          o[2 * p] = csub(a, c);
          o[3 * p] = csub(bb, d);
        }
    }
    group_sync<SYNC_GT>();
    p *= 4;
  }
  if constexpr (LOG & 1) {
    constexpr int B2 = N / 2 / GT;
    const int step = N / (2 * p);
    C w[B2];
#pragma unroll
    for (int b = 0; b < B2; ++b) w[b] = tw[((lane + GT * b) & (p - 1)) * step];
#pragma unroll
    for (int c0 = 0; c0 < NSER; c0 += CH) {
      C v[CH][B2][2];
#pragma unroll
      for (int s = 0; s < CH; ++s)
#pragma unroll
        for (int b = 0; b < B2; ++b) {
          int i = lane + GT * b;
          v[s][b][0] = buf[(c0 + s) * N + i];
          v[s][b][1] = buf[(c0 + s) * N + i + N / 2];
        }
      group_sync<SYNC_GT>();
#pragma unroll
      for (int s = 0; s < CH; ++s)
#pragma unroll
        for (int b = 0; b < B2; ++b) {
          int i = lane + GT * b;
          int k = i & (p - 1);
          C u1 = cmul(v[s][b][1], w[b]);
          int j = (i - k) * 2 + k;
          buf[(c0 + s) * N + j] = cadd(v[s][b][0], u1);
          buf[(c0 + s) * N + j + p] = csub(v[s][b][0], u1);
        }
    }
    group_sync<SYNC_GT>();
  }
}

// ---------------------------------------------------- register-resident FFT
// Shared-memory index of point e of a series whose rows of 16 points are
// padded to 17: the strided accesses of the stages below then fall on
// distinct banks.
__host__ __device__ constexpr int pad16(int e) { return e + (e >> 4); }

// v * exp(-2 pi i J / 16) for a compile-time J.
//
// The rotations must not change |v| on average: a template's power sits in a
// few output bins, so a gain error common to every use of a constant becomes
// a relative error of (h|h), which delta logL carries times (h|h) (1e-7 of a
// template power of 1e6 is 0.1).  Rounded to floats, cos and sin of pi/8 give
// |w|^2 - 1 = -5.7e-8 and those of pi/4 -3.4e-8: a gain of -2.3e-8 in every
// 16-point pass.  So each constant is a hi + lo pair of floats and a product
// takes two fused multiply-adds per term; only the two main products round.
template <int J>
__device__ __forceinline__ float2 w16mul(float2 v) {
  constexpr int j = J & 15;
  if constexpr (j == 0) {
    return v;
  } else if constexpr (j == 4) {
    return cmi(v);
  } else if constexpr (j == 8) {
    return make_float2(-v.x, -v.y);
  } else if constexpr (j == 12) {
    return make_float2(-v.y, v.x);
  } else {
    // cos(k pi/8) = hi + lo: 1, cos(pi/8), sqrt(1/2), sin(pi/8), 0, ...
    constexpr float Ch = 0.9238795042037964f, Cl = 2.830748968563057e-08f;
    constexpr float Kh = 0.7071067690849304f, Kl = 1.2101617485882343e-08f;
    constexpr float Sh = 0.3826834261417389f, Sl = 6.2233507236442165e-09f;
    constexpr float hi[16] = {1.f, Ch, Kh, Sh, 0.f, -Sh, -Kh, -Ch, -1.f, -Ch, -Kh, -Sh, 0.f, Sh, Kh, Ch};
    constexpr float lo[16] = {0.f, Cl, Kl, Sl, 0.f, -Sl, -Kl, -Cl, 0.f, -Cl, -Kl, -Sl, 0.f, Sl, Kl, Cl};
    constexpr int js = (j + 12) & 15;  // sin x = cos(x - pi/2)
    constexpr float c = hi[j], cl = lo[j], s = hi[js], sl = lo[js];
    // (x c + y s, y c - x s)
    return make_float2(fmaf(v.x, c, fmaf(v.y, s, fmaf(v.x, cl, v.y * sl))),
                       fmaf(v.y, c, fmaf(-v.x, s, fmaf(v.y, cl, -(v.x * sl)))));
  }
}

__device__ __forceinline__ void dft4_inplace(float2 &v0, float2 &v1, float2 &v2, float2 &v3) {
  const float2 a = cadd(v0, v2), b = csub(v0, v2), c = cadd(v1, v3), d = cmi(csub(v1, v3));
  v0 = cadd(a, c);
  v1 = cadd(b, d);
  v2 = csub(a, c);
  v3 = csub(b, d);
}

// Forward DFT of R = 2, 4, 8 or 16 points in registers, natural order out.
// R = R1 R2 is split as m = m1 + R1 m2, k = k2 + R2 k1: R1 DFTs of R2 points,
// twiddles exp(-2 pi i m1 k2 / R), R2 DFTs of R1 points.
template <int R>
__device__ __forceinline__ void dft_reg(float2 *v) {
  if constexpr (R == 2) {
    const float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if constexpr (R == 4) {
    dft4_inplace(v[0], v[1], v[2], v[3]);
  } else if constexpr (R == 8) {
    dft4_inplace(v[0], v[2], v[4], v[6]);
    dft4_inplace(v[1], v[3], v[5], v[7]);
    v[3] = w16mul<2>(v[3]);
    v[5] = w16mul<4>(v[5]);
    v[7] = w16mul<6>(v[7]);
    float2 o[8];
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) {
      o[k2] = cadd(v[2 * k2], v[2 * k2 + 1]);
      o[k2 + 4] = csub(v[2 * k2], v[2 * k2 + 1]);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = o[q];
  } else {
    static_assert(R == 16, "radix");
#pragma unroll
    for (int m1 = 0; m1 < 4; ++m1) dft4_inplace(v[m1], v[m1 + 4], v[m1 + 8], v[m1 + 12]);
    // v[m1 + 4 k2] *= w16^(m1 k2)
    v[5] = w16mul<1>(v[5]);
    v[6] = w16mul<2>(v[6]);
    v[7] = w16mul<3>(v[7]);
    v[9] = w16mul<2>(v[9]);
    v[10] = w16mul<4>(v[10]);
    v[11] = w16mul<6>(v[11]);
    v[13] = w16mul<3>(v[13]);
    v[14] = w16mul<6>(v[14]);
    v[15] = w16mul<9>(v[15]);
    float2 o[16];
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) {
      float2 a0 = v[4 * k2], a1 = v[4 * k2 + 1], a2 = v[4 * k2 + 2], a3 = v[4 * k2 + 3];
      dft4_inplace(a0, a1, a2, a3);
      o[k2] = a0;
      o[k2 + 4] = a1;
      o[k2 + 8] = a2;
      o[k2 + 12] = a3;
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = o[q];
  }
}

// Twiddle products of the register FFT: a float2 twiddle, or a float4
// holding a twiddle as hi + lo floats (x, y: hi; z, w: lo), whose product
// rounds only at its two main terms.  In a loud narrowband template the few
// twiddles on its bins' paths set an error common to the template.
__device__ __forceinline__ float2 twmul(float2 v, float2 t) { return cmul(v, t); }
__device__ __forceinline__ float2 twmul(float2 v, float4 t) {
  return make_float2(fmaf(v.x, t.x, fmaf(-v.y, t.y, fmaf(v.x, t.z, -(v.y * t.w)))),
                     fmaf(v.x, t.y, fmaf(v.y, t.x, fmaf(v.x, t.w, v.y * t.z))));
}

// One Stockham stage of radix R and sub-transform size P on a padded series
// y of length N, by the M = N/16 threads of the series (thread t does the
// 16/R butterflies i = t + M b): reads x[i + m N/R], multiplies by
// exp(-2 pi i m k / (P R)), k = i mod P, and writes y[(i - k) R + k + q P].
// tw: exp(-2 pi i j / N) at pad16(j) (float2, or float4 as hi + lo).
template <int N, int R, int P, typename TW>
__device__ __forceinline__ void reg_stage_load(const float2 *y, const TW *tw, int t, float2 *v) {
  constexpr int M = N / 16, NB = 16 / R, STRIDE = N / R, TS = N / (P * R);
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const int i = t + M * b, k = i & (P - 1);
#pragma unroll
    for (int m = 0; m < R; ++m) {
      float2 val = y[pad16(i + m * STRIDE)];
      if (P > 1 && m > 0) val = twmul(val, tw[pad16(m * k * TS)]);
      v[b * R + m] = val;
    }
  }
}
template <int N, int R, int P>
__device__ __forceinline__ void reg_stage_store(float2 *y, int t, float2 *v) {
  constexpr int M = N / 16, NB = 16 / R;
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    dft_reg<R>(v + b * R);
    const int i = t + M * b, k = i & (P - 1);
#pragma unroll
    for (int q = 0; q < R; ++q) y[pad16((i - k) * R + k + q * P)] = v[b * R + q];
  }
}
template <int N, int GT, int R, int P, typename TW>
__device__ __forceinline__ void reg_stage(float2 *y, const TW *tw, int t, float2 *v) {
  reg_stage_load<N, R, P>(y, tw, t, v);
  group_sync<GT>();  // every read of the stage before the in-place writes
  reg_stage_store<N, R, P>(y, t, v);
  group_sync<GT>();
}

// One stage of fft_reg_smem over NSER series in rounds of GT/M (one series
// per M threads): rounds touch disjoint series, so a round's loads need no
// barrier after the previous round's stores, only one before its own stores.
template <int N, int GT, int NSER, int R, int P, typename TW>
__device__ __forceinline__ void reg_stage_rounds(float2 *sbuf, const TW *tw, int s, int t, float2 *v) {
  constexpr int SN = pad16(N), SPR = GT / (N / 16);
#pragma unroll 1
  for (int r = 0; r < NSER / SPR; ++r) {
    float2 *y = sbuf + (SPR * r + s) * SN;
    reg_stage_load<N, R, P>(y, tw, t, v);
    group_sync<GT>();
    reg_stage_store<N, R, P>(y, t, v);
  }
  group_sync<GT>();
}

// As fft4_reg for NSER series already in the padded shared-memory layout
// (series stride pad16(N)), transformed in place by GT threads: GT/M series
// at a time (a multiple of 4 dividing NSER).
template <int N, int GT, int NSER, typename TW>
__device__ __forceinline__ void fft_reg_smem(float2 *sbuf, const TW *tw, int lane) {
  constexpr int M = N / 16;
  static_assert(GT % (4 * M) == 0 && NSER % (GT / M) == 0 && N >= 32 && N <= 4096, "fft_reg_smem shape");
  const int s = lane / M, t = lane - (lane / M) * M;
  float2 v[16];
  reg_stage_rounds<N, GT, NSER, 16, 1>(sbuf, tw, s, t, v);
  if constexpr (M >= 16) {
    reg_stage_rounds<N, GT, NSER, 16, 16>(sbuf, tw, s, t, v);
    if constexpr (N / 256 > 1) reg_stage_rounds<N, GT, NSER, N / 256, 256>(sbuf, tw, s, t, v);
  } else {
    reg_stage_rounds<N, GT, NSER, M, 16>(sbuf, tw, s, t, v);
  }
}

// Forward DFT (exp(-2 pi i k n / N), unnormalised) of the 4 series of one
// proposal, N = 16 M with 32 <= N <= 4096, by a group of GT = 4 M threads:
// series s = lane / M, thread t = lane % M holds 16 points in registers.
// Stockham stages of radix 16 (a 4 x 4 split in registers) and one final stage
// of the remaining radix: 2 stages for N <= 256, 3 up to 4096 (the radix-4
// version, group_fft, needs log4 N).  The first stage reads the series from
// global memory (src, 4 series of N back to back); every stage writes the
// padded shared-memory series sbuf (stride pad16(N)), natural order at the end.
template <int N, int GT, typename TW>
__device__ __forceinline__ void fft4_reg(const float2 *src, float2 *sbuf, const TW *tw, int lane) {
  constexpr int M = N / 16, SN = pad16(N);
  static_assert(4 * M == GT && N >= 32 && N <= 4096, "fft4_reg shape");
  const int s = lane / M, t = lane - (lane / M) * M;
  const float2 *x = src + (size_t)s * N;
  float2 *y = sbuf + s * SN;
  float2 v[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) v[m] = x[t + m * M];
  dft_reg<16>(v);
#pragma unroll
  for (int q = 0; q < 16; ++q) y[pad16(t * 16 + q)] = v[q];
  group_sync<GT>();
  if constexpr (M >= 16) {
    reg_stage<N, GT, 16, 16>(y, tw, t, v);
    if constexpr (N / 256 > 1) reg_stage<N, GT, N / 256, 256>(y, tw, t, v);
  } else {
    reg_stage<N, GT, M, 16>(y, tw, t, v);
  }
}

// ------------------------------------------------------- per-proposal constants
// utils/src/glass_lisa.c:1188-1198 (AEnoise) with rednoise (:1183).
static __device__ double aenoise_dev(double f, double L, double fstar) {
  double fonfstar = f / fstar;
  double sf = sin(fonfstar);
  double trans = sf * sf;
  double r = 1.0e-4 / f;
  double red = 1. + 16.0 * (pow((2.0e-5 / f), 10.0) + r * r);
  double w = kPI2 * f;
  double w4 = w * w * w * w;
  double cf = cos(fonfstar);
  return (16.0 / 3.0) * trans *
         ((2.0 + cf) * (kSPS + kSLOC) + 2.0 * (3.0 + 2.0 * cf + cos(2.0 * fonfstar)) * (kSLOC / 2.0 + kSACC / w4 * red)) /
         ((2.0 * L) * (2.0 * L));
}

// (int)pow(2, (int)log2(v) + 1) of ucb/src/glass_ucb_waveform.c:712,719.  Every
// v < 8 ends below the clamp Nmin = 16, so only v >= 1 needs the exact form,
// where (int)log2(v) is the binary exponent of v.
__device__ __forceinline__ int pow2_above_dev(double v) {
  if (!(v >= 1.0)) return 1;
  int e = ilogb(v) + 1;
  return e > 30 ? (1 << 30) : (1 << e);
}

// FP64 re-evaluation of the two spreads of the bandwidth rule for the mixed
// plans, taken when the FP32 estimate lies within 1e-4 of a power of two.
// Same formulas as ucb/src/glass_ucb_waveform.c:708-722 and AEnoise
// (utils/src/glass_lisa.c:1188-1198), evaluated with one sincos and products:
// sin(acos(c)) as sqrt((1 - c)(1 + c)), x^10 as ((x^2)^2)^2 x^2, cos 2x as
// 2 cos^2 x - 1.  These agree with the library forms to a few ulp, so N can
// differ from the reference's only for a spread within ~1e-15 of a power of
// two (where the reference's own result depends on its libm).  A lane that
// takes this path runs a few hundred FP64 instructions; the library forms
// (acos, sin, pow) cost several times that on the FP64 pipe and made this rare
// lane the tail of the whole plan launch.
__device__ __forceinline__ int doppler_spread_fp64(double T, double f0, double fdot, double costheta) {
  const double sintheta = sqrt((1.0 - costheta) * (1.0 + costheta));
  return pow2_above_dev(2 * T * ((4. + kPI2 * f0 * (kAU / kCLIGHT) * sintheta) / kYEAR + fabs(fdot) * T) - 1);
}
__device__ __forceinline__ int snr_spread_fp64(double T, double f0, double lnA, double L, double fstar) {
  const double x = f0 / fstar;
  double sf, cf;
  sincos(x, &sf, &cf);
  const double r = 1.0e-4 / f0, q = 2.0e-5 / f0, q2 = q * q, q4 = q2 * q2;
  const double red = 1. + 16.0 * (q4 * q4 * q2 + r * r);
  const double w = kPI2 * f0, w2 = w * w;
  const double c2x = 2.0 * cf * cf - 1.0;
  const double sn = (16.0 / 3.0) * sf * sf *
                    ((2.0 + cf) * (kSPS + kSLOC) + 2.0 * (3.0 + 2.0 * cf + c2x) * (kSLOC / 2.0 + kSACC / (w2 * w2) * red)) /
                    ((2.0 * L) * (2.0 * L));
  return pow2_above_dev(exp(lnA) * sqrt(T) * sf / sqrt(sn) - 1);
}

// ucb/src/glass_ucb_waveform.c:698-725 (ucb_bandwidth).
static __device__ int bandwidth_dev(double L, double fstar, double f, double fdot, double costheta, double A,
                                    double T, int NFFT) {
  const int Nmin = 16;
  int half = NFFT / 2;
  int Nmax = half >= 1 ? (1 << (31 - __clz(half))) : 0;
  double sqT = sqrt(T);
  double sf = sin(f / fstar);
  double sn = aenoise_dev(f, L, fstar);
  double sintheta = sin(acos(costheta));
  double bw = 2 * T * ((4. + kPI2 * f * (kAU / kCLIGHT) * sintheta) / kYEAR + fabs(fdot) * T);
  int DS = pow2_above_dev(bw - 1);
  if (DS > Nmax) DS = Nmax;
  if (DS < Nmin) DS = Nmin;
  double SNRm = A * sqT * sf / sqrt(sn);  // analytic_snr, ucb/src/glass_ucb_waveform.c:22-25
  int SS = pow2_above_dev(SNRm - 1);
  if (SS > Nmax) SS = Nmax;
  if (SS < Nmin) SS = Nmin;
  return (DS > SS) ? DS : SS;
}

// Source geometry shared by both precisions (ucb/src/glass_ucb_waveform.c:802-838,
// utils/src/glass_lisa.c:1566-1596).
struct SourceGeom {
  double f0, fdot, phi0, amp, eps, dfq;
  double k[3], ep[6], ec[6];
  double DPr, DPi, DCr, DCi;
};

static __host__ __device__ void source_geometry(const double *p, int NP, double T, SourceGeom &g) {
  double f0 = p[0] / T, costh = p[1], phi = p[2], cosi = p[4], psi = p[5];
  g.f0 = f0;
  g.amp = exp(p[3]);
  g.phi0 = p[6];
  g.fdot = NP > 7 ? p[7] / (T * T) : 0.0;
  double fT = f0 * T;
  long long q = (long long)fT;
  g.eps = fT - (double)q;
  g.dfq = kPI2 * (((double)q) / T);
  double sinps, cosps;
  sincos(2. * psi, &sinps, &cosps);
  double Aplus = (1. + cosi * cosi) * 0.5, Across = -cosi;
  g.DPr = Aplus * cosps;
  g.DPi = -Across * sinps;
  g.DCr = -Aplus * sinps;
  g.DCi = -Across * cosps;
  double sinth = sqrt(1.0 - costh * costh);
  double sinph, cosph;
  sincos(phi, &sinph, &cosph);
  double u[3] = {costh * cosph, costh * sinph, -sinth};
  double v[3] = {sinph, -cosph, 0.};
  g.k[0] = -sinth * cosph;
  g.k[1] = -sinth * sinph;
  g.k[2] = -costh;
  int idx = 0;
  for (int i = 0; i < 3; i++)
    for (int j = i; j < 3; j++, idx++) {
      g.ep[idx] = v[i] * v[j] - u[i] * u[j];
      g.ec[idx] = u[i] * v[j] + v[i] * u[j];
    }
}

static __host__ __device__ void make_item_f64(const SourceGeom &g, int N, ItemF64 &c) {
  for (int i = 0; i < 3; i++) c.k[i] = g.k[i];
  for (int i = 0; i < 6; i++) {
    c.ep[i] = g.ep[i];
    c.ec[i] = g.ec[i];
  }
  c.DPr = g.DPr;
  c.DPi = g.DPi;
  c.DCr = g.DCr;
  c.DCi = g.DCi;
  c.f0 = g.f0;
  c.fdot = g.fdot;
  c.phi0 = g.phi0;
  c.dfq = g.dfq;
  c.amp_s = g.amp / (2.0 * (double)N);
}

static __device__ void make_item_mix(const SourceGeom &g, int N, double T, double fstar, ItemMix &c) {
  for (int i = 0; i < 3; i++) {
    c.k[i] = (float)g.k[i];
    c.kl[i] = (float)(g.k[i] - (double)c.k[i]);
  }
  c.k[3] = 0.f;
  const double s = g.amp / (2.0 * (double)N);
  const int e = ilogb(s);
  const double m = scalbn(s, -e);  // in [1, 2)
  c.amp_p2 = (float)scalbn(1.0, e);
  for (int i = 0; i < 6; i++) {
    const double mr = m * (g.DPr * g.ep[i] + g.DCr * g.ec[i]), mi = m * (g.DPi * g.ep[i] + g.DCi * g.ec[i]);
    c.Mr[i] = (float)mr;
    c.Mi[i] = (float)mi;
    c.Mrl[i] = (float)(mr - (double)c.Mr[i]);
    c.Mil[i] = (float)(mi - (double)c.Mi[i]);
  }
  c.fonfs0 = (float)(g.f0 / fstar);
  c.fonfs0l = (float)(g.f0 / fstar - (double)c.fonfs0);
  c.fdfs = (float)(g.fdot * T / fstar);
  c.fdfsl = (float)(g.fdot * T / fstar - (double)c.fdfs);
  c.aef = (float)(0.66666666666666666666 * g.fdot * T / g.f0);
  c.aefl = (float)(0.66666666666666666666 * g.fdot * T / g.f0 - (double)c.aef);
  c.w0c = (float)(kPI2 * g.f0 / kCLIGHT);
  c.w0cl = (float)(kPI2 * g.f0 / kCLIGHT - (double)c.w0c);
  c.p7pi = (float)(kPI * g.fdot * T * T);
  c.amp_hi = (float)s;
  c.amp_lo = (float)(s - (double)c.amp_hi);
  c.eps2pi = df_from_double(kPI2 * g.eps);
  double bscale = kPI2 * g.f0 * (kAU / kCLIGHT);
  c.beta1 = df_from_double(bscale * g.k[0]);
  c.beta2 = df_from_double(bscale * g.k[1]);
  c.phi0 = df_from_double(g.phi0);
  c.p7pi_d = df_from_double(kPI * g.fdot * T * T);
}

// ----------------------------------------------------------------- slow part
// Symmetric 3x3 quadratic form r^T E r, E stored as xx, xy, xz, yy, yz, zz.
template <typename R>
__device__ __forceinline__ R quad(const R *e, R x, R y, R z) {
  return e[0] * x * x + e[3] * y * y + e[5] * z * z + (R)2 * (e[1] * x * y + e[2] * x * z + e[4] * y * z);
}

// sin(x)/x: Taylor series through x^12 for |x| <= 1 (truncation < 1e-12).
// sinc(x) - 1, so that a product with sinc(x) ~ 1 need not round it near 1
// (as 1 + small it would round to the same float over many samples of a
// slowly varying argument: a relative error common to the whole template).
__device__ __forceinline__ float sinc_m1_f(float x) {
  if (fabsf(x) > 1.0f) return sinf(x) / x - 1.0f;
  float x2 = x * x;
  float s = 1.6059043836821613e-10f;          // 1/13!
  s = fmaf(s, x2, -2.505210838544172e-08f);   // -1/11!
  s = fmaf(s, x2, 2.755731922398589e-06f);    // 1/9!
  s = fmaf(s, x2, -1.984126984126984e-04f);   // -1/7!
  s = fmaf(s, x2, 8.333333333333333e-03f);    // 1/5!
  s = fmaf(s, x2, -1.666666666666667e-01f);   // -1/3!
  return s * x2;
}

__device__ __forceinline__ float sinc_f(float x) {
  if (fabsf(x) > 1.0f) return sinf(x) / x;
  float x2 = x * x;
  float s = 1.6059043836821613e-10f;          // 1/13!
  s = fmaf(s, x2, -2.505210838544172e-08f);   // -1/11!
  s = fmaf(s, x2, 2.755731922398589e-06f);    // 1/9!
  s = fmaf(s, x2, -1.984126984126984e-04f);   // -1/7!
  s = fmaf(s, x2, 8.333333333333333e-03f);    // 1/5!
  s = fmaf(s, x2, -1.666666666666667e-01f);   // -1/3!
  return fmaf(s, x2, 1.0f);
}

// sin and cos of an FP32 argument of a few radians, FMA-only: Cody-Waite
// reduction by pi/2 (two-part constant, exact first product under FMA) to
// r in [-pi/4, pi/4], then sin r = r + r^3 P(r^2) (degree 11) and
// cos r = 1 + r^2 Q(r^2) (degree 12), coefficients fitted for this library by
// least squares in 40-digit arithmetic and rounded to float: the polynomial
// error (a few 1e-10) is far below the final rounding, so what is left is
// the rounding of the result.  (A polynomial error at the FP32 rounding level
// is a smooth function of the phase: a template-wide error, not noise.)
// Valid for |x| < ~1e3.
__device__ __forceinline__ void fast_sincos(float x, float *s, float *c) {
  const float q = rintf(x * 0.63661977236758134f);  // 2/pi
  float r = fmaf(-q, 1.57079637050628662f, x);      // float(pi/2)
  r = fmaf(-q, -4.37113900018624283e-08f, r);       // pi/2 - float(pi/2)
  const float z = r * r;
  float ps = -2.4744322334957435e-08f;
  ps = fmaf(ps, z, 2.755507975968258e-06f);
  ps = fmaf(ps, z, -1.9841262250796924e-04f);
  ps = fmaf(ps, z, 8.333333321634624e-03f);
  ps = fmaf(ps, z, -0.16666666666603547f);
  const float sr = fmaf(r * z, ps, r);
  float pc = 2.0646641311441812e-09f;
  pc = fmaf(pc, z, -2.7555547982977536e-07f);
  pc = fmaf(pc, z, 2.4801580851006652e-05f);
  pc = fmaf(pc, z, -1.3888888877952254e-03f);
  pc = fmaf(pc, z, 4.1666666666599225e-02f);
  pc = fmaf(pc, z, -0.5f);
  const float cr = fmaf(z, pc, 1.0f);
  const int qi = ((int)q) & 3;
  const float ss = (qi & 1) ? cr : sr;
  const float cc = (qi & 1) ? sr : cr;
  *s = (qi & 2) ? -ss : ss;
  *c = ((qi + 1) & 2) ? -cc : cc;
}

// Delay of spacecraft i's sample, xi = t - k.x_i / c, and the carrier
// argument w0 xi - phi0 - dfq t + wd xi^2 (ucb/src/glass_ucb_waveform.c:858-870),
// every operation rounded on its own.
__device__ __forceinline__ double slow_xi64(const ItemF64 &c, const OrbitSample64 &o, int i) {
  const double kx = __dadd_rn(__dadd_rn(__dmul_rn(o.x[i], c.k[0]), __dmul_rn(o.y[i], c.k[1])), __dmul_rn(o.z[i], c.k[2]));
  return __dsub_rn(o.t, __ddiv_rn(kx, kCLIGHT));
}
__device__ __forceinline__ double slow_arg2_64(const ItemF64 &c, double t, double w0, double wd, double xi) {
  const double a2 = __dsub_rn(__dsub_rn(__dmul_rn(w0, xi), c.phi0), __dmul_rn(c.dfq, t));
  return __dadd_rn(a2, __dmul_rn(__dmul_rn(wd, xi), xi));
}
// One arm from its spacecraft's terms and its own projections
// (ucb/src/glass_ucb_waveform.c:880-922).
__device__ __forceinline__ double2 slow_arm64(const ItemF64 &c, double fon, double aev, double arg2, double dp,
                                              double dcr, double kr) {
  const double arg1 = 0.5 * fon * (1.0 + kr);
  const double sinc = 0.25 * sin(arg1) / arg1;
  const double t1r = aev * (dp * c.DPr + dcr * c.DCr);
  const double t1i = aev * (dp * c.DPi + dcr * c.DCi);
  double s2, c2;
  sincos(__dsub_rn(arg1, arg2), &s2, &c2);
  return make_double2(sinc * (t1r * c2 + t1i * s2), sinc * (-t1r * s2 + t1i * c2));
}

// The six arm series d_ij at one sample (order 12, 13, 21, 23, 31, 32),
// amplitude-free, in FP64 with the reference's own sequence of operations
// (ucb/src/glass_ucb_waveform.c:840-922).  The carrier argument arg2 reaches
// ~1e6 rad, where every rounding step is worth ~1e-10 rad: the delay xi and
// the carrier phase round every product and sum separately (explicit
// round-to-nearest operations, which multiply-add contraction leaves alone),
// as the reference's C does; everything else may contract.
__device__ __forceinline__ void slow_sample64(const ItemF64 &c, const OrbitSample64 &o, double fstar, double L,
                                              double2 d[6]) {
  double r12[3] = {(o.x[1] - o.x[0]) / L, (o.y[1] - o.y[0]) / L, (o.z[1] - o.z[0]) / L};
  double r13[3] = {(o.x[2] - o.x[0]) / L, (o.y[2] - o.y[0]) / L, (o.z[2] - o.z[0]) / L};
  double r23[3] = {(o.x[2] - o.x[1]) / L, (o.y[2] - o.y[1]) / L, (o.z[2] - o.z[1]) / L};
  double dp12 = quad(c.ep, r12[0], r12[1], r12[2]), dc12 = quad(c.ec, r12[0], r12[1], r12[2]);
  double dp13 = quad(c.ep, r13[0], r13[1], r13[2]), dc13 = quad(c.ec, r13[0], r13[1], r13[2]);
  double dp23 = quad(c.ep, r23[0], r23[1], r23[2]), dc23 = quad(c.ec, r23[0], r23[1], r23[2]);
  double kr12 = c.k[0] * r12[0] + c.k[1] * r12[1] + c.k[2] * r12[2];
  double kr13 = c.k[0] * r13[0] + c.k[1] * r13[1] + c.k[2] * r13[2];
  double kr23 = c.k[0] * r23[0] + c.k[1] * r23[1] + c.k[2] * r23[2];
  const double t = o.t;
  const double w0 = kPI2 * c.f0, wd = kPI * c.fdot, ae = 0.66666666666666666666 * c.fdot / c.f0;
  double fon[3], arg2[3], aev[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const double xi = slow_xi64(c, o, i);
    fon[i] = (c.f0 + c.fdot * xi) / fstar;
    arg2[i] = slow_arg2_64(c, t, w0, wd, xi);
    aev[i] = 1.0 + ae * xi;
  }
  const int ai[6] = {0, 0, 1, 1, 2, 2};
  const double dps[6] = {dp12, dp13, dp12, dp23, dp13, dp23};
  const double dcs[6] = {dc12, dc13, dc12, dc23, dc13, dc23};
  const double krs[6] = {kr12, kr13, -kr12, kr23, -kr13, -kr23};
#pragma unroll
  for (int a = 0; a < 6; a++) {
    int i = ai[a];
    d[a] = slow_arm64(c, fon[i], aev[i], arg2[i], dps[a], dcs[a], krs[a]);
  }
}

// The two arms of spacecraft i (12, 13 | 21, 23 | 31, 32) with the same
// operations as slow_sample64, for a slow part that spreads the arms of a
// sample over three warps.
__device__ __forceinline__ void slow_arms64(const ItemF64 &c, const OrbitSample64 &o, double fstar, double L, int i,
                                            double2 d[2]) {
  // arm vectors: spacecraft 0 needs r12, r13; 1 needs r12 (as r21 = -r12), r23; 2 needs r13, r23
  const int pb = i == 2 ? 2 : 1;  // first vector r_{0 pb}: r12 (i = 0, 1) or r13 (i = 2)
  const int qa = i == 0 ? 0 : 1;  // second vector r_{qa 2}: r13 (i = 0) or r23 (i = 1, 2)
  const int pa = 0, qb = 2;
  const double u[3] = {(o.x[pb] - o.x[pa]) / L, (o.y[pb] - o.y[pa]) / L, (o.z[pb] - o.z[pa]) / L};
  const double v[3] = {(o.x[qb] - o.x[qa]) / L, (o.y[qb] - o.y[qa]) / L, (o.z[qb] - o.z[qa]) / L};
  const double dpu = quad(c.ep, u[0], u[1], u[2]), dcu = quad(c.ec, u[0], u[1], u[2]);
  const double dpv = quad(c.ep, v[0], v[1], v[2]), dcv = quad(c.ec, v[0], v[1], v[2]);
  const double kru = c.k[0] * u[0] + c.k[1] * u[1] + c.k[2] * u[2];
  const double krv = c.k[0] * v[0] + c.k[1] * v[1] + c.k[2] * v[2];
  const double w0 = kPI2 * c.f0, wd = kPI * c.fdot, ae = 0.66666666666666666666 * c.fdot / c.f0;
  const double xi = slow_xi64(c, o, i);
  const double fon = (c.f0 + c.fdot * xi) / fstar;
  const double arg2 = slow_arg2_64(c, o.t, w0, wd, xi);
  const double aev = 1.0 + ae * xi;
  // arm order: i = 0: 12 (u), 13 (v); i = 1: 21 (-u), 23 (v); i = 2: 31 (-u), 32 (-v)
  d[0] = slow_arm64(c, fon, aev, arg2, dpu, dcu, i == 0 ? kru : -kru);
  d[1] = slow_arm64(c, fon, aev, arg2, dpv, dcv, i == 2 ? -krv : krv);
}

// Carrier phase common to the three spacecraft, reduced mod 2 pi:
//   eps2pi u - (beta1 cos a + beta2 sin a) - phi0 + p7pi u^2
// from double-float constants and table values, as one error-free dot
// product: exact high products (two_prod), their cross terms and every
// rounding error of the high-part sum (two_sum) collected in one FP32 error
// term, one reduction at the end (~55 FP32 instructions; the same to FP32
// rounding of the reduced angle as df_mul/df_add chains, which take ~100).
__device__ __forceinline__ df carrier_phase_mix(const ItemMix &c, const OrbitSampleMix &o) {
  const float uh = o.u_hi, ul = o.u_lo;
  // u^2 as hi + lo
  const df uu = two_prod(uh, uh);
  const float uul = fmaf(2.f * uh, ul, uu.lo);
  // products
  const df p1 = two_prod(c.eps2pi.hi, uh);
  float err = fmaf(c.eps2pi.hi, ul, fmaf(c.eps2pi.lo, uh, p1.lo));
  const df p2 = two_prod(-c.beta1.hi, o.ca_hi);
  err += fmaf(-c.beta1.hi, o.ca_lo, fmaf(-c.beta1.lo, o.ca_hi, p2.lo));
  const df p3 = two_prod(-c.beta2.hi, o.sa_hi);
  err += fmaf(-c.beta2.hi, o.sa_lo, fmaf(-c.beta2.lo, o.sa_hi, p3.lo));
  const df p4 = two_prod(c.p7pi_d.hi, uu.hi);
  err += fmaf(c.p7pi_d.hi, uul, fmaf(c.p7pi_d.lo, uu.hi, p4.lo));
  // high parts, exactly
  df sum = two_sum(p1.hi, p2.hi);
  err += sum.lo;
  sum = two_sum(sum.hi, p3.hi);
  err += sum.lo;
  sum = two_sum(sum.hi, p4.hi);
  err += sum.lo;
  sum = two_sum(sum.hi, -c.phi0.hi);
  err += sum.lo - c.phi0.lo;
  return df_reduce_2pi_df(quick_two_sum(sum.hi, err));
}

// Mixed precision: the carrier phase common to the three spacecraft
// (heterodyne 2 pi (f0 T - q) t/T, guiding-centre Doppler 2 pi f0 k.x_gc/c,
// phi0 and pi fdot t^2) is summed in double-float and reduced mod 2 pi; the
// per-spacecraft corrections (< 0.5 rad) and everything else are FP32.
__device__ __forceinline__ void slow_sample_mix(const ItemMix &c, const OrbitSampleMix &o, const GeoSampleMix &gm,
                                                float invL, float AUc, float invT, float2 d[6]) {
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
  // k.(x_i - x_gc) per spacecraft (metres); k.r_ij from their differences
  float kd[3];
#pragma unroll
  for (int i = 0; i < 3; i++)
    kd[i] = fmaf(c.k[0], f[3 * i], fmaf(c.k[1], f[3 * i + 1], fmaf(c.k[2], f[3 * i + 2],
            fmaf(c.kl[0], f[3 * i], fmaf(c.kl[1], f[3 * i + 1], c.kl[2] * f[3 * i + 2])))));
  const float kr12 = (kd[1] - kd[0]) * invL, kr13 = (kd[2] - kd[0]) * invL, kr23 = (kd[2] - kd[1]) * invL;
  // r^T M r with M = hi + lo: the lo part's sum first, so that only the
  // products of the hi part round at full size
  auto quad6 = [&](const float *M, const float *Ml, int a) {
    const float *mo = f + 9 + 6 * a;
    const float l = fmaf(Ml[0], mo[0], fmaf(Ml[1], mo[1], fmaf(Ml[2], mo[2], fmaf(Ml[3], mo[3], fmaf(Ml[4], mo[4], Ml[5] * mo[5])))));
    return fmaf(M[0], mo[0], fmaf(M[1], mo[1], fmaf(M[2], mo[2], fmaf(M[3], mo[3], fmaf(M[4], mo[4], fmaf(M[5], mo[5], l))))));
  };
  const float mr12 = quad6(c.Mr, c.Mrl, 0), mi12 = quad6(c.Mi, c.Mil, 0);
  const float mr13 = quad6(c.Mr, c.Mrl, 1), mi13 = quad6(c.Mi, c.Mil, 1);
  const float mr23 = quad6(c.Mr, c.Mrl, 2), mi23 = quad6(c.Mi, c.Mil, 2);

  // The phase of each arm is carried as hi + lo until the rotation: rounded
  // to float it would carry ~2e-7 rad of noise per sample from three
  // roundings, which the first-order correction of the sine and cosine
  // below removes.
  const df psi0 = carrier_phase_mix(c, o);
  const float uf = o.u_hi;
  const float tgc = AUc * (c.k[0] * ca + c.k[1] * sa);  // guiding-centre delay (s)

  // aev_i = 1 + aef v is kept as aef v: for a slowly chirping source it is
  // below one float ulp of 1, and rounded it would be the same float over
  // many samples (a relative error common to the template)
  float fon[3], aevm1[3];
  df arg2[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float kdx = kd[i];  // k.(x_i - x_gc), metres
    float taui = tgc + kdx * (float)(1.0 / kCLIGHT);
    float tT = taui * invT;
    float v = uf - tT;  // xi / T
    fon[i] = c.fonfs0 + fmaf(c.fdfs, v, c.fonfs0l);
    aevm1[i] = c.aef * v;
    const df wk = two_prod(c.w0c, kdx);
    arg2[i] = df_add(psi0, df{-wk.hi, fmaf(c.p7pi * tT, tT - 2.0f * uf, -fmaf(c.w0cl, kdx, wk.lo))});
  }
  const int ai[6] = {0, 0, 1, 1, 2, 2};
  const float mrs[6] = {mr12, mr13, mr12, mr23, mr13, mr23};
  const float mis[6] = {mi12, mi13, mi12, mi23, mi13, mi23};
  const float krs[6] = {kr12, kr13, -kr12, kr23, -kr13, -kr23};
#pragma unroll
  for (int a = 0; a < 6; a++) {
    int i = ai[a];
    const float arg1 = 0.5f * fon[i] * (1.0f + krs[a]);
    const float sm1 = sinc_m1_f(arg1);  // sinc - 1
    const float t1r = fmaf(aevm1[i], mrs[a], mrs[a]);
    const float t1i = fmaf(aevm1[i], mis[a], mis[a]);
    const df th = two_sum(arg1, -arg2[i].hi);
    const float tl = th.lo - arg2[i].lo;
    float s2, c2;
    fast_sincos(th.hi, &s2, &c2);
    const float s2c = fmaf(tl, c2, s2), c2c = fmaf(-tl, s2, c2);  // sin, cos of th.hi + tl
    const float pr = t1r * c2c + t1i * s2c, pi = -t1r * s2c + t1i * c2c;
    d[a] = make_float2(0.25f * fmaf(sm1, pr, pr), 0.25f * fmaf(sm1, pi, pi));
  }
}

// Arm combinations whose FFTs give the A and E channels:
//   A = (Z - X)/sqrt2 needs FFT(a2) (factor of the exp(-2ix)-type weight) and FFT(a1);
//   E = (X - 2Y + Z)/sqrt6 needs FFT(e2) and FFT(e1).
// (utils/src/glass_lisa.c:645-710 and :429-441)
template <typename C>
__device__ __forceinline__ void ae_combos(const C d[6], C out[4]) {
  // d: 12, 13, 21, 23, 31, 32
  const C d12 = d[0], d13 = d[1], d21 = d[2], d23 = d[3], d31 = d[4], d32 = d[5];
  out[0] = csub(cadd(d31, d13), cadd(d32, d12));                                     // a2
  out[1] = csub(cadd(d13, d31), cadd(d23, d21));                                     // a1
  out[2] = cadd(csub(csub(cadd(d12, d31), d13), d32), cscale(csub(d21, d23), 2));    // e2
  out[3] = cadd(csub(csub(cadd(d13, d21), d23), d31), cscale(csub(d12, d32), 2));    // e1
}

// ------------------------------------------------------------- kernel args
struct PlanArgs {
  int nitems, nseg, NFFT, cap, precision;
  int n_fixed;  // 0: bandwidth rule
  int per_cta = 16;  // mixed plan: proposals per CTA (16..32 lanes of each role warp)
  double T, fstar, L;
  const int *item_seg;
  const double *params;
  const double *term_x;
  const int *seg_qmin;
  ItemF64 *items64;
  ItemMix *itemsmix;
  int *bin_count, *bin_list;
  double *dlogl, *term_y, *hh;
  int *status;
};

// Outputs of a proposal that is not evaluated (bad input, or a template
// entirely outside its segment).
__device__ __forceinline__ void plan_write_skipped(const PlanArgs &a, int i, int st) {
  const double tx = a.term_x ? a.term_x[i] : 0.0;
  if (st & 3) {
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    a.dlogl[i] = nan;
    if (a.term_y) a.term_y[i] = nan;
    if (a.hh) a.hh[i] = nan;
  } else {  // outside: logL is unchanged
    a.dlogl[i] = 0.0 - tx;
    if (a.term_y) a.term_y[i] = 0.0;
    if (a.hh) a.hh[i] = 0.0;
  }
  if (a.status) a.status[i] = st;
}

// Warp-aggregated binning: one atomic per distinct size per warp.
__device__ __forceinline__ void plan_bin(const PlanArgs &a, int i, int b) {
  const int lane = threadIdx.x & 31;
  const unsigned active = __ballot_sync(0xffffffffu, b >= 0);
  if (b >= 0) {
    const unsigned same = __match_any_sync(active, b);
    const int first = __ffs(same) - 1;
    int base = 0;
    if (lane == first) base = atomicAdd(&a.bin_count[b], __popc(same));
    base = __shfl_sync(same, base, first);
    const int slot = base + __popc(same & ((1u << lane) - 1));
    if (chk(slot < a.cap && b < kNumBins, kChkBinList)) a.bin_list[(size_t)b * a.cap + slot] = i;
  }
}

__device__ __forceinline__ int plan_validate(const PlanArgs &a, int i, double *p, int &seg) {
  bool finite = true;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    p[k] = a.params[8 * (size_t)i + k];
    finite = finite && isfinite(p[k]);
  }
  seg = a.item_seg[i];
  int st = 0;
  if (seg < 0 || seg >= a.nseg) st |= 2;
  if (!finite || fabs(p[1]) > 1.0 || fabs(p[4]) > 1.0) st |= 1;
  return st;
}

// (int)pow(2, (int)log2(v) + 1) from an FP32 estimate of v, or -1 when v lies
// within 1e-4 (relative) of a power of two, where an FP32 estimate could fall
// on the other side of the boundary than the reference's FP64 value.
__device__ __forceinline__ int pow2_above_f32(float v) {
  if (!(v >= 1.0f)) return (v < 0.99f) ? 1 : -1;
  int e;
  float m = frexpf(v, &e);  // v = m 2^e, m in [0.5, 1)
  if (m < 0.50005f || m > 0.99995f) return -1;
  return e > 30 ? (1 << 30) : (1 << e);  // (int)log2(v) = e - 1
}

// Mixed-precision plan of proposal i: FP32 except where a constant sets the
// carrier phase (f0 T - q, the Doppler amplitude 2 pi f0 AU/c k, phi0,
// pi fdot T^2), and the bandwidth rule, which is evaluated in FP32 and
// re-evaluated in FP64 only for values near a power-of-two boundary, so N is
// always the reference's.  N_fixed > 0 replaces the rule by that size.
// Returns the status bits; fills c when they are 0.
__device__ __forceinline__ int planmix_item(const PlanArgs &a, int i, int N_fixed, ItemMix &c) {
  double p[8];
  int seg;
  int st = plan_validate(a, i, p, seg);
  const double T = a.T;
  const double f0 = p[0] / T;
  const float Tf = (float)T, f0f = (float)f0, costhf = (float)p[1];
  const float fdotf = (float)(p[7] / (T * T));
  const float ampf = expf((float)p[3]);
  const float sinthf = sqrtf(fmaxf(0.f, 1.f - costhf * costhf));
  int N = 0;
  if (!st && N_fixed > 0) {
    N = N_fixed;
  } else if (!st) {
    const int Nmin = 16;
    const int half = a.NFFT / 2;
    const int Nmax = half >= 1 ? (1 << (31 - __clz(half))) : 0;
    // Doppler spread (ucb/src/glass_ucb_waveform.c:708-714)
    float bw = 2.f * Tf * ((4.f + 6.2831853f * f0f * (float)(kAU / kCLIGHT) * sinthf) / (float)kYEAR + fabsf(fdotf) * Tf);
    int DS = pow2_above_f32(bw - 1.f);
    if (DS < 0) DS = doppler_spread_fp64(T, f0, p[7] / (T * T), p[1]);
    if (DS > Nmax) DS = Nmax;
    if (DS < Nmin) DS = Nmin;
    // SNR spread (:717-722) with AEnoise (utils/src/glass_lisa.c:1188-1198)
    const float x = f0f / (float)a.fstar;
    float sx, cx;
    sincosf(x, &sx, &cx);
    const float c2x = 2.f * cx * cx - 1.f;
    const float w = 6.2831853f * f0f, w2 = w * w;
    const float q1 = 2.0e-5f / f0f, q2 = q1 * q1, q4 = q2 * q2, r1 = 1.0e-4f / f0f;
    const float red = 1.f + 16.f * (q4 * q4 * q2 + r1 * r1);
    // AEnoise times (2L)^2: AEnoise itself (~1e-42) is below FP32's normal range
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
    if (N < kMinN || N > kMaxN) st |= 1;
  }
  const double fT = f0 * T;
  const long long q = (long long)fT;
  int imin = 0;
  if (!st) {
    imin = (int)(q - N / 2) - a.seg_qmin[seg];
    if (imin >= a.NFFT || imin + N <= 0) st = 4;
  }
  if (!st) {
    // Geometry, polarisation and amplitude in FP64, rounded once: an FP32
    // exp of lnA ~ -50, or FP32 trigonometry of phi and 2 psi, would put a
    // systematic 1e-7..1e-6 error on the template that shows up in delta
    // logL even at the likelihood maximum.
    SourceGeom g;
    source_geometry(p, 8, T, g);
    make_item_mix(g, N, T, a.fstar, c);
    c.seg = seg;
    c.N = N;
    c.imin = imin;
    c.pad = 0;
  }
  return st;
}

// Stage 1: slow part of every (proposal, sample) pair, written to scratch as the
// four arm-combination series of each proposal.
struct SlowArgs {
  int cap, NFFT;
  double fstar, L;
  float Rf, invLf, AUcf, invTf;  // orbit radius, 1/L, AU/c, 1/T for the FP32 path
  const int *bin_count, *bin_list;
  const ItemF64 *items64;
  const ItemMix *itemsmix;
  const OrbitSample64 *pos64[kNumBins];
  const OrbitSampleMix *mix[kNumBins];
  const GeoSampleMix *geo[kNumBins] = {};  // mixed only
  void *series;  // float2 (mixed) or double2 (FP64)
  // double-float slow part of the re-evaluation: the geometry's low parts
  // and 1/L, AU/c, 1/T, 1/c as hi + lo floats; series as float4
  const GeoSampleMix *geolo[kNumBins] = {};
  df invLd, AUcd, invTd, invcd;
  // extents for the checked build: proposals, and series elements
  int nitems = 0;
  long long series_len = 0;
};

// Stage 2: FFTs, TDI weights, whitening and the residual power, per size.
struct SpecArgs {
  int NFFT, cap, bin;
  // extents for the checked build: proposals, segments, series elements
  int nitems = 0, nseg = 0;
  long long series_len = 0;
  const int *bin_count;
  const int *bin_list;  // this size's list
  const ItemF64 *items64;
  const ItemMix *itemsmix;
  const void *series;
  const void *tw;
  const float4 *w32;
  const float4 *w32lo;
  const float4 *g32;
  const float4 *g32lo = nullptr;
  const double *Q;
  const double2 *w64;
  const double2 *g64;
  const double *term_x;
  double *dlogl, *term_y, *hh;
  int *status;
  // per-channel form (the PERCH kernels): term_ch[2 i + c] is channel c's
  // share of term_y (c = 0 A, 1 E); QA the A channel's part of Q
  double *term_ch = nullptr;
  const double *QA = nullptr;
  // mixed precision: a proposal whose error estimate
  //   (fb_e1 sqrt(hw_full rr / N) + fb_e2 |(h|r - h)|) / scale_i
  // (hw = |h|^2, rr = |r - h|^2, whitened sums over the template support;
  // hw_full = hw scaled by the template's raw power over all its N bins
  // against the power inside the segment) exceeds 1 is listed for the
  // double-float re-evaluation in its size's list, hp_list[bin cap ..]
  // (count hp_count[bin]), the total in *fb_count; fb_total counts them over
  // the context's life.  No list: no estimate.
  int *fb_count = nullptr, *hp_count = nullptr, *hp_list = nullptr;
  unsigned long long *fb_total = nullptr;
  float fb_e1 = 0.f, fb_e2 = 0.f;
  // per-proposal tolerance scale: 1/scale_i for i < fb_nscale (null: 1)
  const float *fb_inv_scale = nullptr;
  int fb_nscale = 0;
};

// The estimate's factor for proposal i (1 / its tolerance scale).
__device__ __forceinline__ float fb_scale_of(const float *inv_scale, int n, int i) {
  return (inv_scale && i < n) ? inv_scale[i] : 1.f;
}

// Double-float re-evaluation (ucb_fd_hp.cu) of listed mixed proposals: their
// series in double-float, laid out by the size counts, and the spectral stage
// in double-float.
struct HpArgs {
  int NFFT, cap;
  // extents for the checked build: proposals, segments, series elements
  int nitems = 0, nseg = 0;
  long long series_len = 0;
  int nmax;  // largest template size the bank allows (shared memory is sized for it)
  const int *bin_count = nullptr, *bin_list = nullptr;
  const ItemMix *itemsmix = nullptr;
  const float4 *series = nullptr;  // (hi re, hi im, lo re, lo im) per sample
  // zeroing at the end: the last CTA zeroes nzero ints at zero_at
  int *zero_at = nullptr;
  int nzero = 0;
  int *done = nullptr;  // CTA-done counter (zeroed by the last CTA)
  // segment tables, as hi + lo floats: whitened residual {A, E}, TDI/whitening
  // weights {G2, G1} per channel, and twiddles of each size
  const float4 *w32, *w32lo, *g32, *g32lo;
  const double *Q, *QA;
  const float4 *tw32x[kNumBins];
  // outputs
  const double *term_x;
  double *dlogl, *term_y, *hh, *term_ch;
  int *status;
};
// Computes the listed proposals' series in double-float and evaluates their
// spectral stage in double-float, writing over the mixed results; the
// re-evaluation's counts end at zero.
cudaError_t fd_launch_reeval(const SlowArgs &sa, const HpArgs &h, bool perch, int num_sms, cudaStream_t stream,
                             int *nlaunch);
// The re-evaluation's constant tables on the current device (once per device).
cudaError_t fd_hp_tables_init();

// Start (in samples) of size bin `bin` in the scratch series: sizes are laid
// out in increasing order, proposals of one size back to back, each holding 4
// series of N samples.  Computed in registers from the per-size counts.
__device__ __forceinline__ long long bin_sample_start(const int *bin_count, int NFFT, int bin) {
  long long acc = 0;
#pragma unroll
  for (int b = 0; b < kNumBins; b++)
    if (b < bin && (32 << b) <= NFFT) acc += (long long)bin_count[b] * (32 << b);
  return acc;
}

// ------------------------------------------------------- stage 1 (templated)
// One warp per 32 consecutive samples of one proposal (every N is a multiple
// of 32), grid-stride over all proposals of every size.
template <bool MIX, int BLOCK = 256>
__global__ void __launch_bounds__(BLOCK) fd_slow_kernel(SlowArgs a) {
  using C = typename std::conditional<MIX, float2, double2>::type;
  // chunk offsets per size (chunks of 32 samples: N/32 = 2^b per proposal), in registers
  int cs[kNumBins + 1];
  int acc = 0;
#pragma unroll
  for (int b = 0; b < kNumBins; b++) {
    cs[b] = acc;
    if ((32 << b) <= a.NFFT) acc += a.bin_count[b] << b;
  }
  cs[kNumBins] = acc;
  const int nchunks = acc;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  C *series = reinterpret_cast<C *>(a.series);
#pragma unroll 1
  for (int ch = warp; ch < nchunks; ch += nwarps) {
    int b = 0, cb = 0;
#pragma unroll
    for (int bb = 1; bb < kNumBins; bb++)
      if (ch >= cs[bb]) {
        b = bb;
        cb = cs[bb];
      }
    const int N = 32 << b;
    const int local = ch - cb;
    const int slot = local >> b;
    const int n = ((local & ((1 << b) - 1)) << 5) + lane;
    if (!chk(slot < a.cap, kChkBinList)) continue;
    const int item = a.bin_list[(size_t)b * a.cap + slot];
    if (!chk(item >= 0 && item < a.nitems, kChkItem)) continue;
    C d[6], cmb[4];
    if constexpr (MIX) {
      slow_sample_mix(a.itemsmix[item], a.mix[b][n], a.geo[b][n], a.invLf, a.AUcf, a.invTf, d);
    } else {
      slow_sample64(a.items64[item], a.pos64[b][n], a.fstar, a.L, d);
    }
    ae_combos(d, cmb);
    const long long o0 = ((long long)cb * 32 + (long long)slot * N) * 4 + n;
    if (!chk(o0 >= 0 && o0 + 3LL * N < a.series_len, kChkSeriesWrite)) continue;
    C *out = series + o0;
#pragma unroll
    for (int s = 0; s < 4; s++) out[(size_t)s * N] = cmb[s];
  }
}

// ------------------------------------------------------- stage 2 (templated)
template <int N>
struct SpecCfg {
  static constexpr int GT = N / 4;  // one radix-4 butterfly per series per thread
  static constexpr int CTA = GT >= 64 ? GT : 128;
  static constexpr int GPC = CTA / GT;
};

template <int N, bool MIX>
struct SpecSmem {
  using C = typename std::conditional<MIX, float2, double2>::type;
  // twiddles: FP64, or hi + lo floats for the mixed register FFT
  using TW = typename std::conditional<MIX, float4, double2>::type;
  static constexpr int NSER = (!MIX && N == 4096) ? 2 : 4;  // series resident at once
  static constexpr int PASSES = 4 / NSER;
  // mixed: twiddles and series in padded rows (pad16)
  static constexpr int SN = MIX ? pad16(N) : N;
  static constexpr size_t bytes =
      sizeof(TW) * (size_t)SN + sizeof(C) * (size_t)SN * (size_t)SpecCfg<N>::GPC * NSER + sizeof(double) * 3 * 32;
};

// Sum over the threads of one group (result valid in lane 0 of the group).
template <int GT>
__device__ __forceinline__ double group_sum(double v, double *red, int lane) {
#pragma unroll
  for (int off = (GT < 32 ? GT : 32) / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if constexpr (GT > 32) {
    __syncthreads();
    if ((lane & 31) == 0) red[lane >> 5] = v;
    __syncthreads();
    if (lane == 0) {
      double s = 0;
      for (int w = 0; w < GT / 32; w++) s += red[w];
      v = s;
    }
  }
  return v;
}

// The same in double-float arithmetic (FP32 operations only: the FP64 pipe of
// this GPU runs at 1/64 of the FP32 rate).  Result valid in lane 0 of the group.
template <int GT>
__device__ __forceinline__ df group_sum_df(float v, float2 *red, int lane) {
  df s = {v, 0.f};
#pragma unroll
  for (int off = (GT < 32 ? GT : 32) / 2; off > 0; off >>= 1) {
    df o = {__shfl_xor_sync(0xffffffffu, s.hi, off), __shfl_xor_sync(0xffffffffu, s.lo, off)};
    s = df_add(s, o);
  }
  if constexpr (GT > 32) {
    __syncthreads();
    if ((lane & 31) == 0) red[lane >> 5] = make_float2(s.hi, s.lo);
    __syncthreads();
    if (lane == 0) {
      df t = {0.f, 0.f};
      for (int w = 0; w < GT / 32; w++) t = df_add(t, df{red[w].x, red[w].y});
      s = t;
    }
  }
  return s;
}

// Four float sums at once (FP32: the mixed path's error estimate).  red: 4
// floats per warp of the group; result valid in lane 0.
template <int GT>
__device__ __forceinline__ float4 group_sum4(float4 v, float *red, int lane) {
#pragma unroll
  for (int off = (GT < 32 ? GT : 32) / 2; off > 0; off >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, off);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, off);
    v.z += __shfl_xor_sync(0xffffffffu, v.z, off);
    v.w += __shfl_xor_sync(0xffffffffu, v.w, off);
  }
  if constexpr (GT > 32) {
    __syncthreads();
    if ((lane & 31) == 0) {
      float *o = red + 4 * (lane >> 5);
      o[0] = v.x;
      o[1] = v.y;
      o[2] = v.z;
      o[3] = v.w;
    }
    __syncthreads();
    if (lane == 0) {
      v = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int w = 0; w < GT / 32; w++) {
        v.x += red[4 * w];
        v.y += red[4 * w + 1];
        v.z += red[4 * w + 2];
        v.w += red[4 * w + 3];
      }
    }
  }
  return v;
}

// The same for a double-float value per thread.
template <int GT>
__device__ __forceinline__ df group_sum_df(df s, float2 *red, int lane) {
#pragma unroll
  for (int off = (GT < 32 ? GT : 32) / 2; off > 0; off >>= 1) {
    df o = {__shfl_xor_sync(0xffffffffu, s.hi, off), __shfl_xor_sync(0xffffffffu, s.lo, off)};
    s = df_add(s, o);
  }
  if constexpr (GT > 32) {
    __syncthreads();
    if ((lane & 31) == 0) red[lane >> 5] = make_float2(s.hi, s.lo);
    __syncthreads();
    if (lane == 0) {
      df t = {0.f, 0.f};
      for (int w = 0; w < GT / 32; w++) t = df_add(t, df{red[w].x, red[w].y});
      s = t;
    }
  }
  return s;
}

// Adds (w_hi + w_lo - h)^2 to the compensated sum (S, E): the residual's
// rounding error and the square's are carried exactly (two_sum, two_prod)
// and every addition's error collects in E (cascaded summation), so the sum
// has no rounding of the order of its terms.  A loud template far from the
// data puts |r|^2 ~ 1e6 into a few bins; rounded there, the sum would carry
// an error of ~1e-8 of itself into delta logL.
__device__ __forceinline__ void acc_resid_sq(float whi, float wlo, float h, float &S, float &E) {
  const df r = two_sum(whi, -h);
  const float rl = r.lo + wlo;
  const df p = two_prod(r.hi, r.hi);
  const df t = two_sum(S, p.hi);
  S = t.hi;
  E += t.lo + fmaf(2.f * r.hi, rl, p.lo);
}

// a b + c, complex, with fused multiply-adds
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}

}  // namespace glass
#include "ucb_fd_hp.cuh"
namespace glass {

// One unit of the spectral stage: GPC proposals of size N, one group of N/4
// threads each, in a CTA of GPC N/4 threads.  Per proposal: the 4 A/E series
// (from the slow kernel's scratch) are FFT'd in shared memory, weighted per bin
// by the segment's TDI/whitening table and reduced to the residual power.
// reds: 96 doubles of reduction scratch per group.
template <int N, bool MIX, int GPC, bool PERCH = false>
__device__ __forceinline__ void spec_unit(const SpecArgs &a, const int *bin_list, int count, int base,
                                          const typename SpecSmem<N, MIX>::C *series,
                                          const typename SpecSmem<N, MIX>::TW *tw,
                                          typename SpecSmem<N, MIX>::C *bufs, double *reds) {
  using S = SpecSmem<N, MIX>;
  using C = typename S::C;
  constexpr int GT = N / 4, NSER = S::NSER, PASSES = S::PASSES;
  constexpr int CH = MIX ? 4 : 2;
  constexpr int B = N / GT;  // bins per thread (4)
  const int g = threadIdx.x / GT, lane = threadIdx.x % GT;
  constexpr int SN = S::SN;
  C *buf = bufs + (size_t)g * NSER * SN;
  double *red = reds + 96 * g;
  const int NFFT = a.NFFT;
  const int slot = base + g;
  const bool valid = slot < count;
  const int sl = valid ? slot : count - 1;
  // checked build: an index outside its buffer is recorded, the group reads
  // from the buffers' starts instead (it still runs its FFT and barriers) and
  // the proposal's results are not written
  const bool lok = chk(sl >= 0 && sl < a.cap, kChkBinList);
  const int item = lok ? bin_list[sl] : 0;
  const bool iok = chk(item >= 0 && item < a.nitems, kChkItem);
  int seg = 0, imin = 0;
  if constexpr (MIX) {
    if (iok) {
      seg = a.itemsmix[item].seg;
      imin = a.itemsmix[item].imin;
    }
  } else {
    if (iok) {
      seg = a.items64[item].seg;
      imin = a.items64[item].imin;
    }
  }
  const bool sok = chk(seg >= 0 && seg < a.nseg, kChkBankRead);
  const bool rok = chk((long long)(sl + 1) * 4 * N <= a.series_len, kChkSeriesRead);
  const bool inb = lok && iok && sok && rok;
  if (!inb) seg = 0;
  const C *src = series + (inb ? (size_t)sl * 4 * N : 0);
  // the error estimate's sums: only with a re-evaluation list; the raw
  // spectral power only for a template the segment edge clips
  const bool est_on = MIX && a.hp_list != nullptr;
  const bool clipped = imin < 0 || imin + N > NFFT;
  // mixed: per-thread compensated sums of |r - h|^2 (A in (rS, eS), E in
  // (rE, eE): two independent chains) and a float sum of |h|^2; for the error
  // estimate, Re and Im of (h|r - h) over the support (x, y) and the
  // template's raw spectral power inside the segment (z) and over all its
  // bins (w)
  float rS = 0.f, rE = 0.f, eS = 0.f, eE = 0.f, fh = 0.f;
  float4 ev = make_float4(0.f, 0.f, 0.f, 0.f);
  double acc = 0.0, hacc = 0.0;
  double accE = 0.0;
#pragma unroll 1
  for (int pass = 0; pass < PASSES; ++pass) {
    if constexpr (MIX) {
      fft4_reg<N, GT>(src, buf, tw, lane);
    } else {
#pragma unroll
      for (int s = 0; s < NSER; ++s)
#pragma unroll
        for (int r = 0; r < B; ++r) buf[s * N + lane + GT * r] = src[(size_t)(pass * NSER + s) * N + lane + GT * r];
      group_sync<GT>();
      group_fft<N, GT, NSER, (CH < NSER ? CH : NSER)>(buf, tw, lane);
    }
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const int k = lane + GT * r;
      const int m = (k + N / 2) & (N - 1);  // fftshift: output bin m holds FFT index m + N/2
      const int j = imin + m;
      if constexpr (MIX) {
        const int kp = pad16(k);
        const float2 b0 = buf[0 * SN + kp], b1 = buf[1 * SN + kp], b2 = buf[2 * SN + kp], b3 = buf[3 * SN + kp];
        const bool inside = j >= 0 && j < NFFT;
        if (est_on && clipped) {
          const float pw = fmaf(b0.x, b0.x, fmaf(b0.y, b0.y, fmaf(b1.x, b1.x, fmaf(b1.y, b1.y,
                           fmaf(b2.x, b2.x, fmaf(b2.y, b2.y, fmaf(b3.x, b3.x, b3.y * b3.y)))))));
          ev.w += pw;
          if (inside) ev.z += pw;
        }
        if (!inside) continue;
        const size_t sj = (size_t)seg * NFFT + j;
        const float4 w = a.w32[sj], wl = a.w32lo[sj];
        const float4 gA = a.g32[2 * sj], gE = a.g32[2 * sj + 1];
        const float4 gAl = a.g32lo[2 * sj], gEl = a.g32lo[2 * sj + 1];
        const float p2 = a.itemsmix[item].amp_p2;
        // the bin's table entries as hi + lo (the lo products first), then
        // the amplitude's power of two, which is exact: O(1) whitened values
        // (unscaled, their squares would overflow FP32)
        const float2 HA = cfma(b0, make_float2(gA.x, gA.y),
                               cfma(b1, make_float2(gA.z, gA.w),
                                    cfma(b0, make_float2(gAl.x, gAl.y), cmul(b1, make_float2(gAl.z, gAl.w)))));
        const float2 HE = cfma(b2, make_float2(gE.x, gE.y),
                               cfma(b3, make_float2(gE.z, gE.w),
                                    cfma(b2, make_float2(gEl.x, gEl.y), cmul(b3, make_float2(gEl.z, gEl.w)))));
        const float2 hA = cscale(HA, p2), hE = cscale(HE, p2);
        acc_resid_sq(w.x, wl.x, hA.x, rS, eS);
        acc_resid_sq(w.y, wl.y, hA.y, rS, eS);
        acc_resid_sq(w.z, wl.z, hE.x, rE, eE);
        acc_resid_sq(w.w, wl.w, hE.y, rE, eE);
        fh += fmaf(hA.x, hA.x, hA.y * hA.y) + fmaf(hE.x, hE.x, hE.y * hE.y);
        if (est_on) {
          const float dAx = w.x - hA.x, dAy = w.y - hA.y, dEx = w.z - hE.x, dEy = w.w - hE.y;
          ev.x += fmaf(hA.x, dAx, fmaf(hA.y, dAy, fmaf(hE.x, dEx, hE.y * dEy)));
          ev.y += fmaf(hA.x, dAy, fmaf(-hA.y, dAx, fmaf(hE.x, dEy, -hE.y * dEx)));
        }
      } else {
        if (j < 0 || j >= NFFT) continue;
        const size_t sj = (size_t)seg * NFFT + j;
        const double s = a.items64[item].amp_s;
        // series (2 ch, 2 ch + 1) of this pass hold the A (chan 0) or E (chan 1) pair
#pragma unroll
        for (int ch = 0; ch < NSER / 2; ++ch) {
          const int chan = pass * (NSER / 2) + ch;
          const double2 w = a.w64[2 * sj + chan];
          const double2 g2 = a.g64[4 * sj + 2 * chan], g1 = a.g64[4 * sj + 2 * chan + 1];
          double2 h = cadd(cmul(buf[(2 * ch) * N + k], g2), cmul(buf[(2 * ch + 1) * N + k], g1));
          h = cscale(h, s);
          if (PERCH && chan == 1)
            accE += 2.0 * (w.x * h.x + w.y * h.y) - (h.x * h.x + h.y * h.y);
          else
            acc += 2.0 * (w.x * h.x + w.y * h.y) - (h.x * h.x + h.y * h.y);
          hacc += h.x * h.x + h.y * h.y;
        }
      }
    }
    group_sync<GT>();
  }
  df sa, sh, saE;
  if constexpr (MIX) {
    float2 *redf = reinterpret_cast<float2 *>(red);
    if constexpr (PERCH) {
      sa = group_sum_df<GT>(quick_two_sum(rS, eS), redf, lane);
      saE = group_sum_df<GT>(quick_two_sum(rE, eE), redf + 64, lane);
    } else {
      sa = group_sum_df<GT>(df_add(quick_two_sum(rS, eS), quick_two_sum(rE, eE)), redf, lane);
    }
    sh = group_sum_df<GT>(fh, redf + 32, lane);
    if (est_on) ev = group_sum4<GT>(ev, reinterpret_cast<float *>(red), lane);
  } else {
    acc = group_sum<GT>(acc, red, lane);
    hacc = group_sum<GT>(hacc, red + 32, lane);
    if constexpr (PERCH) accE = group_sum<GT>(accE, red + 64, lane);
  }
  if (valid && inb && lane == 0) {
    double term, hh;
    if constexpr (MIX) {
      // FP64 only for the final sum (GB300's FP64 pipe is slow, and this runs
      // once per proposal at the end of every unit)
      int jlo = imin < 0 ? 0 : imin;
      int jhi = imin + N > NFFT ? NFFT : imin + N;
      const double *Qs = a.Q + (size_t)seg * (NFFT + 1);
      float rr;  // |r - h|^2 over the support, both channels
      if constexpr (PERCH) {
        const double *QAs = a.QA + (size_t)seg * (NFFT + 1);
        const double qa = QAs[jhi] - QAs[jlo];
        const double tA = (qa - (double)sa.hi) - (double)sa.lo;
        const double tE = (((Qs[jhi] - Qs[jlo]) - qa) - (double)saE.hi) - (double)saE.lo;
        a.term_ch[2 * (size_t)item] = tA;
        a.term_ch[2 * (size_t)item + 1] = tE;
        term = tA + tE;
        rr = sa.hi + saE.hi;
      } else {
        term = ((Qs[jhi] - Qs[jlo]) - (double)sa.hi) - (double)sa.lo;
        rr = sa.hi;
      }
      const float hw = sh.hi + sh.lo;
      hh = 2.0 * (double)hw;
      if (a.hp_list) {
        // the FP32 template's rounding: spread evenly over its N bins (a
        // random part ~ sqrt(hw_full rr / N), hw_full the power of the whole
        // template when the segment edge clips it, from the raw spectra's
        // power ratio) plus a systematic part along h (~ |(h|r - h)|, from
        // the FP32 per-proposal constants)
        const float hf = clipped && ev.z > 0.f ? hw * (ev.w / ev.z) : hw;
        const float he = sqrtf(fmaf(ev.x, ev.x, ev.y * ev.y));
        const float est = fmaf(a.fb_e1, sqrtf(hf * rr * (1.f / (float)N)), a.fb_e2 * he) *
                          fb_scale_of(a.fb_inv_scale, a.fb_nscale, item);
        if (!(est <= 1.f)) {  // also a non-finite estimate
          atomicAdd(a.fb_total, 1ull);
          atomicAdd(a.fb_count, 1);
          constexpr int bin = fd_bin_of(N);
          const int k = atomicAdd(&a.hp_count[bin], 1);
          if (chk(k < a.cap, kChkReevalList)) a.hp_list[(size_t)bin * a.cap + k] = item;
        }
      }
    } else {
      if constexpr (PERCH) {
        a.term_ch[2 * (size_t)item] = acc;
        a.term_ch[2 * (size_t)item + 1] = accE;
        term = acc + accE;
      } else {
        term = acc;
      }
      hh = 2.0 * hacc;
    }
    const double tx = a.term_x ? a.term_x[item] : 0.0;
    a.dlogl[item] = term - tx;
    if (a.term_y) a.term_y[item] = term;
    if (a.hh) a.hh[item] = hh;
    if (a.status) a.status[item] = isfinite(term) ? 0 : 1;
  }
  if constexpr (GT > 32) __syncthreads();
}

template <int N, bool MIX, bool PERCH = false>
__global__ void __launch_bounds__(SpecCfg<N>::CTA) fd_spec_kernel(SpecArgs a) {
  using Cfg = SpecCfg<N>;
  using S = SpecSmem<N, MIX>;
  using C = typename S::C;
  using TW = typename S::TW;
  constexpr int GPC = Cfg::GPC, NSER = S::NSER;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int SN = S::SN;
  TW *tw = reinterpret_cast<TW *>(smem_raw);
  C *bufs = reinterpret_cast<C *>(tw + SN);
  double *red = reinterpret_cast<double *>(bufs + (size_t)GPC * NSER * SN);

  const TW *twg = reinterpret_cast<const TW *>(a.tw);
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[MIX ? pad16(i) : i] = twg[i];
  __syncthreads();
  const int count = a.bin_count[a.bin];
  const C *series = reinterpret_cast<const C *>(a.series) + bin_sample_start(a.bin_count, a.NFFT, a.bin) * 4;
  for (int base = blockIdx.x * GPC; base < count; base += gridDim.x * GPC)
    spec_unit<N, MIX, GPC, PERCH>(a, a.bin_list, count, base, series, tw, bufs, red);
}

// ------------------------------------------- mixed spectral unit, size at run time
// The persistent spectral kernel runs units of six sizes side by side on every
// SM.  Instantiated per size, each unit is a separate fully unrolled copy of
// the FFT and the bin epilogue, and together they overflow the SM's
// instruction caches: a launch of the headline step missed in the per-SM
// instruction cache on ~40% of its fetches and its warps stalled on
// instruction fetch more than on any load.  The versions below take log2 N at
// run time, so every size shares one copy of the epilogue, the reductions and
// each radix's stage (the radix, which sets the register DFT, stays a
// template argument: 16 for the first stage of every size and the second of
// 256..1024, then 2, 4 or 8).  The arithmetic and its order are those of
// fft4_reg and the mixed branch of spec_unit.

__device__ __forceinline__ void group_sync_rt(int gt) {
  if (gt <= 32) {
    __syncwarp();
  } else {
    __syncthreads();
  }
}

// One Stockham stage of radix R (as reg_stage), sub-transform size P = 2^lp,
// on a padded series of N = 2^ln points.
template <int R, typename TW>
__device__ __forceinline__ void reg_stage_rt(float2 *y, const TW *tw, int t, float2 *v, int ln, int lp, int gt) {
  constexpr int NB = 16 / R, LR = ilog2c(R);
  const int M = 1 << (ln - 4), lstride = ln - LR, lts = ln - lp - LR, pm = (1 << lp) - 1;
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const int i = t + M * b, k = i & pm;
#pragma unroll
    for (int m = 0; m < R; ++m) {
      float2 val = y[pad16(i + (m << lstride))];
      if (m > 0) val = twmul(val, tw[pad16((m * k) << lts)]);
      v[b * R + m] = val;
    }
  }
  group_sync_rt(gt);  // every read of the stage before the in-place writes
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    dft_reg<R>(v + b * R);
    const int i = t + M * b, k = i & pm;
#pragma unroll
    for (int q = 0; q < R; ++q) y[pad16((i - k) * R + k + (q << lp))] = v[b * R + q];
  }
  group_sync_rt(gt);
}

// fft4_reg for N = 2^ln, 32 <= N <= 1024, by the group's GT = N/4 threads.
template <typename TW>
__device__ __forceinline__ void fft4_reg_rt(const float2 *src, float2 *sbuf, const TW *tw, int lane, int ln) {
  const int N = 1 << ln, M = N >> 4, gt = N >> 2;
  const int s = lane >> (ln - 4), t = lane & (M - 1);
  const float2 *x = src + (size_t)s * N;
  float2 *y = sbuf + s * pad16(N);
  float2 v[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) v[m] = x[t + m * M];
  dft_reg<16>(v);
#pragma unroll
  for (int q = 0; q < 16; ++q) y[pad16(t * 16 + q)] = v[q];
  group_sync_rt(gt);
  if (ln >= 8) {
    reg_stage_rt<16>(y, tw, t, v, ln, 4, gt);
    if (ln == 9) {
      reg_stage_rt<2>(y, tw, t, v, ln, 8, gt);
    } else if (ln == 10) {
      reg_stage_rt<4>(y, tw, t, v, ln, 8, gt);
    }
  } else if (ln == 7) {
    reg_stage_rt<8>(y, tw, t, v, ln, 4, gt);
  } else if (ln == 6) {
    reg_stage_rt<4>(y, tw, t, v, ln, 4, gt);
  } else {
    reg_stage_rt<2>(y, tw, t, v, ln, 4, gt);
  }
}

// group_sum_df / group_sum4 for a group of gt threads.
__device__ __forceinline__ df group_sum_df_rt(df s, float2 *red, int lane, int gt) {
  for (int off = (gt < 32 ? gt : 32) >> 1; off > 0; off >>= 1) {
    df o = {__shfl_xor_sync(0xffffffffu, s.hi, off), __shfl_xor_sync(0xffffffffu, s.lo, off)};
    s = df_add(s, o);
  }
  if (gt > 32) {
    __syncthreads();
    if ((lane & 31) == 0) red[lane >> 5] = make_float2(s.hi, s.lo);
    __syncthreads();
    if (lane == 0) {
      df t = {0.f, 0.f};
      for (int w = 0; w < gt / 32; w++) t = df_add(t, df{red[w].x, red[w].y});
      s = t;
    }
  }
  return s;
}
__device__ __forceinline__ float4 group_sum4_rt(float4 v, float *red, int lane, int gt) {
  for (int off = (gt < 32 ? gt : 32) >> 1; off > 0; off >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, off);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, off);
    v.z += __shfl_xor_sync(0xffffffffu, v.z, off);
    v.w += __shfl_xor_sync(0xffffffffu, v.w, off);
  }
  if (gt > 32) {
    __syncthreads();
    if ((lane & 31) == 0) {
      float *o = red + 4 * (lane >> 5);
      o[0] = v.x;
      o[1] = v.y;
      o[2] = v.z;
      o[3] = v.w;
    }
    __syncthreads();
    if (lane == 0) {
      v = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int w = 0; w < gt / 32; w++) {
        v.x += red[4 * w];
        v.y += red[4 * w + 1];
        v.z += red[4 * w + 2];
        v.w += red[4 * w + 3];
      }
    }
  }
  return v;
}

// The mixed branch of spec_unit for N = 2^ln (32 <= N <= 1024): 1024/N
// proposals of the unit, one group of N/4 threads each, in a 256-thread CTA.
template <bool PERCH>
__device__ __forceinline__ void spec_unit_mix_rt(const SpecArgs &a, const int *bin_list, int count, int base, int ln,
                                                 const float2 *series, const float4 *tw, float2 *bufs,
                                                 double *reds) {
  const int N = 1 << ln, GT = N >> 2, SN = pad16(N);
  constexpr int B = 4;  // bins per thread
  const int g = threadIdx.x >> (ln - 2), lane = threadIdx.x & (GT - 1);
  float2 *buf = bufs + (size_t)g * 4 * SN;
  double *red = reds + 96 * g;
  const int NFFT = a.NFFT;
  const int slot = base + g;
  const bool valid = slot < count;
  const int sl = valid ? slot : count - 1;
  // checked build: as in spec_unit
  const bool lok = chk(sl >= 0 && sl < a.cap, kChkBinList);
  const int item = lok ? bin_list[sl] : 0;
  const bool iok = chk(item >= 0 && item < a.nitems, kChkItem);
  int seg = 0, imin = 0;
  if (iok) {
    seg = a.itemsmix[item].seg;
    imin = a.itemsmix[item].imin;
  }
  const bool sok = chk(seg >= 0 && seg < a.nseg, kChkBankRead);
  const bool rok = chk((long long)(sl + 1) * 4 * N <= a.series_len, kChkSeriesRead);
  const bool inb = lok && iok && sok && rok;
  if (!inb) seg = 0;
  const float2 *src = series + (inb ? (size_t)sl * 4 * N : 0);
  const bool est_on = a.hp_list != nullptr;
  const bool clipped = imin < 0 || imin + N > NFFT;
  float rS = 0.f, rE = 0.f, eS = 0.f, eE = 0.f, fh = 0.f;
  float4 ev = make_float4(0.f, 0.f, 0.f, 0.f);
  fft4_reg_rt(src, buf, tw, lane, ln);
#pragma unroll
  for (int r = 0; r < B; ++r) {
    const int k = lane + GT * r;
    const int m = (k + N / 2) & (N - 1);  // fftshift: output bin m holds FFT index m + N/2
    const int j = imin + m;
    const int kp = pad16(k);
    const float2 b0 = buf[0 * SN + kp], b1 = buf[1 * SN + kp], b2 = buf[2 * SN + kp], b3 = buf[3 * SN + kp];
    const bool inside = j >= 0 && j < NFFT;
    if (est_on && clipped) {
      const float pw = fmaf(b0.x, b0.x, fmaf(b0.y, b0.y, fmaf(b1.x, b1.x, fmaf(b1.y, b1.y,
                       fmaf(b2.x, b2.x, fmaf(b2.y, b2.y, fmaf(b3.x, b3.x, b3.y * b3.y)))))));
      ev.w += pw;
      if (inside) ev.z += pw;
    }
    if (!inside) continue;
    const size_t sj = (size_t)seg * NFFT + j;
    const float4 w = a.w32[sj], wl = a.w32lo[sj];
    const float4 gA = a.g32[2 * sj], gE = a.g32[2 * sj + 1];
    const float4 gAl = a.g32lo[2 * sj], gEl = a.g32lo[2 * sj + 1];
    const float p2 = a.itemsmix[item].amp_p2;
    const float2 HA = cfma(b0, make_float2(gA.x, gA.y),
                           cfma(b1, make_float2(gA.z, gA.w),
                                cfma(b0, make_float2(gAl.x, gAl.y), cmul(b1, make_float2(gAl.z, gAl.w)))));
    const float2 HE = cfma(b2, make_float2(gE.x, gE.y),
                           cfma(b3, make_float2(gE.z, gE.w),
                                cfma(b2, make_float2(gEl.x, gEl.y), cmul(b3, make_float2(gEl.z, gEl.w)))));
    const float2 hA = cscale(HA, p2), hE = cscale(HE, p2);
    acc_resid_sq(w.x, wl.x, hA.x, rS, eS);
    acc_resid_sq(w.y, wl.y, hA.y, rS, eS);
    acc_resid_sq(w.z, wl.z, hE.x, rE, eE);
    acc_resid_sq(w.w, wl.w, hE.y, rE, eE);
    fh += fmaf(hA.x, hA.x, hA.y * hA.y) + fmaf(hE.x, hE.x, hE.y * hE.y);
    if (est_on) {
      const float dAx = w.x - hA.x, dAy = w.y - hA.y, dEx = w.z - hE.x, dEy = w.w - hE.y;
      ev.x += fmaf(hA.x, dAx, fmaf(hA.y, dAy, fmaf(hE.x, dEx, hE.y * dEy)));
      ev.y += fmaf(hA.x, dAy, fmaf(-hA.y, dAx, fmaf(hE.x, dEy, -hE.y * dEx)));
    }
  }
  group_sync_rt(GT);
  df sa, sh, saE;
  float2 *redf = reinterpret_cast<float2 *>(red);
  if constexpr (PERCH) {
    sa = group_sum_df_rt(quick_two_sum(rS, eS), redf, lane, GT);
    saE = group_sum_df_rt(quick_two_sum(rE, eE), redf + 64, lane, GT);
  } else {
    sa = group_sum_df_rt(df_add(quick_two_sum(rS, eS), quick_two_sum(rE, eE)), redf, lane, GT);
  }
  sh = group_sum_df_rt(df{fh, 0.f}, redf + 32, lane, GT);
  if (est_on) ev = group_sum4_rt(ev, reinterpret_cast<float *>(red), lane, GT);
  if (valid && inb && lane == 0) {
    double term, hh;
    // FP64 only for the final sum, once per proposal
    int jlo = imin < 0 ? 0 : imin;
    int jhi = imin + N > NFFT ? NFFT : imin + N;
    const double *Qs = a.Q + (size_t)seg * (NFFT + 1);
    float rr;  // |r - h|^2 over the support, both channels
    if constexpr (PERCH) {
      const double *QAs = a.QA + (size_t)seg * (NFFT + 1);
      const double qa = QAs[jhi] - QAs[jlo];
      const double tA = (qa - (double)sa.hi) - (double)sa.lo;
      const double tE = (((Qs[jhi] - Qs[jlo]) - qa) - (double)saE.hi) - (double)saE.lo;
      a.term_ch[2 * (size_t)item] = tA;
      a.term_ch[2 * (size_t)item + 1] = tE;
      term = tA + tE;
      rr = sa.hi + saE.hi;
    } else {
      term = ((Qs[jhi] - Qs[jlo]) - (double)sa.hi) - (double)sa.lo;
      rr = sa.hi;
    }
    const float hw = sh.hi + sh.lo;
    hh = 2.0 * (double)hw;
    if (a.hp_list) {
      // the error estimate of spec_unit
      const float hf = clipped && ev.z > 0.f ? hw * (ev.w / ev.z) : hw;
      const float he = sqrtf(fmaf(ev.x, ev.x, ev.y * ev.y));
      const float est = fmaf(a.fb_e1, sqrtf(hf * rr * (1.f / (float)N)), a.fb_e2 * he) *
                        fb_scale_of(a.fb_inv_scale, a.fb_nscale, item);
      if (!(est <= 1.f)) {  // also a non-finite estimate
        atomicAdd(a.fb_total, 1ull);
        atomicAdd(a.fb_count, 1);
        const int bin = ln - 5;
        const int k = atomicAdd(&a.hp_count[bin], 1);
        if (chk(k < a.cap, kChkReevalList)) a.hp_list[(size_t)bin * a.cap + k] = item;
      }
    }
    const double tx = a.term_x ? a.term_x[item] : 0.0;
    a.dlogl[item] = term - tx;
    if (a.term_y) a.term_y[item] = term;
    if (a.hh) a.hh[item] = hh;
    if (a.status) a.status[item] = isfinite(term) ? 0 : 1;
  }
  if (GT > 32) __syncthreads();
}

// All sizes up to 1024 in one launch: a persistent grid of 256-thread CTAs
// walks the units (GPC = 1024/N proposals of one size each), largest sizes
// first so that the long units start early; a CTA reloads the twiddles when
// it changes size.  Shared memory: twiddles for 1024 points, 4 x 1024 series
// values and four groups' reduction scratch, whatever the size.
constexpr int kSpecAllThreads = 256;
constexpr int kSpecAllBins = 6;  // N = 32 .. 1024

template <bool MIX>
struct SpecAllSmem {
  using C = typename std::conditional<MIX, float2, double2>::type;
  using TW = typename std::conditional<MIX, float4, double2>::type;
  static constexpr int SN = MIX ? pad16(1024) : 1024;  // mixed: padded rows
  static constexpr size_t bytes = sizeof(TW) * SN + sizeof(C) * 4 * SN + sizeof(double) * 96 * 4;
};

struct SpecAllArgs {
  SpecArgs a;                    // a.bin_list: all sizes' lists, stride cap; a.tw unused
  const void *tw[kSpecAllBins];  // twiddles per size
  int nbins;                     // sizes 32 << b for b < nbins
  int *zero_counts;              // non-null: the last CTA to finish zeroes the kNumBins counts there
  int *done = nullptr;           // CTA-done counter (zero between launches)
};

template <bool MIX, bool PERCH = false>
__global__ void __launch_bounds__(kSpecAllThreads, 4) fd_spec_all_kernel(SpecAllArgs A) {
  using C = typename SpecAllSmem<MIX>::C;
  using TW = typename SpecAllSmem<MIX>::TW;
  const SpecArgs &a = A.a;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int SN = SpecAllSmem<MIX>::SN;
  TW *tw = reinterpret_cast<TW *>(smem_raw);
  C *bufs = reinterpret_cast<C *>(tw + SN);
  double *reds = reinterpret_cast<double *>(bufs + 4 * SN);
  // unit ranges per size, largest first; in shared memory so that they hold
  // no registers while a unit runs
  __shared__ int ustart[kSpecAllBins + 1];
  if (threadIdx.x == 0) {
    int total = 0;
#pragma unroll
    for (int q = 0; q < kSpecAllBins; q++) {
      const int b = kSpecAllBins - 1 - q;
      ustart[q] = total;
      if (b < A.nbins) {
        const int gpc = 32 >> b;
        total += (a.bin_count[b] + gpc - 1) / gpc;
      }
    }
    ustart[kSpecAllBins] = total;
  }
  __syncthreads();
  const int total = ustart[kSpecAllBins];
  int cur = -1;
  for (int unit = blockIdx.x; unit < total; unit += gridDim.x) {
    int q = 0;
#pragma unroll
    for (int qq = 1; qq < kSpecAllBins; qq++)
      if (unit >= ustart[qq]) q = qq;
    const int b = kSpecAllBins - 1 - q;
    const int N = 32 << b;
    if (b != cur) {
      __syncthreads();
      const TW *twg = reinterpret_cast<const TW *>(A.tw[b]);
      for (int i = threadIdx.x; i < N; i += blockDim.x) tw[MIX ? pad16(i) : i] = twg[i];
      __syncthreads();
      cur = b;
    }
    const int gpc = 32 >> b;
    const int base = (unit - ustart[q]) * gpc;
    const int count = a.bin_count[b];
    const int *bl = a.bin_list + (size_t)b * a.cap;
    const C *series = reinterpret_cast<const C *>(a.series) + bin_sample_start(a.bin_count, a.NFFT, b) * 4;
    if constexpr (MIX) {
      spec_unit_mix_rt<PERCH>(a, bl, count, base, b + 5, series, tw, bufs, reds);
      continue;
    }
    switch (b) {
      case 0: spec_unit<32, MIX, 32, PERCH>(a, bl, count, base, series, tw, bufs, reds); break;
      case 1: spec_unit<64, MIX, 16, PERCH>(a, bl, count, base, series, tw, bufs, reds); break;
      case 2: spec_unit<128, MIX, 8, PERCH>(a, bl, count, base, series, tw, bufs, reds); break;
      case 3: spec_unit<256, MIX, 4, PERCH>(a, bl, count, base, series, tw, bufs, reds); break;
      case 4: spec_unit<512, MIX, 2, PERCH>(a, bl, count, base, series, tw, bufs, reds); break;
      default: spec_unit<1024, MIX, 1, PERCH>(a, bl, count, base, series, tw, bufs, reds); break;
    }
  }
  // the last CTA to finish leaves the size counts at zero for the next
  // launch sequence (every CTA has read them for the last time once it gets
  // here) and resets its done counter
  if (A.zero_counts) {
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      if (atomicAdd(A.done, 1) == (int)gridDim.x - 1) {
#pragma unroll
        for (int b = 0; b < kNumBins; b++) A.zero_counts[b] = 0;
        *A.done = 0;
      }
    }
  }
}

template <bool MIX, bool PERCH = false>
static cudaError_t launch_spec_all(const SpecAllArgs &A, int num_sms, cudaStream_t stream, int cap = 0) {
  const size_t smem = SpecAllSmem<MIX>::bytes;
  static LaunchSetup setup;
  int occ = 0;
  cudaError_t e = launch_setup(setup, [&](int *o) {
    cudaError_t r = cudaFuncSetAttribute(fd_spec_all_kernel<MIX, PERCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (r != cudaSuccess) return r;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, fd_spec_all_kernel<MIX, PERCH>, kSpecAllThreads, smem);
  }, &occ);
  if (e != cudaSuccess) return e;
  if (cap > 0 && cap < occ) occ = cap;
  fd_spec_all_kernel<MIX, PERCH><<<occ * num_sms, kSpecAllThreads, smem, stream>>>(A);
  return cudaGetLastError();
}

// Launch of one size's kernel with a grid bounded by the SM count times the
// occupancy of the kernel.
template <int N, bool MIX, bool PERCH = false>
static cudaError_t launch_spec(const SpecArgs &a, int nitems_bound, int num_sms, cudaStream_t stream) {
  using Cfg = SpecCfg<N>;
  size_t smem = SpecSmem<N, MIX>::bytes;
  static LaunchSetup setup;
  int occ = 0;
  cudaError_t e = launch_setup(setup, [&](int *o) {
    cudaError_t r = cudaFuncSetAttribute(fd_spec_kernel<N, MIX, PERCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (r != cudaSuccess) return r;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, fd_spec_kernel<N, MIX, PERCH>, Cfg::CTA, smem);
  }, &occ);
  if (e != cudaSuccess) return e;
  int need = (nitems_bound + Cfg::GPC - 1) / Cfg::GPC;
  int grid = occ * num_sms;
  if (need < grid) grid = need;
  if (grid < 1) grid = 1;
  fd_spec_kernel<N, MIX, PERCH><<<grid, Cfg::CTA, smem, stream>>>(a);
  return cudaGetLastError();
}

template <bool MIX, int BLOCK = 256>
static cudaError_t launch_slow(const SlowArgs &a, int num_sms, cudaStream_t stream, int cap = 0) {
  static LaunchSetup setup;
  int occ = 0;
  cudaError_t e = launch_setup(setup, [&](int *o) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, fd_slow_kernel<MIX, BLOCK>, BLOCK, 0);
  }, &occ);
  if (e != cudaSuccess) return e;
  if (cap > 0 && cap < occ) occ = cap;
  fd_slow_kernel<MIX, BLOCK><<<occ * num_sms, BLOCK, 0, stream>>>(a);
  return cudaGetLastError();
}

// The slow part of a few proposals (the FP64 re-evaluation of flagged mixed
// ones): one warp per CTA, so that the chunks of 32 samples spread over the
// SMs instead of filling the first few (an FP64 sample costs ~700 FP64
// instructions and the FP64 pipe of an SM issues a warp's in 16 cycles).

}  // namespace glass
