// Double-float (pairs of floats) arithmetic: complex operations, division,
// sine, cosine and sinc, the CTA-wide Stockham FFT and reduction, and the
// result write of the double-float re-evaluation of mixed proposals
// (ucb_fd_hp.cu).
#pragma once
#include "glass_common.cuh"

namespace glass {

struct dc {
  df re, im;
};
__device__ __forceinline__ dc dc_add(dc a, dc b) { return {df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ dc dc_sub(dc a, dc b) { return {df_add(a.re, df_neg(b.re)), df_add(a.im, df_neg(b.im))}; }
__device__ __forceinline__ dc dc_mul(dc a, dc b) {
  return {df_add(df_mul(a.re, b.re), df_neg(df_mul(a.im, b.im))), df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
__device__ __forceinline__ dc dc_mi(dc a) { return {a.im, df_neg(a.re)}; }  // -i a
// complex hi + lo floats (x, y: hi; z, w: lo), as the tables store them: no
// FP64 conversion in the inner loops (GB300's FP64 pipe runs at 1/64 rate)
__device__ __forceinline__ dc dc_from(float4 v) { return {{v.x, v.z}, {v.y, v.w}}; }
__device__ __forceinline__ dc dc_from(float2 hi, float2 lo) { return {{hi.x, lo.x}, {hi.y, lo.y}}; }
__device__ __forceinline__ df df_sq_sum(dc a) { return df_add(df_mul(a.re, a.re), df_mul(a.im, a.im)); }
// a times an exact power of two
__device__ __forceinline__ dc dc_scale2(dc a, float p2) {
  return {{a.re.hi * p2, a.re.lo * p2}, {a.im.hi * p2, a.im.lo * p2}};
}
__device__ __forceinline__ dc dc_scale(dc a, df s) { return {df_mul(a.re, s), df_mul(a.im, s)}; }

// Double-float division (one Newton correction of the float quotient).
__device__ __forceinline__ df df_div(df a, df b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const df r = df_add(a, df_neg(df_mul_f(b, q1)));
  return quick_two_sum(q1, __fdiv_rn(r.hi, b.hi));
}

// Inverse factorials 1/n! as hi + lo floats, n = 0..19 (the Taylor
// coefficients of sin and cos).
__device__ __forceinline__ df inv_fact(int n) {
  switch (n) {
    case 0: case 1: return {1.f, 0.f};
    case 2: return {0.5f, 0.f};
    case 3: return {0.1666666716337204f, -4.967053879312289e-09f};
    case 4: return {0.0416666679084301f, -1.2417634698280722e-09f};
    case 5: return {0.008333333767950535f, -4.34617203337595e-10f};
    case 6: return {0.0013888889225199819f, -3.3631094437103215e-11f};
    case 7: return {0.00019841270113829523f, -2.725596874933456e-12f};
    case 8: return {2.4801587642286904e-05f, -3.40699609366682e-13f};
    case 9: return {2.7557318844628753e-06f, 3.793571224297229e-14f};
    case 10: return {2.755731998149713e-07f, -7.575112209051195e-15f};
    case 11: return {2.5052107943679403e-08f, 4.4176230446483665e-16f};
    case 12: return {2.0876755879584152e-09f, 1.1082839147459852e-16f};
    case 13: return {1.6059044372074283e-10f, -5.352526511562726e-18f};
    case 14: return {1.147074536050896e-11f, 2.372207689231238e-19f};
    case 15: return {7.647163609812713e-13f, 1.2200710471178288e-20f};
    case 16: return {4.7794772561329454e-14f, 7.62544404448643e-22f};
    case 17: return {2.8114573589663704e-15f, -1.0462084739763658e-22f};
    case 18: return {1.5619206814541513e-16f, 1.5404471465941993e-24f};
    default: return {8.220635078476521e-18f, 1.681478096855898e-25f};
  }
}

// sum_k (-1)^k x2^k / (2k + first)!, k = 0..terms-1, by Horner in
// double-float (first = 1: sin(x)/x; first = 0: cos x).
template <int FIRST, int TERMS>
__device__ __forceinline__ df df_alt_series(df x2) {
  df p = inv_fact(2 * (TERMS - 1) + FIRST);
  if ((TERMS - 1) & 1) p = df_neg(p);
#pragma unroll
  for (int k = TERMS - 2; k >= 0; k--) {
    df c = inv_fact(2 * k + FIRST);
    if (k & 1) c = df_neg(c);
    p = df_add(df_mul(p, x2), c);
  }
  return p;
}

// sin and cos of a double-float angle of at most a few tens of radians:
// reduction by pi/2 (three-part constant, exact products of the quadrant
// count), then the Taylor series of sin (through r^17) and cos (through
// r^16) on r in [-pi/4, pi/4] (truncation below 1e-16).
__device__ __forceinline__ void df_sincos(df x, df *s, df *c) {
  const float q = rintf(x.hi * 0.63661977236758134f);
  df r = df_add(x, df_neg(two_prod(q, 1.5707963705062866f)));
  r = df_add(r, df_neg(two_prod(q, -4.371138828673793e-08f)));
  r = df_add(r, df{q * 1.7151245100058819e-15f, 0.f});
  const df r2 = df_mul(r, r);
  const df sr = df_mul(r, df_alt_series<1, 9>(r2));
  const df cr = df_alt_series<0, 9>(r2);
  const int qi = ((int)q) & 3;
  const df ss = (qi & 1) ? cr : sr;
  const df cc = (qi & 1) ? sr : cr;
  *s = (qi & 2) ? df_neg(ss) : ss;
  *c = ((qi + 1) & 2) ? df_neg(cc) : cc;
}

// sin and cos of a double-float angle with a table: tab[k] = (sin, cos) of
// k pi/32 as hi + lo floats (float4: sin hi, sin lo, cos hi, cos lo), k mod
// 64; x = k pi/32 + d with |d| <= pi/64 (three-part pi/32), whose sine
// (through d^7) and cosine (through d^8) have truncation errors below 1e-15;
// then the angle-sum formulas.
__device__ __forceinline__ void df_sincos_tab(df x, const float4 *tab, df *s, df *c) {
  const float q = rintf(x.hi * 10.185916357881302f);  // 32/pi
  df d = df_add(x, df_neg(two_prod(q, 0.09817477315664291f)));
  d = df_add(d, df_neg(two_prod(q, -2.7319617679211206e-09f)));
  d = df_add(d, df{q * 1.0719528187536762e-16f, 0.f});
  const df d2 = df_mul(d, d);
  const df sd = df_mul(d, df_alt_series<1, 4>(d2));
  const df cd = df_alt_series<0, 5>(d2);
  const float4 t = tab[((int)q) & 63];
  const df sk = {t.x, t.y}, ck = {t.z, t.w};
  *s = df_add(df_mul(sk, cd), df_mul(ck, sd));
  *c = df_add(df_mul(ck, cd), df_neg(df_mul(sk, sd)));
}

// sin(x)/x in double-float: Taylor series through x^12 for |x| <= 1/2 and
// through x^18 for |x| <= 1 (truncation below 1e-17), sin x / x beyond.
__device__ __forceinline__ df df_sinc(df x, const float4 *tab) {
  const float ax = fabsf(x.hi);
  if (ax <= 0.5f) return df_alt_series<1, 7>(df_mul(x, x));
  if (ax <= 1.f) return df_alt_series<1, 10>(df_mul(x, x));
  df s, c;
  df_sincos_tab(x, tab, &s, &c);
  return df_div(s, x);
}

// Stockham FFT of one series of N double-floats by the CTA, ping-ponging
// between x and y: radix-4 stages (sub-transform size p: butterfly i < N/4,
// k = i mod p, reads x[i + m N/4], m = 0..3, times exp(-2 pi i m k / (4p)),
// writes y[(i - k) 4 + k + m p]) and a final radix-2 stage when log2 N is
// odd.  tw[j] = exp(-2 pi i j / N) as hi + lo floats.  Returns the buffer
// holding the result.
__device__ __forceinline__ dc *hp_fft(dc *x, dc *y, int N, const float4 *tw) {
  int p = 1;
  for (; 4 * p <= N; p <<= 2) {
    const int step = N / (4 * p), q = N / 4;
    for (int i = threadIdx.x; i < q; i += blockDim.x) {
      const int k = i & (p - 1);
      dc u0 = x[i], u1 = x[i + q], u2 = x[i + 2 * q], u3 = x[i + 3 * q];
      if (p > 1) {
        u1 = dc_mul(u1, dc_from(tw[k * step]));
        u2 = dc_mul(u2, dc_from(tw[2 * k * step]));
        u3 = dc_mul(u3, dc_from(tw[3 * k * step]));
      }
      const dc a = dc_add(u0, u2), b = dc_sub(u0, u2), c = dc_add(u1, u3), d = dc_mi(dc_sub(u1, u3));
      const int j = (i - k) * 4 + k;
      y[j] = dc_add(a, c);
      y[j + p] = dc_add(b, d);
      y[j + 2 * p] = dc_sub(a, c);
      y[j + 3 * p] = dc_sub(b, d);
    }
    __syncthreads();
    dc *t = x;
    x = y;
    y = t;
  }
  if (p < N) {  // log2 N odd: one radix-2 stage, p = N/2
    for (int i = threadIdx.x; i < N / 2; i += blockDim.x) {
      const int k = i & (p - 1);
      const dc a = x[i], b = dc_mul(x[i + N / 2], dc_from(tw[k]));
      const int j = (i - k) * 2 + k;
      y[j] = dc_add(a, b);
      y[j + p] = dc_sub(a, b);
    }
    __syncthreads();
    dc *t = x;
    x = y;
    y = t;
  }
  return x;
}

// Sum over the CTA of a double-float per thread (valid in thread 0).
static __device__ df hp_block_sum(df v, float2 *red) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    df o = {__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off)};
    v = df_add(v, o);
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_float2(v.hi, v.lo);
  __syncthreads();
  df t = {0.f, 0.f};
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t = df_add(t, df{red[w].x, red[w].y});
  return t;
}

// Writes a re-evaluated proposal's results (thread 0), as the spectral
// kernels do; returns term_y.
__device__ __forceinline__ double hp_write(int item, int N, int seg, int imin, int NFFT, const df s[3],
                                           const double *Q, const double *QA, bool perch, const double *term_x,
                                           double *dlogl, double *term_y, double *hh, double *term_ch,
                                           int *status) {
  const int jlo = imin < 0 ? 0 : imin;
  const int jhi = imin + N > NFFT ? NFFT : imin + N;
  const double *Qs = Q + (size_t)seg * (NFFT + 1);
  double term;
  if (perch) {
    const double *QAs = QA + (size_t)seg * (NFFT + 1);
    const double qa = QAs[jhi] - QAs[jlo];
    const double tA = (qa - (double)s[0].hi) - (double)s[0].lo;
    const double tE = (((Qs[jhi] - Qs[jlo]) - qa) - (double)s[1].hi) - (double)s[1].lo;
    term_ch[2 * (size_t)item] = tA;
    term_ch[2 * (size_t)item + 1] = tE;
    term = tA + tE;
  } else {
    const df r = df_add(s[0], s[1]);
    term = ((Qs[jhi] - Qs[jlo]) - (double)r.hi) - (double)r.lo;
  }
  const double tx = term_x ? term_x[item] : 0.0;
  dlogl[item] = term - tx;
  if (term_y) term_y[item] = term;
  if (hh) hh[item] = 2.0 * ((double)s[2].hi + (double)s[2].lo);
  if (status) status[item] = isfinite(term) ? 0 : 1;
  return term;
}

}  // namespace glass
