// Double-float (pairs of floats) complex arithmetic, the CTA-wide Stockham
// FFT and reduction, and the result write of the double-float re-evaluation
// of mixed proposals (ucb_fd_hp.cu).
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
