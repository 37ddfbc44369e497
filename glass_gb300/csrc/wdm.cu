// WDM (Wilson-Daubechies-Meyer) wavelet transforms for sm_103a.
//
// Forward (utils/src/glass_wavelet.c:293-303 and :410-460): a real FFT of the
// ND = NF*NT samples, then for every layer m = 0..NF the NT-1 FFT bins around
// m NT/2, weighted by the Meyer window, inverse-FFT'd over NT points; the
// layer's NT coefficients are the real or imaginary parts by the parity of
// n + m (layout wdm[n + NT m], DC and Nyquist layers packed into row 0).
// Inverse (:351-405 and utils/src/glass_math.c:819-828): per layer an NT-point
// FFT of the coefficients, windowed overlap-add into the ND/2+1 bins, inverse
// real FFT.
//
// GPU structure:
//  * the real FFT of ND samples is a complex FFT of M = ND/2 packed samples
//    (x[2n] + i x[2n+1]), done four-step as M1 x M2: FFTs down the M2 columns
//    with the exp(-2 pi i n2 k1 / M) twiddle folded in, then FFTs along the M1
//    rows; the real spectrum is unpacked on the fly where it is read;
//  * one CTA per layer for the windowed NT-point transforms;
//  * the inverse overlap-add runs in two launches (even, then odd layers): the
//    supports of same-parity layers are disjoint, so no atomics are needed and
//    the sum order is fixed;
//  * all FFTs are mixed-radix (3, 4, 2) Stockham transforms in shared memory
//    with ping-pong buffers, so NF = 1536 (the reference's default grid) works.
// Templated on the arithmetic type: FP64 (parity with the reference) and FP32.
#include <math.h>

#include <mutex>
#include <type_traits>
#include <vector>

#include "wdm.cuh"

namespace glass {
namespace {

template <typename R>
struct Cx;
template <>
struct Cx<double> {
  using T = double2;
};
template <>
struct Cx<float> {
  using T = float2;
};

template <typename C>
__device__ __forceinline__ C cm(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename C>
__device__ __forceinline__ C ca(C a, C b) {
  C r;
  r.x = a.x + b.x;
  r.y = a.y + b.y;
  return r;
}
template <typename C>
__device__ __forceinline__ C cs(C a, C b) {
  C r;
  r.x = a.x - b.x;
  r.y = a.y - b.y;
  return r;
}
template <typename C>
__device__ __forceinline__ C cconj(C a) {
  a.y = -a.y;
  return a;
}
template <typename C, typename R>
__device__ __forceinline__ C csc(C a, R s) {
  a.x *= s;
  a.y *= s;
  return a;
}
template <typename C>
__device__ __forceinline__ C mk(decltype(C().x) x, decltype(C().x) y) {
  C r;
  r.x = x;
  r.y = y;
  return r;
}

// e^{sign 2 pi i p / P} from two tables: lo[j] = e^{-2 pi i j/P} (j < K) and
// hi[j] = e^{-2 pi i j K/P}, p = hi K + lo.
template <typename C>
__device__ __forceinline__ C twiddle2(const C *lo, const C *hi, long long p, int K, int sign) {
  C t = cm(hi[p / K], lo[p % K]);
  return sign > 0 ? cconj(t) : t;
}

// In-place-looking mixed-radix Stockham FFT of nser series of length L stored
// series-major in a; b is a scratch buffer of the same size; tw[j] =
// exp(-2 pi i j / L).  All threads of the CTA take part.  Returns the buffer
// holding the result.  sign -1: forward, +1: inverse (unnormalised).
template <typename C>
__device__ C *block_fft(C *a, C *b, int L, int nser, const C *tw, int sign) {
  using R = decltype(C().x);
  int p = 1, rem = L;
  const R s3 = (R)0.86602540378443864676;  // sin(2 pi/3)
  while (rem > 1) {
    const int Rd = (rem % 3 == 0) ? 3 : (rem % 4 == 0) ? 4 : 2;
    const int nb = L / Rd;
    const int step = L / (p * Rd);
    for (int t = threadIdx.x; t < nser * nb; t += blockDim.x) {
      const int s = t / nb, i = t - s * nb;
      const int k = i % p;
      const C *src = a + (size_t)s * L;
      C *dst = b + (size_t)s * L;
      const int j = (i - k) * Rd + k;
      if (Rd == 4) {
        C v0 = src[i], v1 = src[i + nb], v2 = src[i + 2 * nb], v3 = src[i + 3 * nb];
        C w1 = tw[k * step], w2 = tw[2 * k * step], w3 = tw[3 * k * step];
        if (sign > 0) {
          w1 = cconj(w1);
          w2 = cconj(w2);
          w3 = cconj(w3);
        }
        v1 = cm(v1, w1);
        v2 = cm(v2, w2);
        v3 = cm(v3, w3);
        C t0 = ca(v0, v2), t1 = cs(v0, v2), t2 = ca(v1, v3), t3 = cs(v1, v3);
        // t3 * (-i sign): forward uses -i
        C t3r = sign < 0 ? mk<C>(t3.y, -t3.x) : mk<C>(-t3.y, t3.x);
        dst[j] = ca(t0, t2);
        dst[j + p] = ca(t1, t3r);
        dst[j + 2 * p] = cs(t0, t2);
        dst[j + 3 * p] = cs(t1, t3r);
      } else if (Rd == 2) {
        C v0 = src[i], v1 = src[i + nb];
        C w1 = tw[k * step];
        if (sign > 0) w1 = cconj(w1);
        v1 = cm(v1, w1);
        dst[j] = ca(v0, v1);
        dst[j + p] = cs(v0, v1);
      } else {
        C v0 = src[i], v1 = src[i + nb], v2 = src[i + 2 * nb];
        C w1 = tw[k * step], w2 = tw[2 * k * step];
        if (sign > 0) {
          w1 = cconj(w1);
          w2 = cconj(w2);
        }
        v1 = cm(v1, w1);
        v2 = cm(v2, w2);
        // radix-3 DFT with w = exp(sign 2 pi i / 3) = -1/2 + i sign sqrt(3)/2
        C sum = ca(v1, v2), dif = cs(v1, v2);
        C y0 = ca(v0, sum);
        C m1 = mk<C>(v0.x - (R)0.5 * sum.x, v0.y - (R)0.5 * sum.y);
        C m2 = mk<C>(-(R)sign * s3 * dif.y, (R)sign * s3 * dif.x);  // i sign sqrt3/2 dif
        dst[j] = y0;
        dst[j + p] = ca(m1, m2);
        dst[j + 2 * p] = cs(m1, m2);
      }
    }
    __syncthreads();
    C *tmp = a;
    a = b;
    b = tmp;
    p *= Rd;
    rem /= Rd;
  }
  return a;
}

template <typename C>
__device__ void load_twiddles(C *tw, const C *twg, int L) {
  for (int i = threadIdx.x; i < L; i += blockDim.x) tw[i] = twg[i];
}

// Four-step pass 1: FFTs of length M1 down ncol adjacent columns (stride M2)
// of src, times exp(sign 2 pi i n2 k1/M), written to dst at the same
// positions.  src may be the real input viewed as packed complex samples.
template <typename C>
__global__ void wdm_col_kernel(const C *src, C *dst, int M1, int M2, int ncol, const C *tw1, const C *tlo,
                               const C *thi, int K, int sign) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  C *tw = reinterpret_cast<C *>(sm_raw);
  C *a = tw + M1;
  C *b = a + (size_t)ncol * M1;
  load_twiddles(tw, tw1, M1);
  const int c0 = blockIdx.x * ncol;
  for (int t = threadIdx.x; t < ncol * M1; t += blockDim.x) {
    const int n1 = t / ncol, c = t - n1 * ncol;
    a[(size_t)c * M1 + n1] = src[(size_t)n1 * M2 + c0 + c];
  }
  __syncthreads();
  C *r = block_fft(a, b, M1, ncol, tw, sign);
  const long long M = (long long)M1 * M2;
  for (int t = threadIdx.x; t < ncol * M1; t += blockDim.x) {
    const int k1 = t / ncol, c = t - k1 * ncol;
    const long long p = ((long long)(c0 + c) * k1) % M;
    dst[(size_t)k1 * M2 + c0 + c] = cm(r[(size_t)c * M1 + k1], twiddle2(tlo, thi, p, K, sign));
  }
}

// Four-step pass 2: FFTs of length M2 along nrow rows of src; output index
// k1 + M1 k2 (natural order), times `scale`.
template <typename C>
__global__ void wdm_row_kernel(const C *src, C *dst, int M1, int M2, int nrow, const C *tw2, int sign,
                               decltype(C().x) scale) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  C *tw = reinterpret_cast<C *>(sm_raw);
  C *a = tw + M2;
  C *b = a + (size_t)nrow * M2;
  load_twiddles(tw, tw2, M2);
  const int r0 = blockIdx.x * nrow;
  for (int t = threadIdx.x; t < nrow * M2; t += blockDim.x) a[t] = src[(size_t)r0 * M2 + t];
  __syncthreads();
  C *r = block_fft(a, b, M2, nrow, tw, sign);
  for (int t = threadIdx.x; t < nrow * M2; t += blockDim.x) {
    const int rr = t / M2, k2 = t - rr * M2;
    dst[(size_t)(r0 + rr) + (size_t)M1 * k2] = csc(r[t], scale);
  }
}

// Bin k (0 <= k <= M) of the real spectrum of ND = 2M samples from the complex
// spectrum Z of the packed samples: X = (Z_k + Z*_{M-k})/2 - i e^{-2 pi i k/ND} (Z_k - Z*_{M-k})/2.
template <typename C>
__device__ __forceinline__ C real_bin(const C *Z, long long M, long long k, const C *tlo, const C *thi, int K) {
  using R = decltype(C().x);
  const C zk = Z[k % M], zm = cconj(Z[(M - k) % M]);
  const C e = twiddle2(tlo, thi, k, K, -1);  // e^{-2 pi i k/(2M)}
  const C s = ca(zk, zm), d = cs(zk, zm);
  const C ed = cm(e, d);
  return mk<C>((R)0.5 * (s.x + ed.y), (R)0.5 * (s.y - ed.x));
}

// Forward layers: one CTA per layer m in [0, NF].  The spectrum is either X
// (bins 0..M given) or unpacked on the fly from Z, the FFT of the packed samples.
template <typename C>
__global__ void wdm_fwd_layer_kernel(const C *Z, const C *X, long long M, int NF, int NT,
                                     const decltype(C().x) *phif, const C *twNT, const C *tlo, const C *thi, int K,
                                     decltype(C().x) *wdm) {
  using R = decltype(C().x);
  extern __shared__ __align__(16) unsigned char sm_raw[];
  C *tw = reinterpret_cast<C *>(sm_raw);
  C *a = tw + NT;
  C *b = a + NT;
  load_twiddles(tw, twNT, NT);
  const int m = blockIdx.x;
  const int center = m * NT / 2;
  for (int t = threadIdx.x; t < NT; t += blockDim.x) {
    const int j = t - NT / 2;
    C v = mk<C>((R)0, (R)0);
    const int idx = center + j;
    bool ok = j > -NT / 2;
    if (m == 0 && idx < 0) ok = false;
    if (m == NF && idx > center) ok = false;
    if (ok) {
      R w = phif[j < 0 ? -j : j];
      if (j == 0 && (m == 0 || m == NF)) w *= (R)0.5;
      v = csc(X ? X[idx] : real_bin(Z, M, (long long)idx, tlo, thi, K), w);
    }
    a[t] = v;
  }
  __syncthreads();
  C *r = block_fft(a, b, NT, 1, tw, +1);
  const R inv = (R)1 / (R)NT;
  const R sq2 = (R)1.41421356237309504880;
  for (int n = threadIdx.x; n < NT; n += blockDim.x) {
    const C v = r[n];
    if (m == 0) {
      if (!(n & 1)) wdm[n] = v.x * inv * sq2;
    } else if (m == NF) {
      if (!(n & 1)) wdm[n + 1] = v.x * inv * sq2;
    } else {
      const R sgn = (m % 2 == 0) ? (R)1 : (R)-1;
      wdm[n + (size_t)NT * m] = ((n + m) % 2 == 0) ? v.x * inv : sgn * v.y * inv;
    }
  }
}

// Inverse layers of one parity: X[i] += window * FFT(prefactors) for the
// layer's support; layers m = parity, parity + 2, ...
template <typename C>
__global__ void wdm_inv_layer_kernel(const decltype(C().x) *wdm, int NF, int NT, int parity,
                                     const decltype(C().x) *phif, const C *twNT, C *X) {
  using R = decltype(C().x);
  extern __shared__ __align__(16) unsigned char sm_raw[];
  C *tw = reinterpret_cast<C *>(sm_raw);
  C *a = tw + NT;
  C *b = a + NT;
  load_twiddles(tw, twNT, NT);
  const int m = parity + 2 * blockIdx.x;
  if (m > NF) return;
  const R isq2 = (R)0.70710678118654752440;
  for (int n = threadIdx.x; n < NT; n += blockDim.x) {
    C v;
    if (m == 0) {
      v = mk<C>(wdm[(2 * n) % NT] * isq2, (R)0);
    } else if (m == NF) {
      v = mk<C>(wdm[(2 * n) % NT + 1] * isq2, (R)0);
    } else {
      const R w = wdm[n + (size_t)NT * m];
      v = ((n + m) % 2 == 0) ? mk<C>(w, (R)0) : mk<C>((R)0, -w);
    }
    a[n] = v;
  }
  __syncthreads();
  C *r = block_fft(a, b, NT, 1, tw, -1);
  const long long ND = (long long)NF * NT;
  const int center = m * NT / 2;
  int imin = center - NT / 2, imax = center + NT / 2;
  if (imin < 0) imin = 0;
  if (imax > ND / 2 + 1) imax = (int)(ND / 2 + 1);
  const R scale = (R)NF / (R)2;
  for (int i = imin + threadIdx.x; i < imax; i += blockDim.x) {
    const int iind = i > center ? i - center : center - i;
    const C v = (m == 0 || m == NF) ? r[(2 * i) % NT] : r[i % NT];
    const R w = phif[iind] * scale;
    C acc = X[i];
    acc.x += v.x * w;
    acc.y += v.y * w;
    X[i] = acc;
  }
}

// Complex spectrum of the packed samples from the real spectrum X (bins 0..M,
// the imaginary parts of bins 0 and M ignored as an inverse real FFT does):
// Z_k = (X_k + X*_{M-k}) + i e^{2 pi i k/ND} (X_k - X*_{M-k}).
template <typename C>
__global__ void wdm_pack_kernel(const C *X, long long M, const C *tlo, const C *thi, int K, C *Z) {
  using R = decltype(C().x);
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= M) return;
  C xk = X[k], xm = X[M - k];
  if (k == 0) {
    xk.y = (R)0;
    xm.y = (R)0;
  }
  xm = cconj(xm);
  const C s = ca(xk, xm), d = cs(xk, xm);
  const C e = twiddle2(tlo, thi, k, K, +1);
  const C ed = cm(e, d);
  Z[k] = mk<C>(s.x - ed.y, s.y + ed.x);
}

template <typename C>
__global__ void wdm_zero_kernel(C *X, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) X[i] = mk<C>((decltype(C().x))0, (decltype(C().x))0);
}

template <typename C>
__global__ void wdm_cast_kernel(const double *in, decltype(C().x) *out, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (decltype(C().x))in[i];
}

template <typename C>
__global__ void wdm_uncast_kernel(const decltype(C().x) *in, double *out, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i];
}

}  // namespace

// ------------------------------------------------------------------ host side
static bool smooth23(long long x) {
  if (x <= 0) return false;
  while (x % 3 == 0) x /= 3;
  return (x & (x - 1)) == 0;
}

// M = M1 M2 with both factors of the form 2^a 3^b and at most maxL, as close
// to sqrt(M) as possible (balanced passes coalesce best).
static int split_factor(long long M, int maxL) {
  int best = 0;
  double bestd = 1e300;
  for (int L = 2; L <= maxL; L++) {
    if (M % L || !smooth23(L)) continue;
    const long long M2 = M / L;
    if (M2 < 2 || M2 > maxL || !smooth23(M2)) continue;
    const double d = fabs(log((double)L) - log((double)M2));
    if (d < bestd - 1e-12) {
      bestd = d;
      best = L;
    }
  }
  return best;
}

template <typename C>
static size_t fft_smem(int L, int nser) {
  return sizeof(C) * ((size_t)L + 2 * (size_t)nser * L);
}

// series per CTA for a pass over `count` series of length L
template <typename C>
static int pick_batch(int L, int count) {
  for (int n = 8; n > 1; n /= 2)
    if (count % n == 0 && fft_smem<C>(L, n) <= 200 * 1024) return n;
  return 1;
}

static cudaError_t set_smem(const void *fn, size_t bytes) {
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// e^{-2 pi i j / P}: the angle is reduced to [0, pi] by conjugate symmetry
// before sin and cos are taken.
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

template <typename C>
static void fill_roots(std::vector<C> &h, long long L) {
  h.resize((size_t)L);
  for (long long j = 0; j < L; j++) {
    double c, s;
    unit_root(j, L, &c, &s);
    h[(size_t)j].x = (decltype(C().x))c;
    h[(size_t)j].y = (decltype(C().x))s;
  }
}

// two-level table for e^{-2 pi i p / P}, p = hi K + lo
template <typename C>
static void fill_two_level(std::vector<C> &lo, std::vector<C> &hi, long long P, int K) {
  lo.resize(K);
  const long long nh = (P + K) / K;
  hi.resize((size_t)nh);
  for (int j = 0; j < K; j++) {
    double c, s;
    unit_root(j, P, &c, &s);
    lo[j].x = (decltype(C().x))c;
    lo[j].y = (decltype(C().x))s;
  }
  for (long long j = 0; j < nh; j++) {
    double c, s;
    unit_root(j * K, P, &c, &s);
    hi[(size_t)j].x = (decltype(C().x))c;
    hi[(size_t)j].y = (decltype(C().x))s;
  }
}

template <typename T>
static cudaError_t upload(void *dst, const std::vector<T> &v, cudaStream_t s) {
  return cudaMemcpyAsync(dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s);
}

template <typename C>
static cudaError_t prepare_t(WdmPlan &P, int NF, int NT, const double *window, cudaStream_t s) {
  using R = decltype(C().x);
  const long long ND = (long long)NF * NT, M = ND / 2;
  P.NF = NF;
  P.NT = NT;
  P.M = M;
  P.M1 = split_factor(M, 4096);
  if (!P.M1) return cudaErrorInvalidValue;
  P.M2 = (int)(M / P.M1);
  P.K = 1024;
  std::vector<C> t1, t2, tn, mlo, mhi, nlo, nhi;
  fill_roots(t1, P.M1);
  fill_roots(t2, P.M2);
  fill_roots(tn, NT);
  fill_two_level(mlo, mhi, M, P.K);
  fill_two_level(nlo, nhi, ND, P.K);
  std::vector<R> win(NT / 2 + 1);
  for (int i = 0; i <= NT / 2; i++) win[i] = (R)window[i];
  const size_t elem = sizeof(C);
  auto pad = [](size_t n) { return (n + 255) / 256 * 256; };
  const size_t sizes[12] = {elem * t1.size(), elem * t2.size(), elem * tn.size(), elem * mlo.size(),
                            elem * mhi.size(), elem * nlo.size(), elem * nhi.size(), sizeof(R) * win.size(),
                            elem * (size_t)(M + 1), elem * (size_t)(M + 1), elem * (size_t)(M + 1),
                            sizeof(double) * (size_t)ND};
  size_t bytes = 0;
  for (size_t b : sizes) bytes += pad(b);
  cudaError_t e = cudaMalloc(&P.base, bytes);
  if (e != cudaSuccess) {
    P.base = nullptr;
    return e;
  }
  void **slots[12] = {&P.tw1, &P.tw2, &P.twNT, &P.mlo, &P.mhi, &P.nlo, &P.nhi, &P.win, &P.bufA, &P.bufB, &P.bufX, &P.rbuf};
  char *p = (char *)P.base;
  for (int i = 0; i < 12; i++) {
    *slots[i] = p;
    p += pad(sizes[i]);
  }
  if ((e = upload(P.tw1, t1, s)) != cudaSuccess) return e;
  if ((e = upload(P.tw2, t2, s)) != cudaSuccess) return e;
  if ((e = upload(P.twNT, tn, s)) != cudaSuccess) return e;
  if ((e = upload(P.mlo, mlo, s)) != cudaSuccess) return e;
  if ((e = upload(P.mhi, mhi, s)) != cudaSuccess) return e;
  if ((e = upload(P.nlo, nlo, s)) != cudaSuccess) return e;
  if ((e = upload(P.nhi, nhi, s)) != cudaSuccess) return e;
  if ((e = upload(P.win, win, s)) != cudaSuccess) return e;
  return cudaStreamSynchronize(s);  // the host vectors go out of scope
}

// Complex FFT of M = M1 x M2 points, src -> dst (natural order), four-step.
template <typename C>
static cudaError_t four_step(const WdmPlan &P, const C *src, C *tmp, C *dst, int sign, decltype(C().x) scale,
                             cudaStream_t s) {
  const int M1 = P.M1, M2 = P.M2;
  const int nc = pick_batch<C>(M1, M2), nr = pick_batch<C>(M2, M1);
  const size_t sm1 = fft_smem<C>(M1, nc), sm2 = fft_smem<C>(M2, nr);
  cudaError_t e;
  if ((e = set_smem((const void *)wdm_col_kernel<C>, sm1)) != cudaSuccess) return e;
  if ((e = set_smem((const void *)wdm_row_kernel<C>, sm2)) != cudaSuccess) return e;
  wdm_col_kernel<C><<<M2 / nc, 256, sm1, s>>>(src, tmp, M1, M2, nc, (const C *)P.tw1, (const C *)P.mlo,
                                               (const C *)P.mhi, P.K, sign);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  wdm_row_kernel<C><<<M1 / nr, 256, sm2, s>>>(tmp, dst, M1, M2, nr, (const C *)P.tw2, sign, scale);
  return cudaGetLastError();
}

static unsigned blocks_for(long long n) { return (unsigned)((n + 255) / 256); }

template <typename C>
static cudaError_t forward_t(const WdmPlan &P, const double *time, double *wdm, cudaStream_t s) {
  using R = decltype(C().x);
  constexpr bool kF64 = std::is_same<R, double>::value;
  const long long ND = (long long)P.NF * P.NT;
  cudaError_t e;
  const C *packed;
  R *out;
  if (kF64) {
    if ((uintptr_t)time % 16) {  // the packed complex view needs 16-byte alignment
      if ((e = cudaMemcpyAsync(P.rbuf, time, sizeof(double) * ND, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return e;
      packed = reinterpret_cast<const C *>(P.rbuf);
    } else {
      packed = reinterpret_cast<const C *>(time);
    }
    out = reinterpret_cast<R *>(wdm);
  } else {
    wdm_cast_kernel<C><<<blocks_for(ND), 256, 0, s>>>(time, (R *)P.rbuf, ND);
    packed = reinterpret_cast<const C *>(P.rbuf);
    out = (R *)P.rbuf;  // consumed by the first FFT pass before the layers write
  }
  if ((e = four_step<C>(P, packed, (C *)P.bufB, (C *)P.bufA, -1, (R)1, s)) != cudaSuccess) return e;
  const size_t sm = fft_smem<C>(P.NT, 1);
  if ((e = set_smem((const void *)wdm_fwd_layer_kernel<C>, sm)) != cudaSuccess) return e;
  wdm_fwd_layer_kernel<C><<<P.NF + 1, 256, sm, s>>>((const C *)P.bufA, nullptr, P.M, P.NF, P.NT, (const R *)P.win,
                                                     (const C *)P.twNT, (const C *)P.nlo, (const C *)P.nhi, P.K,
                                                     out);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (!kF64) wdm_uncast_kernel<C><<<blocks_for(ND), 256, 0, s>>>(out, wdm, ND);
  return cudaGetLastError();
}

// WDM -> spectrum: bins 0..M summed into P.bufX by the windowed layer transforms.
template <typename C>
static cudaError_t inverse_layers_t(const WdmPlan &P, const double *wdm, cudaStream_t s) {
  using R = decltype(C().x);
  constexpr bool kF64 = std::is_same<R, double>::value;
  const long long ND = (long long)P.NF * P.NT, M = P.M;
  const int NT = P.NT, NF = P.NF;
  cudaError_t e;
  const R *in;
  if (kF64) {
    in = reinterpret_cast<const R *>(wdm);
  } else {
    wdm_cast_kernel<C><<<blocks_for(ND), 256, 0, s>>>(wdm, (R *)P.rbuf, ND);
    in = (const R *)P.rbuf;
  }
  wdm_zero_kernel<C><<<blocks_for(M + 1), 256, 0, s>>>((C *)P.bufX, M + 1);
  const size_t sm = fft_smem<C>(NT, 1);
  if ((e = set_smem((const void *)wdm_inv_layer_kernel<C>, sm)) != cudaSuccess) return e;
  // even layers, then odd: same-parity layers have disjoint supports
  for (int parity = 0; parity < 2; parity++)
    wdm_inv_layer_kernel<C><<<(NF - parity) / 2 + 1, 256, sm, s>>>(in, NF, NT, parity, (const R *)P.win,
                                                                    (const C *)P.twNT, (C *)P.bufX);
  return cudaGetLastError();
}

template <typename C>
static cudaError_t inverse_t(const WdmPlan &P, const double *wdm, double *time, cudaStream_t s) {
  using R = decltype(C().x);
  constexpr bool kF64 = std::is_same<R, double>::value;
  const long long ND = (long long)P.NF * P.NT, M = P.M;
  cudaError_t e;
  if ((e = inverse_layers_t<C>(P, wdm, s)) != cudaSuccess) return e;
  wdm_pack_kernel<C><<<blocks_for(M), 256, 0, s>>>((const C *)P.bufX, M, (const C *)P.nlo, (const C *)P.nhi, P.K,
                                                   (C *)P.bufA);
  const bool direct = kF64 && (uintptr_t)time % 16 == 0;
  C *dst = direct ? reinterpret_cast<C *>(time) : reinterpret_cast<C *>(P.rbuf);
  if ((e = four_step<C>(P, (const C *)P.bufA, (C *)P.bufB, dst, +1, (R)(1.0 / (double)ND), s)) != cudaSuccess)
    return e;
  if (!kF64)
    wdm_uncast_kernel<C><<<blocks_for(ND), 256, 0, s>>>((const R *)P.rbuf, time, ND);
  else if (!direct)
    return cudaMemcpyAsync(time, P.rbuf, sizeof(double) * ND, cudaMemcpyDeviceToDevice, s);
  return cudaGetLastError();
}

// wdm -> ND/2 + 1 complex bins (ND + 2 doubles), wavelet_transform_inverse_freq
template <typename C>
static cudaError_t to_freq_t(const WdmPlan &P, const double *wdm, double *freq, cudaStream_t s) {
  using R = decltype(C().x);
  constexpr bool kF64 = std::is_same<R, double>::value;
  const long long n = 2 * (P.M + 1);
  cudaError_t e;
  if ((e = inverse_layers_t<C>(P, wdm, s)) != cudaSuccess) return e;
  if (kF64) return cudaMemcpyAsync(freq, P.bufX, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
  wdm_uncast_kernel<C><<<blocks_for(n), 256, 0, s>>>((const R *)P.bufX, freq, n);
  return cudaGetLastError();
}

// ND/2 + 1 complex bins -> wdm, wavelet_transform_freq
template <typename C>
static cudaError_t from_freq_t(const WdmPlan &P, const double *freq, double *wdm, cudaStream_t s) {
  using R = decltype(C().x);
  constexpr bool kF64 = std::is_same<R, double>::value;
  const long long ND = (long long)P.NF * P.NT, n = 2 * (P.M + 1);
  cudaError_t e;
  const C *X;
  R *out;
  if (kF64) {
    if ((uintptr_t)freq % 16) {
      if ((e = cudaMemcpyAsync(P.bufX, freq, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
      X = (const C *)P.bufX;
    } else {
      X = reinterpret_cast<const C *>(freq);
    }
    out = reinterpret_cast<R *>(wdm);
  } else {
    wdm_cast_kernel<C><<<blocks_for(n), 256, 0, s>>>(freq, (R *)P.bufX, n);
    X = (const C *)P.bufX;
    out = (R *)P.rbuf;
  }
  const size_t sm = fft_smem<C>(P.NT, 1);
  if ((e = set_smem((const void *)wdm_fwd_layer_kernel<C>, sm)) != cudaSuccess) return e;
  wdm_fwd_layer_kernel<C><<<P.NF + 1, 256, sm, s>>>(nullptr, X, P.M, P.NF, P.NT, (const R *)P.win, (const C *)P.twNT,
                                                     (const C *)P.nlo, (const C *)P.nhi, P.K, out);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (!kF64) wdm_uncast_kernel<C><<<blocks_for(ND), 256, 0, s>>>(out, wdm, ND);
  return cudaGetLastError();
}

bool wdm_grid_supported(int NF, int NT) {
  if (NF < 2 || NT < 8 || NT > 4096 || NT % 2 || !smooth23(NT)) return false;
  const long long M = (long long)NF * NT / 2;
  return split_factor(M, 4096) != 0;
}

cudaError_t wdm_prepare(WdmPlan &P, int precision, int NF, int NT, const double *window, cudaStream_t s) {
  wdm_release(P);
  if (!wdm_grid_supported(NF, NT)) return cudaErrorInvalidValue;
  P.precision = precision;
  const cudaError_t e =
      precision == 1 ? prepare_t<float2>(P, NF, NT, window, s) : prepare_t<double2>(P, NF, NT, window, s);
  if (e != cudaSuccess) wdm_release(P);
  return e;
}

void wdm_release(WdmPlan &P) {
  if (P.base) cudaFree(P.base);
  P = WdmPlan();
}

cudaError_t wdm_forward(const WdmPlan &P, const double *time, double *wdm, cudaStream_t s) {
  return P.precision == 1 ? forward_t<float2>(P, time, wdm, s) : forward_t<double2>(P, time, wdm, s);
}

cudaError_t wdm_inverse(const WdmPlan &P, const double *wdm, double *time, cudaStream_t s) {
  return P.precision == 1 ? inverse_t<float2>(P, wdm, time, s) : inverse_t<double2>(P, wdm, time, s);
}

cudaError_t wdm_to_freq(const WdmPlan &P, const double *wdm, double *freq, cudaStream_t s) {
  return P.precision == 1 ? to_freq_t<float2>(P, wdm, freq, s) : to_freq_t<double2>(P, wdm, freq, s);
}

cudaError_t wdm_from_freq(const WdmPlan &P, const double *freq, double *wdm, cudaStream_t s) {
  return P.precision == 1 ? from_freq_t<float2>(P, freq, wdm, s) : from_freq_t<double2>(P, freq, wdm, s);
}

// Meyer window of utils/src/glass_wavelet.c:305-349 with the regularised
// incomplete beta function I_x(nx, nx) of utils/src/glass_math.c:1214-1242
// (hypergeometric series, which terminates for integer nx).
static double hyp2f1_series(double a, double b, double c, double x) {
  const double TOL = 1e-8;
  double term = a * b * x / c, value = 1.0 + term;
  int n = 1;
  while (fabs(term) > TOL) {
    a++, b++, c++, n++;
    term *= a * b * x / c / n;
    value += term;
  }
  return value;
}

void wdm_window(int NF, int NT, double A, double nx, bool forward, double *phif) {
  const double DeltaOmega = M_PI / NF, domega = 2 * DeltaOmega / (double)NT;
  const double B = DeltaOmega - 2 * A, insDOM = 1.0 / sqrt(DeltaOmega);
  const double beta = exp(lgamma(nx) + lgamma(nx) - lgamma(nx + nx));
  for (int i = 0; i < NT / 2 + 1; i++) {
    const double omega = domega * i;
    double z = 0.0;
    if (fabs(omega) >= A && fabs(omega) < A + B) {
      const double x = (fabs(omega) - A) / B;
      const double y = pow(x, nx) * hyp2f1_series(nx, 1 - nx, nx + 1, x) / beta / nx;
      z = insDOM * cos(y * M_PI_2);
    }
    if (fabs(omega) < A) z = insDOM;
    phif[i] = z;
  }
  double norm = 0.0;
  for (int i = 0; i < NT / 2 + 1; i++) norm += (i == 0 ? 1.0 : 2.0) * phif[i] * phif[i];
  norm = sqrt(norm * domega * M_1_PI);
  if (forward) norm *= NF / 2.0;
  for (int i = 0; i < NT / 2 + 1; i++) phif[i] /= norm;
}

}  // namespace glass
