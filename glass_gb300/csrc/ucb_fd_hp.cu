// Double-float re-evaluation of mixed-precision proposals.
//
// The mixed path's template is an FP32 FFT of FP32 series from FP32
// per-proposal constants; its delta logL carries an error of up to
// ~6e-7 sqrt(hw rr / N) + 1.5e-7 |(h|r - h)| (whitened sums over the template
// support): below 1e-3 except for loud templates, near the data of a source
// with SNR ~ 300 or far from the data with (h|h) ~ 1e6.  The mixed spectral
// kernels estimate it and list those
// proposals by size, and they are evaluated again with every step in
// double-float arithmetic (pairs of floats, ~48 bits, on the FP32 pipe, which
// on GB300 runs 64 times the FP64 rate), in two launches:
//   fd_slow_hp_kernel: their four A/E arm-combination series in
//     double-float, three warps per 32 samples: the mixed slow part's formulation
//     (carrier phase heterodyned to the segment and reduced mod 2 pi, so that
//     its absolute error stays ~1e-12 rad) with every product and sum in
//     double-float, double-float sine, cosine (table of k pi/32 plus short
//     Taylor series) and sinc, and the per-sample
//     geometry and per-proposal constants as hi + lo floats;
//   fd_hp_kernel:      thread-block clusters of 4 CTAs, one proposal each:
//     CTA r transforms series r in its shared memory (radix-4 Stockham,
//     twiddles as hi + lo floats), then CTAs 2c and 2c + 1 form channel c's
//     whitened template per bin from their own spectrum and their partner's
//     (read through distributed shared memory), each over half of the bins,
//     and sum the residual power and the template power; CTA 0 gathers the
//     four partial sums and writes the results over the mixed ones.
// What is left is of order 1e-12 of the same scale.
#include <math.h>

#include <cooperative_groups.h>

#include "ucb_fd_device.cuh"

namespace glass {

constexpr int kHpThreads = 256;

// -------------------------------------------------------- slow part, df
// The two arms of spacecraft i (12, 13 | 21, 23 | 31, 32) at one sample, as
// slow_sample_mix computes them, in double-float throughout.  tab: the
// sine/cosine table of df_sincos_tab.
__device__ __forceinline__ void slow_arms_hp(const ItemMix &c, const OrbitSampleMix &o, const GeoSampleMix &gm,
                                             const GeoSampleMix &gl, const SlowArgs &K, const float4 *tab, int i,
                                             dc d[2]) {
  const df k0 = {c.k[0], c.kl[0]}, k1 = {c.k[1], c.kl[1]}, k2 = {c.k[2], c.kl[2]};
  // k.(x_j - x_gc) for the three spacecraft (metres)
  df kd[3];
#pragma unroll
  for (int j = 0; j < 3; j++)
    kd[j] = df_add(df_add(df_mul(k0, df{gm.f[3 * j], gl.f[3 * j]}), df_mul(k1, df{gm.f[3 * j + 1], gl.f[3 * j + 1]})),
                   df_mul(k2, df{gm.f[3 * j + 2], gl.f[3 * j + 2]}));
  // this spacecraft's two arms as unique arms (0: 12, 1: 13, 2: 23) with the
  // orientation signs of k.r: 12 +0, 13 +1 | 21 -0, 23 +2 | 31 -1, 32 -2
  const int ua[2] = {i == 2 ? 1 : 0, i == 0 ? 1 : 2};
  const bool neg[2] = {i != 0, i == 2};
  const int ends[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  const df psi0 = carrier_phase_mix(c, o);
  const df u = {o.u_hi, o.u_lo}, ca = {o.ca_hi, o.ca_lo}, sa = {o.sa_hi, o.sa_lo};
  const df tgc = df_mul(K.AUcd, df_add(df_mul(k0, ca), df_mul(k1, sa)));  // guiding-centre delay (s)
  const df tT = df_mul(df_add(tgc, df_mul(kd[i], K.invcd)), K.invTd);    // tau_i / T
  const df v = df_add(u, df_neg(tT));                                    // xi / T
  const df fon = df_add(df{c.fonfs0, c.fonfs0l}, df_mul(df{c.fdfs, c.fdfsl}, v));
  const df aev = df_add(df{1.f, 0.f}, df_mul(df{c.aef, c.aefl}, v));
  const df arg2 = df_add(df_add(psi0, df_neg(df_mul(df{c.w0c, c.w0cl}, kd[i]))),
                         df_mul(c.p7pi_d, df_mul(tT, df_add(tT, df{-2.f * u.hi, -2.f * u.lo}))));
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int a = ua[q];
    df kr = df_mul(df_add(kd[ends[a][1]], df_neg(kd[ends[a][0]])), K.invLd);
    if (neg[q]) kr = df_neg(kr);
    // r^T M r with M = m (DP e+ + DC ex) as hi + lo
    df mr = {0.f, 0.f}, mi = {0.f, 0.f};
#pragma unroll
    for (int t = 0; t < 6; t++) {
      const df mo = {gm.f[9 + 6 * a + t], gl.f[9 + 6 * a + t]};
      mr = df_add(mr, df_mul(df{c.Mr[t], c.Mrl[t]}, mo));
      mi = df_add(mi, df_mul(df{c.Mi[t], c.Mil[t]}, mo));
    }
    const df h1 = df_add(df{1.f, 0.f}, kr);
    const df arg1 = df_mul(df{0.5f * fon.hi, 0.5f * fon.lo}, h1);
    const df sc = df_sinc(arg1, tab);
    const df sinc = {0.25f * sc.hi, 0.25f * sc.lo};
    const df t1r = df_mul(aev, mr), t1i = df_mul(aev, mi);
    df s2, c2;
    df_sincos_tab(df_add(arg1, df_neg(arg2)), tab, &s2, &c2);
    const df re = df_add(df_mul(t1r, c2), df_mul(t1i, s2));
    const df im = df_add(df_mul(t1i, c2), df_neg(df_mul(t1r, s2)));
    d[q] = {df_mul(sinc, re), df_mul(sinc, im)};
  }
}

// One CTA of three warps per 32 consecutive samples of one binned proposal,
// grid-stride over all of them: warp i computes the arms of spacecraft i (a
// third of the dependent chain of a sample each, on separate SM
// sub-partitions); warps 0 and 1 then form the A and E arm combinations of
// ae_combos in double-float.
// sin(k pi / 32), cos(k pi / 32) as hi + lo floats {s.hi, s.lo, c.hi, c.lo},
// k < 64: built once per device on the host (hp_sincos_table).
static __device__ float4 g_hp_sincos[64];

__global__ void __launch_bounds__(96) fd_slow_hp_kernel(SlowArgs a) {
  __shared__ dc s_d[6][32];
  __shared__ float4 s_tab[64];
  if (threadIdx.x < 64) s_tab[threadIdx.x] = g_hp_sincos[threadIdx.x];
  __syncthreads();
  int cs[kNumBins + 1];
  int acc = 0;
#pragma unroll
  for (int b = 0; b < kNumBins; b++) {
    cs[b] = acc;
    if ((32 << b) <= a.NFFT) acc += a.bin_count[b] << b;
  }
  cs[kNumBins] = acc;
  const int lane = threadIdx.x & 31, sc = threadIdx.x >> 5;
  float4 *series = reinterpret_cast<float4 *>(a.series);
#pragma unroll 1
  for (int ch = blockIdx.x; ch < acc; ch += gridDim.x) {
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
    // checked build: an index outside its buffer is recorded and the chunk
    // computed from proposal 0 without being written (the CTA keeps its
    // barriers)
    const bool lok = chk(slot < a.cap, kChkReevalList);
    int item = lok ? a.bin_list[(size_t)b * a.cap + slot] : 0;
    const bool iok = chk(item >= 0 && item < a.nitems, kChkItem);
    if (!iok) item = 0;
    const long long o0 = ((long long)cb * 32 + (long long)slot * N) * 4 + n;
    const bool wok = lok && iok && chk(o0 >= 0 && o0 + 3LL * N < a.series_len, kChkSeriesWrite);
    dc d2[2];
    slow_arms_hp(a.itemsmix[item], a.mix[b][n], a.geo[b][n], a.geolo[b][n], a, s_tab, sc, d2);
    s_d[2 * sc][lane] = d2[0];
    s_d[2 * sc + 1][lane] = d2[1];
    __syncthreads();
    if (sc < 2 && wok) {
      dc d[6];
#pragma unroll
      for (int q = 0; q < 6; q++) d[q] = s_d[q][lane];
      // d: 12, 13, 21, 23, 31, 32
      dc c0, c1;
      if (sc == 0) {
        c0 = dc_sub(dc_add(d[4], d[1]), dc_add(d[5], d[0]));  // a2
        c1 = dc_sub(dc_add(d[1], d[4]), dc_add(d[3], d[2]));  // a1
      } else {
        const dc t2 = dc_sub(d[2], d[3]), t1 = dc_sub(d[0], d[5]);
        c0 = dc_add(dc_sub(dc_sub(dc_add(d[0], d[4]), d[1]), d[5]), dc_add(t2, t2));  // e2
        c1 = dc_add(dc_sub(dc_sub(dc_add(d[1], d[2]), d[3]), d[4]), dc_add(t1, t1));  // e1
      }
      float4 *out = series + ((long long)cb * 32 + (long long)slot * N) * 4 + (size_t)(2 * sc) * N + n;
      out[0] = make_float4(c0.re.hi, c0.im.hi, c0.re.lo, c0.im.lo);
      out[N] = make_float4(c1.re.hi, c1.im.hi, c1.re.lo, c1.im.lo);
    }
    __syncthreads();
  }
}

// ------------------------------------------------------- spectral stage, df
// The proposal of entry k (in size order): item, size, segment, placement,
// size bin and series offset (float4 elements).
struct HpEntry {
  int item, N, seg, imin, bin;
  long long off;
  float amp_p2;
  bool ok;  // checked build: every index in bounds (else read safely, not written)
};

__device__ __forceinline__ HpEntry hp_entry(const HpArgs &a, int k, const int *cs) {
  int bin = 0;
#pragma unroll
  for (int b = 1; b < kNumBins; b++)
    if (k >= cs[b]) bin = b;
  const int slot = k - cs[bin];
  HpEntry e;
  e.ok = chk(slot < a.cap, kChkReevalList);
  e.item = e.ok ? a.bin_list[(size_t)bin * a.cap + slot] : 0;
  e.ok = e.ok && chk(e.item >= 0 && e.item < a.nitems, kChkItem);
  const ItemMix &c = a.itemsmix[e.ok ? e.item : 0];
  e.N = c.N;
  e.seg = c.seg;
  e.imin = c.imin;
  e.bin = bin;
  e.off = (bin_sample_start(a.bin_count, a.NFFT, bin) + (long long)slot * c.N) * 4;
  e.amp_p2 = c.amp_p2;
  e.ok = e.ok && chk(e.seg >= 0 && e.seg < a.nseg, kChkBankRead) &&
         chk(e.N >= 32 && e.N <= a.nmax && e.off >= 0 && e.off + 4LL * e.N <= a.series_len, kChkSeriesRead);
  if (!e.ok) {
    e.N = 32;
    e.bin = 0;
    e.seg = 0;
    e.off = 0;
  }
  return e;
}

template <bool PERCH>
__global__ void __launch_bounds__(kHpThreads) fd_hp_kernel(HpArgs a) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float2 red[32];
  __shared__ float4 s_part;  // this CTA's {rr hi, rr lo, hw hi, hw lo}
  const int NM = a.nmax, NFFT = a.NFFT;
  dc *xb = reinterpret_cast<dc *>(smem_raw), *yb = xb + NM;
  float4 *tws = reinterpret_cast<float4 *>(yb + NM);
  const int r = (int)cluster.block_rank(), ch = r >> 1;
  const int ncl = (int)(gridDim.x >> 2);
  int cs[kNumBins + 1];
  int total = 0;
#pragma unroll
  for (int b = 0; b < kNumBins; b++) {
    cs[b] = total;
    if ((32 << b) <= NFFT) total += a.bin_count[b];
  }
  cs[kNumBins] = total;
  int cur = -1;
  for (int k = (int)(blockIdx.x >> 2); k < total; k += ncl) {
    const HpEntry e = hp_entry(a, k, cs);
    const int N = e.N;
    if (e.bin != cur) {
      const float4 *tw = a.tw32x[e.bin];
      for (int n = threadIdx.x; n < N; n += blockDim.x) tws[n] = tw[n];
      cur = e.bin;
    }
    const float4 *src = a.series + e.off + (long long)r * N;
    for (int n = threadIdx.x; n < N; n += blockDim.x) xb[n] = dc_from(src[n]);
    __syncthreads();
    dc *S = hp_fft(xb, yb, N, tws);
    cluster.sync();  // every spectrum of the proposal is complete
    const dc *Sp = cluster.map_shared_rank(S, (unsigned)(r ^ 1));
    const dc *S0 = (r & 1) ? Sp : S, *S1 = (r & 1) ? S : Sp;  // the channel's series 2c, 2c + 1
    df rr = {0.f, 0.f}, hw = {0.f, 0.f};
    const int half = N >> 1, q0 = (r & 1) * half;
    for (int q = q0 + threadIdx.x; q < q0 + half; q += blockDim.x) {
      const int j = e.imin + ((q + half) & (N - 1));  // fftshift
      if (j < 0 || j >= NFFT) continue;
      const size_t sj = (size_t)e.seg * NFFT + j;
      const float4 gh = a.g32[2 * sj + ch], gl = a.g32lo[2 * sj + ch];
      dc h = dc_add(dc_mul(S0[q], dc_from(make_float2(gh.x, gh.y), make_float2(gl.x, gl.y))),
                    dc_mul(S1[q], dc_from(make_float2(gh.z, gh.w), make_float2(gl.z, gl.w))));
      h = dc_scale2(h, e.amp_p2);
      const float4 wh = a.w32[sj], wl = a.w32lo[sj];
      const dc w = ch == 0 ? dc_from(make_float2(wh.x, wh.y), make_float2(wl.x, wl.y))
                           : dc_from(make_float2(wh.z, wh.w), make_float2(wl.z, wl.w));
      rr = df_add(rr, df_sq_sum(dc_sub(w, h)));
      hw = df_add(hw, df_sq_sum(h));
    }
    rr = hp_block_sum(rr, red);
    hw = hp_block_sum(hw, red);
    if (threadIdx.x == 0) s_part = make_float4(rr.hi, rr.lo, hw.hi, hw.lo);
    cluster.sync();  // partial sums are published; the partner is done with S
    if (r == 0 && threadIdx.x == 0 && e.ok) {
      df s[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      for (int q = 0; q < 4; q++) {
        const float4 o = *cluster.map_shared_rank(&s_part, (unsigned)q);
        s[q >> 1] = df_add(s[q >> 1], df{o.x, o.y});
        s[2] = df_add(s[2], df{o.z, o.w});
      }
      hp_write(e.item, N, e.seg, e.imin, NFFT, s, a.Q, a.QA, PERCH, a.term_x, a.dlogl, a.term_y, a.hh, a.term_ch,
               a.status);
    }
    cluster.sync();  // s_part is read before the next proposal overwrites it
  }
  // the last CTA leaves the counters it was given at zero
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(a.done, 1) == (int)gridDim.x - 1) {
      for (int q = 0; q < a.nzero; q++) a.zero_at[q] = 0;
      *a.done = 0;
    }
  }
}

static size_t hp_smem_bytes(int nmax) { return (size_t)nmax * (2 * sizeof(dc) + sizeof(float4)); }

template <bool PERCH>
static cudaError_t launch_hp(const HpArgs &a, int num_sms, cudaStream_t stream) {
  const size_t smem = hp_smem_bytes(a.nmax);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 4;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(kHpThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  static LaunchSetup setup[kNumBins];
  int ncl = 0;
  cudaError_t e = launch_setup(setup[fd_bin_of(a.nmax)], [&](int *o) {
    cudaError_t r = cudaFuncSetAttribute(fd_hp_kernel<PERCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)hp_smem_bytes(kMaxN));
    if (r != cudaSuccess) return r;
    cudaLaunchConfig_t q = cfg;
    q.gridDim = dim3(4 * num_sms);
    return cudaOccupancyMaxActiveClusters(o, fd_hp_kernel<PERCH>, &q);
  }, &ncl);
  if (e != cudaSuccess) return e;
  if (ncl < 1) ncl = 1;
  cfg.gridDim = dim3(4 * ncl);
  return cudaLaunchKernelEx(&cfg, fd_hp_kernel<PERCH>, a);
}

// The double-float sine/cosine table of the current device, from
// extended-precision host values; once per device, when a context is created
// (a synchronous copy, never inside a stream capture).
cudaError_t fd_hp_tables_init() {
  static LaunchSetup setup;
  int done = 0;
  return launch_setup(setup, [&](int *o) {
    float4 t[64];
    for (int k = 0; k < 64; k++) {
      const long double x = (long double)k * (3.14159265358979323846264338327950288L / 32.0L);
      const long double sv = sinl(x), cv = cosl(x);
      const float sh = (float)sv, ch = (float)cv;
      t[k] = make_float4(sh, (float)(sv - (long double)sh), ch, (float)(cv - (long double)ch));
    }
    *o = 1;
    return cudaMemcpyToSymbol(g_hp_sincos, t, sizeof(t));
  }, &done);
}

cudaError_t fd_launch_reeval(const SlowArgs &sa, const HpArgs &h, bool perch, int num_sms, cudaStream_t stream,
                             int *nlaunch) {
  cudaError_t e;
  static LaunchSetup slow_setup;
  int occ = 0;
  e = launch_setup(slow_setup, [&](int *o) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, fd_slow_hp_kernel, 96, 0);
  }, &occ);
  if (e != cudaSuccess) return e;
  fd_slow_hp_kernel<<<(occ > 0 ? occ : 1) * num_sms, 96, 0, stream>>>(sa);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  e = perch ? launch_hp<true>(h, num_sms, stream) : launch_hp<false>(h, num_sms, stream);
  if (nlaunch) *nlaunch += 2;
  return e;
}

}  // namespace glass
