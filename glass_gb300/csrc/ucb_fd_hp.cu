// Double-float re-evaluation of mixed-precision proposals.
//
// The mixed path's template is an FP32 FFT of FP32 series; an FP32 FFT leaves
// a relative error of up to ~1e-7 on the few bins that hold a narrowband
// template's power, so its delta logL carries an error of up to ~1e-7 x
// sqrt((h|h)/2 |r - h|^2) (whitened sums over the template support): below
// 1e-3 except for loud templates, near the data of a source with SNR ~ 300 or
// far from the data with (h|h) ~ 1e6.  The mixed spectral kernels list those
// proposals with their series offsets, and their spectral stage is evaluated
// again in double-float arithmetic (pairs of floats, ~48 bits, on the FP32
// pipe, which on GB300 runs 64 times the FP64 rate) by one wide kernel whose
// thread-block clusters of 4 CTAs each take one proposal: CTA r transforms
// series r in its shared memory (radix-4 Stockham, twiddles as hi + lo floats
// in shared memory), then CTAs 2c and 2c + 1 form channel c's whitened
// template per bin from their own spectrum and their partner's (read through
// distributed shared memory), each over half of the bins, and sum the
// residual power and the template power; CTA 0 gathers the four partial sums
// and writes the results over the mixed ones.  A proposal's latency is one
// FFT, and a few hundred proposals take about one wave.
//   list mode reads the mixed series (the error left is their FP32 rounding,
//     up to ~2e-8 of the same scale),
//   bin mode reads FP64 series from the FP64 slow part through the size
//     counts, for the proposals whose bound after list mode would still
//     exceed the tolerance (listed as such by the spectral kernels, and
//     evaluated concurrently with list mode).
#include <cooperative_groups.h>

#include "ucb_fd_device.cuh"

namespace glass {

constexpr int kHpThreads = 256;

// The proposal of entry k: item index, size, segment, placement, series
// offset (elements of the series scratch) and template scale.
struct HpEntry {
  int item, N, seg, imin, bin;
  long long off;
  df amp;
  bool pow2;
};

template <bool BIN>
__device__ __forceinline__ HpEntry hp_entry(const HpArgs &a, int k, const int *cs) {
  HpEntry e;
  if constexpr (BIN) {
    int bin = 0;
#pragma unroll
    for (int b = 1; b < kNumBins; b++)
      if (k >= cs[b]) bin = b;
    const int slot = k - cs[bin];
    e.item = a.bin_list[(size_t)bin * a.cap + slot];
    const ItemF64 &c = a.items64[e.item];
    e.N = c.N;
    e.seg = c.seg;
    e.imin = c.imin;
    e.bin = bin;
    e.off = (bin_sample_start(a.bin_count, a.NFFT, bin) + (long long)slot * c.N) * 4;
    e.amp = df_from_double(c.amp_s);
    e.pow2 = false;
  } else {
    e.item = a.list[k];
    const ItemMix &c = a.itemsmix[e.item];
    e.N = c.N;
    e.seg = c.seg;
    e.imin = c.imin;
    e.bin = fd_bin_of(c.N);
    e.off = a.off[k];
    e.amp = df{c.amp_p2, 0.f};
    e.pow2 = true;
  }
  return e;
}

template <bool BIN>
__device__ __forceinline__ int hp_entries(const HpArgs &a, int *cs) {
  int total = 0;
  if constexpr (BIN) {
#pragma unroll
    for (int b = 0; b < kNumBins; b++) {
      cs[b] = total;
      if ((32 << b) <= a.NFFT) total += a.bin_count[b];
    }
    cs[kNumBins] = total;
  } else {
    total = *a.count;
  }
  return total;
}

// One series of the entry, as double-floats, into x.
template <bool BIN>
__device__ __forceinline__ void hp_load(const HpArgs &a, long long off, int N, dc *x) {
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    if constexpr (BIN) {
      const double2 v = a.series64[off + n];
      x[n] = {df_from_double(v.x), df_from_double(v.y)};
    } else {
      const float2 v = a.series32[off + n];
      x[n] = {{v.x, 0.f}, {v.y, 0.f}};
    }
  }
}

template <bool BIN, bool PERCH>
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
  const int total = hp_entries<BIN>(a, cs);
  int cur = -1;
  for (int k = (int)(blockIdx.x >> 2); k < total; k += ncl) {
    const HpEntry e = hp_entry<BIN>(a, k, cs);
    const int N = e.N;
    if (e.bin != cur) {
      const float4 *tw = a.tw32x[e.bin];
      for (int n = threadIdx.x; n < N; n += blockDim.x) tws[n] = tw[n];
      cur = e.bin;
    }
    hp_load<BIN>(a, e.off + (long long)r * N, N, xb);
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
      h = e.pow2 ? dc_scale2(h, e.amp.hi) : dc_scale(h, e.amp);
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
    if (r == 0 && threadIdx.x == 0) {
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

template <bool BIN, bool PERCH>
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
    cudaError_t r = cudaFuncSetAttribute(fd_hp_kernel<BIN, PERCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)hp_smem_bytes(kMaxN));
    if (r != cudaSuccess) return r;
    cudaLaunchConfig_t q = cfg;
    q.gridDim = dim3(4 * num_sms);
    return cudaOccupancyMaxActiveClusters(o, fd_hp_kernel<BIN, PERCH>, &q);
  }, &ncl);
  if (e != cudaSuccess) return e;
  if (ncl < 1) ncl = 1;
  cfg.gridDim = dim3(4 * ncl);
  return cudaLaunchKernelEx(&cfg, fd_hp_kernel<BIN, PERCH>, a);
}

cudaError_t fd_launch_hp(const HpArgs &a, bool bin_mode, bool perch, int num_sms, cudaStream_t stream) {
  if (bin_mode) return perch ? launch_hp<true, true>(a, num_sms, stream) : launch_hp<true, false>(a, num_sms, stream);
  return perch ? launch_hp<false, true>(a, num_sms, stream) : launch_hp<false, false>(a, num_sms, stream);
}

}  // namespace glass
