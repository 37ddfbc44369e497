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
// pipe, which on GB300 runs 64 times the FP64 rate) by one wide kernel: one
// CTA per (proposal, TDI channel) transforms the channel's two series in
// shared memory (radix-4 Stockham, twiddles as hi + lo floats), forms per bin
// the whitened template and residual from hi + lo tables and sums the
// residual power and the template power; the second CTA of a proposal to
// finish adds the other channel's sums and writes the results over the mixed
// ones.  A proposal's latency is two FFTs by one CTA, and the re-evaluation
// of a few hundred proposals takes about one wave.
//   list mode reads the mixed series (the error left is their FP32 rounding,
//     ~1e-8 of the same scale); proposals still above the tolerance are
//     listed for FP64 series from the FP64 slow part,
//   bin mode reads those FP64 series through the size counts.
#include "ucb_fd_device.cuh"

namespace glass {

constexpr int kHpThreads = 256;
constexpr int kHpSmemTwMax = 2048;  // larger sizes read their twiddles through L1

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
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float2 red[32];
  __shared__ int s_last;
  const int NM = a.nmax, NFFT = a.NFFT;
  dc *xb = reinterpret_cast<dc *>(smem_raw), *yb = xb + NM, *hb = yb + NM;
  float4 *tws = reinterpret_cast<float4 *>(hb + NM);
  int cs[kNumBins + 1];
  const int total = 2 * hp_entries<BIN>(a, cs);
  int cur = -1;
  for (int u = blockIdx.x; u < total; u += gridDim.x) {
    const int k = u >> 1, ch = u & 1;
    const HpEntry e = hp_entry<BIN>(a, k, cs);
    const int N = e.N;
    const float4 *tw = a.tw32x[e.bin];
    __syncthreads();  // the previous unit is done with the buffers
    if (N <= kHpSmemTwMax) {
      if (e.bin != cur)
        for (int n = threadIdx.x; n < N; n += blockDim.x) tws[n] = tw[n];
      cur = e.bin;
      tw = tws;
    }
    // series 2 ch: its spectrum times the channel's G2 weight, kept in hb
    hp_load<BIN>(a, e.off + (long long)(2 * ch) * N, N, xb);
    __syncthreads();
    const dc *S = hp_fft(xb, yb, N, tw);
    for (int q = threadIdx.x; q < N; q += blockDim.x) {
      const int j = e.imin + ((q + N / 2) & (N - 1));  // fftshift
      if (j < 0 || j >= NFFT) continue;
      const size_t sj = 2 * ((size_t)e.seg * NFFT + j) + ch;
      const float4 gh = a.g32[sj], gl = a.g32lo[sj];
      hb[q] = dc_mul(S[q], dc_from(make_float2(gh.x, gh.y), make_float2(gl.x, gl.y)));
    }
    __syncthreads();
    // series 2 ch + 1 times G1, plus the above: the channel's whitened template
    hp_load<BIN>(a, e.off + (long long)(2 * ch + 1) * N, N, xb);
    __syncthreads();
    S = hp_fft(xb, yb, N, tw);
    df rr = {0.f, 0.f}, hw = {0.f, 0.f};
    for (int q = threadIdx.x; q < N; q += blockDim.x) {
      const int j = e.imin + ((q + N / 2) & (N - 1));
      if (j < 0 || j >= NFFT) continue;
      const size_t sj = (size_t)e.seg * NFFT + j;
      const float4 gh = a.g32[2 * sj + ch], gl = a.g32lo[2 * sj + ch];
      dc h = dc_add(hb[q], dc_mul(S[q], dc_from(make_float2(gh.z, gh.w), make_float2(gl.z, gl.w))));
      h = e.pow2 ? dc_scale2(h, e.amp.hi) : dc_scale(h, e.amp);
      const float4 wh = a.w32[sj], wl = a.w32lo[sj];
      const dc w = ch == 0 ? dc_from(make_float2(wh.x, wh.y), make_float2(wl.x, wl.y))
                           : dc_from(make_float2(wh.z, wh.w), make_float2(wl.z, wl.w));
      rr = df_add(rr, df_sq_sum(dc_sub(w, h)));
      hw = df_add(hw, df_sq_sum(h));
    }
    rr = hp_block_sum(rr, red);
    hw = hp_block_sum(hw, red);
    // the channel's sums to the entry's slot; the second CTA to arrive adds
    // both channels and writes the proposal's results
    if (threadIdx.x == 0) {
      a.part[2 * (size_t)k + ch] = make_float4(rr.hi, rr.lo, hw.hi, hw.lo);
      __threadfence();
      s_last = atomicAdd(a.arrive + k, 1) == 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
      __threadfence();
      const float4 o = __ldcg(a.part + 2 * (size_t)k + (ch ^ 1));  // L2: written by the other CTA
      const df ro = {o.x, o.y}, ho = {o.z, o.w};
      df s[3];
      s[ch] = rr;
      s[ch ^ 1] = ro;
      s[2] = df_add(hw, ho);
      a.arrive[k] = 0;
      hp_write(e.item, N, e.seg, e.imin, NFFT, s, a.Q, a.QA, PERCH, a.term_x, a.dlogl, a.term_y, a.hh, a.term_ch,
               a.status);
      if (!BIN && a.next_list) {
        const float est =
            a.next_e1 * sqrtf(s[2].hi * (s[0].hi + s[1].hi)) * fb_scale_of(a.inv_scale, a.nscale, e.item);
        if (!(est <= 1.f)) {
          a.next_list[atomicAdd(a.next_count, 1)] = e.item;
          atomicAdd(a.next_total, 1ull);
        }
      }
    }
  }
  // the last CTA leaves the counters it was given at zero and sets the
  // conditional node that follows (when captured)
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(a.done, 1) == (int)gridDim.x - 1) {
      const int nx = a.next_count ? *(volatile const int *)a.next_count : 0;
      for (int q = 0; q < a.nzero; q++) a.zero_at[q] = 0;
      *a.done = 0;
      __threadfence();
      if (a.has_cond) cudaGraphSetConditional(a.cond, nx > 0 ? 1u : 0u);
    }
  }
}

static size_t hp_smem_bytes(int nmax) {
  return (size_t)nmax * 3 * sizeof(dc) + (size_t)(nmax < kHpSmemTwMax ? nmax : kHpSmemTwMax) * sizeof(float4);
}

template <bool BIN, bool PERCH>
static cudaError_t launch_hp(const HpArgs &a, int num_sms, cudaStream_t stream) {
  const size_t smem = hp_smem_bytes(a.nmax);
  static LaunchSetup setup[kNumBins];
  int occ = 0;
  cudaError_t e = launch_setup(setup[fd_bin_of(a.nmax)], [&](int *o) {
    cudaError_t r = cudaFuncSetAttribute(fd_hp_kernel<BIN, PERCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)hp_smem_bytes(kMaxN));
    if (r != cudaSuccess) return r;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, fd_hp_kernel<BIN, PERCH>, kHpThreads, smem);
  }, &occ);
  if (e != cudaSuccess) return e;
  fd_hp_kernel<BIN, PERCH><<<occ * num_sms, kHpThreads, smem, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t fd_launch_hp(const HpArgs &a, bool bin_mode, bool perch, int num_sms, cudaStream_t stream) {
  if (bin_mode) return perch ? launch_hp<true, true>(a, num_sms, stream) : launch_hp<true, false>(a, num_sms, stream);
  return perch ? launch_hp<false, true>(a, num_sms, stream) : launch_hp<false, false>(a, num_sms, stream);
}

}  // namespace glass
