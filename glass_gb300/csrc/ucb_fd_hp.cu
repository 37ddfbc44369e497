// Double-float re-evaluation of mixed-precision proposals: the standalone
// kernel.
//
// The mixed path's template is an FP32 FFT of FP32 series; an FP32 FFT leaves
// a relative error of up to ~1e-7 on the few bins that hold a narrowband
// template's power, so its delta logL carries an error of up to ~1e-7 x
// sqrt((h|h)/2 |r - h|^2) (whitened sums over the template support): below
// 1e-3 except for loud templates, near the data of a source with SNR ~ 300 or
// far from the data with (h|h) ~ 1e6.  The mixed spectral kernels flag those
// proposals, and the proposal's spectral stage is evaluated again in
// double-float arithmetic (pairs of floats, ~48 bits, on the FP32 pipe, which
// on GB300 runs 64 times the FP64 rate): the persistent kernel for sizes up
// to 1024 does that in place, in the CTA that flagged the unit; this kernel
// does it for the listed proposals of sizes 2048 and 4096 ("list mode"), and
// for every proposal still above the tolerance after that, from the FP64
// series of the FP64 slow part ("bin mode": the error left by FP32 series is
// ~1e-8 of the same scale).
//
// Outputs: as the spectral kernels (dlogl, term_y, hh, status, term_ch).
#include "ucb_fd_device.cuh"

namespace glass {

constexpr int kHpThreads = 256;
constexpr int kHpSharedTwMax = 2048;  // sizes whose twiddles are copied to shared memory

template <bool BIN, bool PERCH>
__global__ void __launch_bounds__(kHpThreads) fd_hp_spec_kernel(HpArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *red = reinterpret_cast<float2 *>(smem_raw);  // 32 entries
  dc *buf = reinterpret_cast<dc *>(smem_raw + 256);
  const int NM = a.nmax;
  // twiddles of the item's size, copied once per item (read by every stage;
  // from global memory each stage would wait on an L2 or DRAM round trip)
  float4 *tws = reinterpret_cast<float4 *>(buf + 3 * NM);
  const bool tw_shared = NM <= kHpSharedTwMax;
  const HpTab tab{a.NFFT, a.w32, a.w32lo, a.g32, a.g32lo};
  // work units: listed items, or every item of every size in the counts
  int total = 0;
  int cs[kNumBins + 1];
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
  for (int u = blockIdx.x; u < total; u += gridDim.x) {
    int item, N, seg, imin, bin;
    long long off;
    df amp;
    if constexpr (BIN) {
      bin = 0;
#pragma unroll
      for (int b = 1; b < kNumBins; b++)
        if (u >= cs[b]) bin = b;
      const int slot = u - cs[bin];
      item = a.bin_list[(size_t)bin * a.cap + slot];
      const ItemF64 &c = a.items64[item];
      N = c.N;
      seg = c.seg;
      imin = c.imin;
      off = (bin_sample_start(a.bin_count, a.NFFT, bin) + (long long)slot * N) * 4;
      amp = df_from_double(c.amp_s);
    } else {
      item = a.list[u];
      off = a.off[u];
      const ItemMix &c = a.itemsmix[item];
      N = c.N;
      seg = c.seg;
      imin = c.imin;
      bin = fd_bin_of(N);
      amp = df{c.amp_p2, 0.f};
    }
    const float4 *tw = a.tw32x[bin];
    if (tw_shared) {
      __syncthreads();  // the previous item is done with the twiddles
      for (int n = threadIdx.x; n < N; n += blockDim.x) tws[n] = tw[n];
      tw = tws;
    }
    df s[3];
    if constexpr (BIN) {
      hp_item_sums(a.series64 + off, N, seg, imin, amp, false, tw, tab, buf, red, s);
    } else {
      hp_item_sums(a.series32 + off, N, seg, imin, amp, true, tw, tab, buf, red, s);
    }
    if (threadIdx.x == 0) {
      hp_write(item, N, seg, imin, a.NFFT, s, a.Q, a.QA, PERCH, a.term_x, a.dlogl, a.term_y, a.hh, a.term_ch,
               a.status);
      if (!BIN && a.next_list) {
        const float est =
            a.next_e1 * sqrtf(s[2].hi * (s[0].hi + s[1].hi)) * fb_scale_of(a.inv_scale, a.nscale, item);
        if (!(est <= 1.f)) {
          a.next_list[atomicAdd(a.next_count, 1)] = item;
          atomicAdd(a.next_total, 1ull);
        }
      }
    }
    __syncthreads();
  }
  // the last CTA leaves the counters it was given at zero
  if (a.zero_at) {
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      if (atomicAdd(a.done, 1) == (int)gridDim.x - 1) {
        for (int q = 0; q < a.nzero; q++) a.zero_at[q] = 0;
        *a.done = 0;
        __threadfence();
        if (a.has_cond) cudaGraphSetConditional(a.cond, *(volatile const int *)a.next_count > 0 ? 1u : 0u);
      }
    }
  }
}

size_t fd_hp_smem_bytes(int nmax) {
  return 256 + 3 * (size_t)nmax * sizeof(dc) + (nmax <= kHpSharedTwMax ? (size_t)nmax * sizeof(float4) : 0);
}

template <bool BIN, bool PERCH>
static cudaError_t launch_hp(const HpArgs &a, int num_sms, cudaStream_t stream) {
  const size_t smem = fd_hp_smem_bytes(a.nmax);
  // per device: the attribute for the largest size (4096: 192 KB), and the
  // occupancy at each size's shared memory (as many CTAs per SM as fit, so
  // that the listed proposals spread over more of them)
  static LaunchSetup setup[kNumBins];
  int occ = 0;
  cudaError_t e = launch_setup(setup[fd_bin_of(a.nmax)], [&](int *o) {
    cudaError_t r = cudaFuncSetAttribute(fd_hp_spec_kernel<BIN, PERCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)fd_hp_smem_bytes(kMaxN));
    if (r != cudaSuccess) return r;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, fd_hp_spec_kernel<BIN, PERCH>, kHpThreads, smem);
  }, &occ);
  if (e != cudaSuccess) return e;
  fd_hp_spec_kernel<BIN, PERCH><<<occ * num_sms, kHpThreads, smem, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t fd_launch_hp(const HpArgs &a, bool bin_mode, bool perch, int num_sms, cudaStream_t stream) {
  if (bin_mode) return perch ? launch_hp<true, true>(a, num_sms, stream) : launch_hp<true, false>(a, num_sms, stream);
  return perch ? launch_hp<false, true>(a, num_sms, stream) : launch_hp<false, false>(a, num_sms, stream);
}

}  // namespace glass
