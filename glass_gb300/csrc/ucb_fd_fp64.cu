// Instantiations of the slow-part and per-size spectral kernels, plain FP64.
#include "ucb_fd_device.cuh"

namespace glass {

cudaError_t fd_launch_slow_fp64(const SlowArgs &a, int num_sms, cudaStream_t stream) {
  return launch_slow<false>(a, num_sms, stream);
}

// FP64 slow part for a handful of proposals, where latency rules: GB300's
// FP64 pipe issues a warp instruction only every few tens of cycles, so each
// chunk of 32 samples is one CTA of three warps, warp i computing the two
// arms of spacecraft i (on its own SM sub-partition); the arm combinations
// follow from shared memory.
__global__ void __launch_bounds__(96) fd_slow64_split_kernel(SlowArgs a) {
  __shared__ double2 s_d[6][32];
  int cs[kNumBins + 1];
  int acc = 0;
#pragma unroll
  for (int b = 0; b < kNumBins; b++) {
    cs[b] = acc;
    if ((32 << b) <= a.NFFT) acc += a.bin_count[b] << b;
  }
  cs[kNumBins] = acc;
  const int lane = threadIdx.x & 31, sc = threadIdx.x >> 5;
  double2 *series = reinterpret_cast<double2 *>(a.series);
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
    const int item = a.bin_list[(size_t)b * a.cap + slot];
    double2 d2[2];
    slow_arms64(a.items64[item], a.pos64[b][n], a.fstar, a.L, sc, d2);
    s_d[2 * sc][lane] = d2[0];
    s_d[2 * sc + 1][lane] = d2[1];
    __syncthreads();
    if (sc == 0) {
      double2 d[6], cmb[4];
#pragma unroll
      for (int q = 0; q < 6; q++) d[q] = s_d[q][lane];
      ae_combos(d, cmb);
      double2 *out = series + ((long long)cb * 32 + (long long)slot * N) * 4 + n;
#pragma unroll
      for (int s = 0; s < 4; s++) out[(size_t)s * N] = cmb[s];
    }
    __syncthreads();
  }
}

cudaError_t fd_launch_slow_fp64_wide(const SlowArgs &a, int num_sms, cudaStream_t stream) {
  fd_slow64_split_kernel<<<4 * num_sms, 96, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t fd_launch_spec_fp64(int N, const SpecArgs &a, int nitems, int num_sms, cudaStream_t stream,
                                bool perch) {
  if (perch) {
    switch (N) {
      case 2048: return launch_spec<2048, false, true>(a, nitems, num_sms, stream);
      case 4096: return launch_spec<4096, false, true>(a, nitems, num_sms, stream);
    }
    return cudaErrorInvalidValue;
  }
  switch (N) {
    case 32: return launch_spec<32, false>(a, nitems, num_sms, stream);
    case 64: return launch_spec<64, false>(a, nitems, num_sms, stream);
    case 128: return launch_spec<128, false>(a, nitems, num_sms, stream);
    case 256: return launch_spec<256, false>(a, nitems, num_sms, stream);
    case 512: return launch_spec<512, false>(a, nitems, num_sms, stream);
    case 1024: return launch_spec<1024, false>(a, nitems, num_sms, stream);
    case 2048: return launch_spec<2048, false>(a, nitems, num_sms, stream);
    case 4096: return launch_spec<4096, false>(a, nitems, num_sms, stream);
  }
  return cudaErrorInvalidValue;
}

cudaError_t fd_launch_spec_all_fp64(const SpecAllArgs &A, int num_sms, cudaStream_t stream, bool perch) {
  if (perch) return launch_spec_all<false, true>(A, num_sms, stream);
  return launch_spec_all<false>(A, num_sms, stream);
}

}  // namespace glass
