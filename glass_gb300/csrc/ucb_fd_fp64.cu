// Instantiations of the slow-part and per-size spectral kernels, plain FP64.
#include "ucb_fd_device.cuh"

namespace glass {

cudaError_t fd_launch_slow_fp64(const SlowArgs &a, int num_sms, cudaStream_t stream) {
  return launch_slow<false>(a, num_sms, stream);
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
