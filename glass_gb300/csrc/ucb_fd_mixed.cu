// Instantiations of the slow-part and per-size spectral kernels, mixed precision.
#include "ucb_fd_device.cuh"

namespace glass {

cudaError_t fd_launch_slow_mixed(const SlowArgs &a, int num_sms, cudaStream_t stream, int block, int cap) {
  switch (block) {
    case 128: return launch_slow<true, 128>(a, num_sms, stream, cap);
    case 512: return launch_slow<true, 512>(a, num_sms, stream, cap);
    default: return launch_slow<true, 256>(a, num_sms, stream, cap);
  }
}

cudaError_t fd_launch_spec_mixed(int N, const SpecArgs &a, int nitems, int num_sms, cudaStream_t stream,
                                bool perch) {
  if (perch) {
    switch (N) {
      case 2048: return launch_spec<2048, true, true>(a, nitems, num_sms, stream);
      case 4096: return launch_spec<4096, true, true>(a, nitems, num_sms, stream);
    }
    return cudaErrorInvalidValue;
  }
  switch (N) {
    case 32: return launch_spec<32, true>(a, nitems, num_sms, stream);
    case 64: return launch_spec<64, true>(a, nitems, num_sms, stream);
    case 128: return launch_spec<128, true>(a, nitems, num_sms, stream);
    case 256: return launch_spec<256, true>(a, nitems, num_sms, stream);
    case 512: return launch_spec<512, true>(a, nitems, num_sms, stream);
    case 1024: return launch_spec<1024, true>(a, nitems, num_sms, stream);
    case 2048: return launch_spec<2048, true>(a, nitems, num_sms, stream);
    case 4096: return launch_spec<4096, true>(a, nitems, num_sms, stream);
  }
  return cudaErrorInvalidValue;
}

cudaError_t fd_launch_spec_all_mixed(const SpecAllArgs &A, int num_sms, cudaStream_t stream, bool perch, int cap) {
  if (perch) return launch_spec_all<true, true>(A, num_sms, stream, cap);
  return launch_spec_all<true>(A, num_sms, stream, cap);
}

}  // namespace glass
