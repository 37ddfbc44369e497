// Instantiations of the fused waveform + delta-logL kernel, plain FP64.
#include "ucb_fd_device.cuh"

namespace glass {

cudaError_t fd_launch_size_fp64(int N, const FdArgs &a, int nitems, int num_sms, cudaStream_t stream) {
  switch (N) {
    case 32: return launch_size<32, false>(a, nitems, num_sms, stream);
    case 64: return launch_size<64, false>(a, nitems, num_sms, stream);
    case 128: return launch_size<128, false>(a, nitems, num_sms, stream);
    case 256: return launch_size<256, false>(a, nitems, num_sms, stream);
    case 512: return launch_size<512, false>(a, nitems, num_sms, stream);
    case 1024: return launch_size<1024, false>(a, nitems, num_sms, stream);
    case 2048: return launch_size<2048, false>(a, nitems, num_sms, stream);
    case 4096: return launch_size<4096, false>(a, nitems, num_sms, stream);
  }
  return cudaErrorInvalidValue;
}

}  // namespace glass
