// Instantiations of the fused waveform + delta-logL kernel, mixed precision.
#include "ucb_fd_device.cuh"

namespace glass {

cudaError_t fd_launch_size_mixed(int N, const FdArgs &a, int nitems, int num_sms, cudaStream_t stream) {
  switch (N) {
    case 32: return launch_size<32, true>(a, nitems, num_sms, stream);
    case 64: return launch_size<64, true>(a, nitems, num_sms, stream);
    case 128: return launch_size<128, true>(a, nitems, num_sms, stream);
    case 256: return launch_size<256, true>(a, nitems, num_sms, stream);
    case 512: return launch_size<512, true>(a, nitems, num_sms, stream);
    case 1024: return launch_size<1024, true>(a, nitems, num_sms, stream);
    case 2048: return launch_size<2048, true>(a, nitems, num_sms, stream);
    case 4096: return launch_size<4096, true>(a, nitems, num_sms, stream);
  }
  return cudaErrorInvalidValue;
}

}  // namespace glass
