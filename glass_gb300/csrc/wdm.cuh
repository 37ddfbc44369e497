// WDM wavelet transforms on the device: plan (tables and work buffers for one
// grid) and the forward/inverse launches.  See wdm.cu.
#pragma once
#include <cuda_runtime.h>

namespace glass {

struct WdmPlan {
  int precision = -1;  // 0 FP64, 1 FP32 (cast at the boundary)
  int NF = 0, NT = 0;
  double A = 0.0, nx = 0.0;
  long long M = 0;  // NF NT / 2 packed complex samples
  int M1 = 0, M2 = 0, K = 0;
  void *base = nullptr;
  void *tw1 = nullptr, *tw2 = nullptr, *twNT = nullptr;
  void *mlo = nullptr, *mhi = nullptr, *nlo = nullptr, *nhi = nullptr;
  void *win = nullptr;
  void *bufA = nullptr, *bufB = nullptr, *bufX = nullptr;
  void *rbuf = nullptr;  // NF NT reals: staging for FP32 casts and unaligned FP64 input
};

// true when NT is even, 8 <= NT <= 4096, NT and NF NT / 2 are of the form
// 2^a 3^b, and NF NT / 2 splits into two such factors of at most 4096.
bool wdm_grid_supported(int NF, int NT);

// Meyer window phif[0..NT/2] (forward normalisation when `forward`).
void wdm_window(int NF, int NT, double A, double nx, bool forward, double *phif);

// Allocates and fills the plan for a grid; window = the forward window.
cudaError_t wdm_prepare(WdmPlan &P, int precision, int NF, int NT, const double *window, cudaStream_t s);
void wdm_release(WdmPlan &P);

// time (NF NT reals) -> wdm (NF NT reals, layout wdm[n + NT m]).  time and wdm
// may be the same buffer.
cudaError_t wdm_forward(const WdmPlan &P, const double *time, double *wdm, cudaStream_t s);
// wdm -> time; may be the same buffer.
cudaError_t wdm_inverse(const WdmPlan &P, const double *wdm, double *time, cudaStream_t s);
// wdm -> ND/2 + 1 complex bins (ND + 2 doubles, re/im interleaved), and back.
// Input and output must not overlap.
cudaError_t wdm_to_freq(const WdmPlan &P, const double *wdm, double *freq, cudaStream_t s);
cudaError_t wdm_from_freq(const WdmPlan &P, const double *freq, double *wdm, cudaStream_t s);

}  // namespace glass
