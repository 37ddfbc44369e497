// Plain-FP64 delta-logL batch that allocates nothing.
//
// Some callers cannot allocate GPU memory while they run: a host that
// pre-allocates everything at start-up and forbids allocation later (hard
// real-time or embedded systems), an application that runs under a memory
// pool it does not own, or code that is not allowed to call into the CUDA
// allocator at all.  For them, glass_gpu_dlogl_fp64_noalloc runs the same
// kernels as glass_gpu_dlogl_batch with PREC_FP64, but every intermediate
// buffer lives in the fixed-size device arrays of this file instead of memory
// from cudaMalloc.  The caller passes inputs and outputs in its own device
// memory and a stream; nothing else is needed.
//
// Consequences of the fixed arrays (also stated in include/glass_gb300.h):
//  * every GPU that loads this library holds them (about 41 MB) until the
//    process exits;
//  * every call on a device uses the same arrays, so calls that overlap on the
//    GPU (two streams, or two host threads) race and corrupt each other;
//  * the first call on a device looks up the arrays' device addresses; make
//    that first call before any stream capture.
#include <mutex>

#include "../../include/glass_gb300.h"
#include "ucb_fd_device.cuh"

namespace glass {

cudaError_t fd_launch_slow_fp64(const SlowArgs &a, int num_sms, cudaStream_t stream);
cudaError_t fd_launch_spec_fp64(int N, const SpecArgs &a, int nitems, int num_sms, cudaStream_t stream, bool perch);
cudaError_t fd_launch_plan64(const PlanArgs &a, cudaStream_t stream);
int report_error(int code, const char *msg);
int report_cuda_error(cudaError_t e, const char *where);

namespace {

constexpr int kNaMaxItems = GLASS_NOALLOC_MAX_ITEMS;
constexpr int kNaMaxBins = GLASS_NOALLOC_MAX_BINS;
constexpr long long kNaMaxSamples = GLASS_NOALLOC_MAX_SAMPLES;
constexpr int kTableSamples = 32 * ((1 << kNumBins) - 1);  // sizes 32..4096 back to back

// The scratch arrays.  In host code these names are stand-ins, not device
// addresses: their addresses come from cudaGetSymbolAddress.
static __device__ __align__(256) double2 na_w64[2 * (size_t)kNaMaxBins];
static __device__ __align__(256) double2 na_g64[4 * (size_t)kNaMaxBins];
static __device__ __align__(256) OrbitSample64 na_pos64[kTableSamples];
static __device__ __align__(256) OrbitSampleMix na_mix[kTableSamples];
static __device__ __align__(256) double2 na_tw64[kTableSamples];
static __device__ __align__(256) float2 na_tw32[kTableSamples];
static __device__ __align__(256) ItemF64 na_items[kNaMaxItems];
static __device__ __align__(256) int na_bin_count[kNumBins];
static __device__ __align__(256) int na_bin_list[kNumBins * kNaMaxItems];
static __device__ __align__(256) double2 na_series[4 * (size_t)kNaMaxSamples];

struct NaAddrs {
  bool ready = false;
  double2 *w64, *g64, *tw64, *series;
  OrbitSample64 *pos64;
  OrbitSampleMix *mix;
  float2 *tw32;
  ItemF64 *items;
  int *bin_count, *bin_list;
  int num_sms;
};
constexpr int kNaMaxDevices = 64;
NaAddrs g_na[kNaMaxDevices];
std::mutex g_na_mutex;

// Device addresses of the arrays, looked up once per device with that device
// current.
cudaError_t na_setup(int dev, NaAddrs *&out) {
  std::lock_guard<std::mutex> lock(g_na_mutex);
  NaAddrs &a = g_na[dev];
  if (!a.ready) {
    cudaError_t e;
    if ((e = cudaGetSymbolAddress((void **)&a.w64, na_w64)) != cudaSuccess) return e;
    if ((e = cudaGetSymbolAddress((void **)&a.g64, na_g64)) != cudaSuccess) return e;
    if ((e = cudaGetSymbolAddress((void **)&a.pos64, na_pos64)) != cudaSuccess) return e;
    if ((e = cudaGetSymbolAddress((void **)&a.mix, na_mix)) != cudaSuccess) return e;
    if ((e = cudaGetSymbolAddress((void **)&a.tw64, na_tw64)) != cudaSuccess) return e;
    if ((e = cudaGetSymbolAddress((void **)&a.tw32, na_tw32)) != cudaSuccess) return e;
    if ((e = cudaGetSymbolAddress((void **)&a.items, na_items)) != cudaSuccess) return e;
    if ((e = cudaGetSymbolAddress((void **)&a.bin_count, na_bin_count)) != cudaSuccess) return e;
    if ((e = cudaGetSymbolAddress((void **)&a.bin_list, na_bin_list)) != cudaSuccess) return e;
    if ((e = cudaGetSymbolAddress((void **)&a.series, na_series)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&a.num_sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    a.ready = true;
  }
  out = &a;
  return cudaSuccess;
}

// FP64 bank tables on the device, one thread per (segment, bin): the whitened
// residual and the per-bin TDI x whitening weights of fd_build_bank_tables.
__global__ void na_bank_kernel(int format, double T, double fstar, int NFFT, int nseg, const int *qmin,
                               const double *rA, const double *rE, const double *invCA, const double *invCE,
                               double2 *w64, double2 *g64) {
  const long long sj = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (sj >= (long long)nseg * NFFT) return;
  const int s = (int)(sj / NFFT), j = (int)(sj % NFFT);
  const double sqT = sqrt(T);
  const double f = (double)(qmin[s] + j) / T;
  const double x = f / fstar;
  double s1, c1;
  sincos(x, &s1, &c1);
  const double c2 = 2. * c1 * c1 - 1.0, s2 = 2. * s1 * c1;
  const double c3 = 2. * c1 * c2 - c1, s3 = 2. * s1 * c2 + s1;
  double pref, w2r, w2i, w1r, w1i;
  if (format == 0) {
    pref = f * (4.0 / fstar * sqT) * s1;
    w2r = c2; w2i = -s2;
    w1r = c1; w1i = -s1;
  } else {
    pref = (format == 1) ? sqT : sqT * 2. * x;
    w2r = c3 - c1; w2i = -s3 + s1;
    w1r = c2 - 1.0; w1i = -s2;
  }
  const double sA = sqrt(invCA[sj]), sE = sqrt(invCE[sj]);
  const double ka = sA * kSQRT1_2 * pref, ke = sE * kINVSQ6 * pref;
  const double conj = (format == 1) ? -1.0 : 1.0;
  w64[2 * sj] = make_double2(rA[2 * sj] * sA, conj * rA[2 * sj + 1] * sA);
  w64[2 * sj + 1] = make_double2(rE[2 * sj] * sE, conj * rE[2 * sj + 1] * sE);
  g64[4 * sj + 0] = make_double2(ka * w2r, ka * w2i);
  g64[4 * sj + 1] = make_double2(ka * w1r, ka * w1i);
  g64[4 * sj + 2] = make_double2(ke * w2r, ke * w2i);
  g64[4 * sj + 3] = make_double2(ke * w1r, ke * w1i);
}

}  // namespace
}  // namespace glass

using namespace glass;

extern "C" int glass_gpu_dlogl_fp64_noalloc(void *stream, int format, double T, double t0, int NFFT, int nseg,
                                            const int *qmin, const double *rA, const double *rE,
                                            const double *invCA, const double *invCE, int nitems,
                                            const int *item_seg, const double *params, const double *term_x,
                                            double *dlogl, double *term_y, double *hh, int *status) {
  if (nitems < 0 || nseg < 1 || NFFT < kMinN || !(T > 0))
    return report_error(GLASS_ERR_ARG, "dlogl_fp64_noalloc: negative item count, no segment, NFFT below 32 or T <= 0");
  if (format < 0 || format > 2) return report_error(GLASS_ERR_FORMAT, "dlogl_fp64_noalloc: unknown format");
  if (nitems == 0) return GLASS_OK;
  if (!qmin || !rA || !rE || !invCA || !invCE || !item_seg || !params || !dlogl)
    return report_error(GLASS_ERR_ARG, "dlogl_fp64_noalloc: null argument");
  if (nitems > kNaMaxItems)
    return report_error(GLASS_ERR_SIZE, "dlogl_fp64_noalloc: more than GLASS_NOALLOC_MAX_ITEMS proposals");
  if ((long long)nseg * NFFT > kNaMaxBins)
    return report_error(GLASS_ERR_SIZE, "dlogl_fp64_noalloc: nseg * NFFT above GLASS_NOALLOC_MAX_BINS");
  if ((long long)nitems * (NFFT < kMaxN ? NFFT : kMaxN) > kNaMaxSamples)
    return report_error(GLASS_ERR_SIZE, "dlogl_fp64_noalloc: nitems * min(NFFT, 4096) above GLASS_NOALLOC_MAX_SAMPLES");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return report_cuda_error(e, "dlogl_fp64_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kNaMaxDevices) return report_error(GLASS_ERR_CUDA, "dlogl_fp64_noalloc: device index above 63");
  NaAddrs *na = nullptr;
  if ((e = na_setup(dev, na)) != cudaSuccess) return report_cuda_error(e, "dlogl_fp64_noalloc: array addresses");
  cudaStream_t s = (cudaStream_t)stream;
  const double fstar = kCLIGHT / (2.0 * kPI * kLARM);

  // tables: bank (whitened residual, per-bin weights), orbits and twiddles
  const long long nb = (long long)nseg * NFFT;
  na_bank_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(format, T, fstar, NFFT, nseg, qmin, rA, rE, invCA,
                                                               invCE, na->w64, na->g64);
  FdTablesDev tab;
  tab.base = na->pos64;  // tables already exist: fd_build_orbit_tables only fills them
  size_t off = 0;
  for (int b = 0; b < kNumBins; b++) {
    tab.pos64[b] = na->pos64 + off;
    tab.mix[b] = na->mix + off;
    tab.tw64[b] = na->tw64 + off;
    tab.tw32[b] = na->tw32 + off;
    off += (size_t)32 << b;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return report_cuda_error(e, "dlogl_fp64_noalloc: bank tables");
  if ((e = fd_build_orbit_tables(tab, T, t0, s)) != cudaSuccess)
    return report_cuda_error(e, "dlogl_fp64_noalloc: orbit tables");
  if ((e = cudaMemsetAsync(na->bin_count, 0, sizeof(int) * kNumBins, s)) != cudaSuccess)
    return report_cuda_error(e, "dlogl_fp64_noalloc: count reset");

  // plan, slow part, per-size spectral kernels (the FP64 path's own kernels)
  PlanArgs pa;
  pa.nitems = nitems;
  pa.nseg = nseg;
  pa.NFFT = NFFT;
  pa.cap = kNaMaxItems;
  pa.precision = 0;
  pa.n_fixed = 0;
  pa.T = T;
  pa.fstar = fstar;
  pa.L = kLARM;
  pa.item_seg = item_seg;
  pa.params = params;
  pa.term_x = term_x;
  pa.seg_qmin = qmin;
  pa.items64 = na->items;
  pa.itemsmix = nullptr;
  pa.bin_count = na->bin_count;
  pa.bin_list = na->bin_list;
  pa.dlogl = dlogl;
  pa.term_y = term_y;
  pa.hh = hh;
  pa.status = status;
  if ((e = fd_launch_plan64(pa, s)) != cudaSuccess) return report_cuda_error(e, "dlogl_fp64_noalloc: plan");

  SlowArgs sa;
  sa.cap = kNaMaxItems;
  sa.NFFT = NFFT;
  sa.fstar = fstar;
  sa.L = kLARM;
  sa.Rf = (float)(kAU * (kLARM / (2.0 * kSQ3 * kAU)));
  sa.invLf = (float)(1.0 / kLARM);
  sa.AUcf = (float)(kAU / kCLIGHT);
  sa.invTf = (float)(1.0 / T);
  sa.bin_count = na->bin_count;
  sa.bin_list = na->bin_list;
  sa.items64 = na->items;
  sa.itemsmix = nullptr;
  for (int b = 0; b < kNumBins; b++) {
    sa.pos64[b] = tab.pos64[b];
    sa.mix[b] = tab.mix[b];
  }
  sa.series = na->series;
  sa.nitems = nitems;
  sa.series_len = 4 * kNaMaxSamples;
  if ((e = fd_launch_slow_fp64(sa, na->num_sms, s)) != cudaSuccess)
    return report_cuda_error(e, "dlogl_fp64_noalloc: slow part");

  SpecArgs a;
  a.NFFT = NFFT;
  a.cap = kNaMaxItems;
  a.bin_count = na->bin_count;
  a.items64 = na->items;
  a.itemsmix = nullptr;
  a.series = na->series;
  a.nitems = nitems;
  a.nseg = nseg;
  a.series_len = 4 * kNaMaxSamples;
  a.w32 = nullptr;
  a.w32lo = nullptr;
  a.g32 = nullptr;
  a.Q = nullptr;
  a.w64 = na->w64;
  a.g64 = na->g64;
  a.term_x = term_x;
  a.dlogl = dlogl;
  a.term_y = term_y;
  a.hh = hh;
  a.status = status;
  for (int b = 0; b < kNumBins; b++) {
    const int N = 32 << b;
    if (N > NFFT) break;
    a.bin = b;
    a.bin_list = na->bin_list + (size_t)b * kNaMaxItems;
    a.tw = tab.tw64[b];
    if ((e = fd_launch_spec_fp64(N, a, nitems, na->num_sms, s, false)) != cudaSuccess)
      return report_cuda_error(e, "dlogl_fp64_noalloc: spectral kernels");
  }
  return GLASS_OK;
}
