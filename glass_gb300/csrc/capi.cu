// C ABI of the GB300 UCB likelihood engine (include/glass_gb300.h).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/glass_gb300.h"
#include "dropin.h"
#include "noise.cuh"
#include "sampler.cuh"
#include "ucb_fd.cuh"
#include "ucb_fd_device.cuh"
#include "ucb_wavelet.cuh"
#include "wdm.cuh"

using namespace glass;

// ------------------------------------------------------------------ errors
static thread_local std::string g_err = "no error";

static int set_err(int code, const char *fmt, const char *arg = "") {
  char buf[512];
  snprintf(buf, sizeof(buf), fmt, arg);
  g_err = buf;
  return code;
}
static int cuda_err(cudaError_t e, const char *where) {
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  g_err = m;
  return GLASS_ERR_CUDA;
}
#define GLASS_CUDA(call, where)                 \
  do {                                          \
    cudaError_t e_ = (call);                    \
    if (e_ != cudaSuccess) return cuda_err(e_, where); \
  } while (0)

extern "C" const char *glass_gpu_last_error(void) { return g_err.c_str(); }

namespace glass {
// The checked build's per-translation-unit check words (glass_common.cuh).
static std::vector<unsigned (*)()> &check_readers() {
  static std::vector<unsigned (*)()> r;
  return r;
}
static std::mutex g_check_mutex;
void register_check_reader(unsigned (*read_reset)()) {
  std::lock_guard<std::mutex> g(g_check_mutex);
  check_readers().push_back(read_reset);
}
unsigned check_status_all() {
  std::lock_guard<std::mutex> g(g_check_mutex);
  unsigned w = 0;
  for (auto f : check_readers()) w |= f();
  return w;
}

// Error reporting for the entry points defined in other translation units.
int report_error(int code, const char *msg) { return set_err(code, "%s", msg); }
int report_cuda_error(cudaError_t e, const char *where) { return cuda_err(e, where); }
}  // namespace glass

// Error model of the mixed-precision delta logL, in the whitened sums the
// spectral kernel has at hand (hw = |h|^2 and rr = |r - h|^2 over the template
// support, so that (h|h) = 2 hw; hw_full the same for the whole template when
// the segment edge clips it):
//   |error| <= kMixedErrKa sqrt(hw_full rr / N) + kMixedErrKs |(h|r - h)|.
// The FP32 template's rounding error has two parts.  The series' and the
// FFT's rounding spreads evenly over the template's N bins, so its inner
// product with the residual grows as sqrt(hw_full rr / N); the FP32 rounding
// of the per-proposal constants (amplitude, polarisation) scales the whole
// template, an error along h that enters as (h|r - h).  Measured (the largest
// |error| minus the systematic part over the random predictor, and the
// systematic ratio, on 1.2e5 proposals of the 64-segment benchmark workload,
// loud templates at amplitude x30 far from the data, and the 1e4-source
// global-fit population with N up to 4096): 5.9e-7 and 1.5e-7; the bound
// takes 9e-7 and 2e-7, which leaves |error| / bound <= 0.6 wherever
// |error| > 1e-4 on those workloads.
static constexpr double kMixedErrKa = 9e-7;
static constexpr double kMixedErrKs = 2e-7;
static constexpr double kMixedTolDefault = 1e-3;

// ----------------------------------------------------------------- context
// Host pointers of one glass_gpu_dlogl_batch_host call (direct host access).
struct HostIo {
  const double *params;
  const double *term_x;
  const int *item_seg;
  double *dlogl, *term_y, *hh;
  int *status;
};

struct glass_gpu_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  FdBankDev bank;
  void *bank_mem = nullptr;
  std::vector<int> h_qmin;
  // host copies needed to rebuild one segment's tables
  std::vector<double> h_invCA, h_invCE;
  FdTablesDev tab;
  bool tab_ready = false;
  double tab_T = 0, tab_t0 = 0;
  FdWorkDev work;
  // staging for the host-pointer entry points
  void *d_stage = nullptr;
  size_t d_stage_cap = 0;
  // glass_gpu_dlogl_batch_host: pinned host staging, and the copy-in, kernels,
  // copy-out sequence recorded as a CUDA graph per (nitems, precision,
  // term_x given); the graphs hold the staging, work and bank addresses, so
  // they are dropped whenever one of those is reallocated
  void *h_stage = nullptr;
  size_t h_stage_cap = 0;
  // Direct host access: where the device reads the caller's pageable memory
  // through the host's page tables (ATS over a coherent CPU-GPU link), a
  // gather kernel reads the inputs and a scatter kernel writes the outputs in
  // place of the staging copies; the call's host pointers sit in a pinned
  // block that the two kernels read, so one graph serves every call of a shape
  bool host_direct_ok = false;  // device attributes allow it
  bool host_direct = false;     // in use
  HostIo *h_io = nullptr;
  std::map<long long, cudaGraphExec_t> host_graphs;
  int last_launches = 0;
  int n_fixed = 0;  // template size override (0: bandwidth rule)
  // mixed precision: proposals whose estimated delta-logL error exceeds this
  // are evaluated again in higher precision (<= 0: never)
  double mixed_tol = kMixedTolDefault;
  WdmPlan wdm;      // tables and work buffers of the last WDM grid used
  void *wdm_stage = nullptr;  // NF NT doubles for the host-pointer WDM calls
  size_t wdm_stage_cap = 0;
  // wavelet-domain segment: grid tables, data, per-source work
  WvGridDev wv{};
  void *wv_grid_mem = nullptr;
  void *wv_data_mem = nullptr;
  bool wv_data_ready = false;
  WvWorkDev wvw;
  void *wv_work_mem = nullptr;
  void *wv_fisher_mem = nullptr;  // perturbed parameters of the Fisher batches
  FsWorkDev fsw;  // F-statistic scratch
  NoiseDev noise;  // noise-model likelihood: per-bin table and chunk sums
  NoiseWvDev noise_wv;  // the same in the wavelet domain
  SplineNoiseDev spline_noise;    // the one- and two-channel spline noise model
  int sgwb_type = -1;             // SGWB template of glass_gpu_noise_sgwb_setup (-1: none)
  std::vector<double> sgwb_resp;  // its response table rows (f, XX, YY, ZZ, XY, XZ, YZ)
  double *eta_scratch = nullptr;  // glass_gpu_noise_eta_batch: 5 doubles per chain
  size_t eta_cap = 0;
};

static void clear_host_graphs(glass_gpu_ctx *ctx) {
  for (auto &g : ctx->host_graphs) cudaGraphExecDestroy(g.second);
  ctx->host_graphs.clear();
}

static int ctx_activate(glass_gpu_ctx *ctx) {
  GLASS_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  return GLASS_OK;
}

extern "C" int glass_gpu_create(int device, glass_gpu_ctx **out) {
  if (!out) return set_err(GLASS_ERR_ARG, "glass_gpu_create: null output pointer");
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess) return cuda_err(e, "cudaGetDeviceCount");
  if (device < 0 || device >= ndev) return set_err(GLASS_ERR_ARG, "glass_gpu_create: no such device");
  glass_gpu_ctx *ctx = new glass_gpu_ctx();
  ctx->device = device;
  if ((e = cudaSetDevice(device)) != cudaSuccess) {
    delete ctx;
    return cuda_err(e, "cudaSetDevice");
  }
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if ((e = fd_hp_tables_init()) != cudaSuccess) {
    delete ctx;
    return cuda_err(e, "re-evaluation tables");
  }
  {
    int pageable = 0, host_tables = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device);
    cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
    // only with the host's own page tables: without them (HMM) a device access
    // migrates the caller's pages instead of reading them in place
    ctx->host_direct_ok = pageable && host_tables;
    ctx->host_direct = ctx->host_direct_ok;
  }
  if ((e = cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking)) != cudaSuccess) {
    delete ctx;
    return cuda_err(e, "cudaStreamCreate");
  }
  ctx->stream = ctx->own;
  for (int b = 0; b < kNumBins; b++) {
    if ((e = cudaStreamCreateWithFlags(&ctx->work.side[b], cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ctx->work.join[b], cudaEventDisableTiming)) != cudaSuccess) {
      glass_gpu_destroy(ctx);
      return cuda_err(e, "stream/event create");
    }
  }
  if ((e = cudaEventCreateWithFlags(&ctx->work.fork, cudaEventDisableTiming)) != cudaSuccess) {
    glass_gpu_destroy(ctx);
    return cuda_err(e, "event create");
  }
  *out = ctx;
  return GLASS_OK;
}

extern "C" int glass_gpu_destroy(glass_gpu_ctx *ctx) {
  if (!ctx) return GLASS_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->bank_mem);
  cudaFree(ctx->tab.base);
  cudaFree(ctx->work.items64);
  cudaFree(ctx->work.itemsmix);
  cudaFree(ctx->work.itemsgrad);
  cudaFree(ctx->work.bin_count);
  cudaFree(ctx->work.bin_list);
  cudaFree(ctx->work.series);
  cudaFree(ctx->work.series2);
  cudaFree(ctx->work.hp_list);
  cudaFree(ctx->work.fb_total);
  cudaFree(ctx->work.fb_inv_scale);
  cudaFree(ctx->d_stage);
  clear_host_graphs(ctx);
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  if (ctx->h_io) cudaFreeHost(ctx->h_io);
  wdm_release(ctx->wdm);
  cudaFree(ctx->wdm_stage);
  cudaFree(ctx->wv_grid_mem);
  cudaFree(ctx->wv_data_mem);
  cudaFree(ctx->wv_work_mem);
  cudaFree(ctx->wv_fisher_mem);
  fs_work_free(ctx->fsw);
  cudaFree(ctx->noise.tab);
  cudaFree(ctx->noise.rsg);
  cudaFree(ctx->noise.partial);
  cudaFree(ctx->noise_wv.mem);
  cudaFree(ctx->noise_wv.rsg);
  cudaFree(ctx->noise_wv.partial);
  cudaFree(ctx->spline_noise.tab);
  cudaFree(ctx->eta_scratch);
  for (int b = 0; b < kNumBins; b++) {
    if (ctx->work.side[b]) cudaStreamDestroy(ctx->work.side[b]);
    if (ctx->work.join[b]) cudaEventDestroy(ctx->work.join[b]);
  }
  if (ctx->work.fork) cudaEventDestroy(ctx->work.fork);
  for (int i = 0; i < 5; i++)
    if (ctx->work.phase[i]) cudaEventDestroy(ctx->work.phase[i]);
  cudaStreamDestroy(ctx->own);
  delete ctx;
  return GLASS_OK;
}

extern "C" int glass_gpu_set_stream(glass_gpu_ctx *ctx, void *stream) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "glass_gpu_set_stream: null context");
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
  return GLASS_OK;
}

extern "C" int glass_gpu_last_launch_count(glass_gpu_ctx *ctx) { return ctx ? ctx->last_launches : 0; }

extern "C" int glass_gpu_set_host_access(glass_gpu_ctx *ctx, int mode) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "glass_gpu_set_host_access: null context");
  if (mode < -1 || mode > 1) return set_err(GLASS_ERR_ARG, "glass_gpu_set_host_access: mode is -1, 0 or 1");
  if (mode == 1 && !ctx->host_direct_ok)
    return set_err(GLASS_ERR_STATE, "glass_gpu_set_host_access: the device cannot read pageable host memory in place");
  ctx->host_direct = mode == 1 || (mode == -1 && ctx->host_direct_ok);
  return GLASS_OK;
}

extern "C" int glass_gpu_get_host_access(glass_gpu_ctx *ctx, int *supported, int *direct) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "glass_gpu_get_host_access: null context");
  if (supported) *supported = ctx->host_direct_ok ? 1 : 0;
  if (direct) *direct = ctx->host_direct ? 1 : 0;
  return GLASS_OK;
}

extern "C" int glass_gpu_set_phase_timing(glass_gpu_ctx *ctx, int enable) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "glass_gpu_set_phase_timing: null context");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  if (enable && !ctx->work.phase[0])
    for (int i = 0; i < 5; i++) GLASS_CUDA(cudaEventCreate(&ctx->work.phase[i]), "phase event create");
  ctx->work.phase_timing = enable != 0;
  ctx->work.phase_recorded = false;
  return GLASS_OK;
}

extern "C" int glass_gpu_last_phase_ms(glass_gpu_ctx *ctx, float *ms) {
  if (!ctx || !ms) return set_err(GLASS_ERR_ARG, "glass_gpu_last_phase_ms: null argument");
  if (!ctx->work.phase_recorded)
    return set_err(GLASS_ERR_STATE, "glass_gpu_last_phase_ms: no step was launched with phase timing on");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  GLASS_CUDA(cudaEventSynchronize(ctx->work.phase[4]), "phase event sync");
  for (int i = 0; i < 4; i++)
    GLASS_CUDA(cudaEventElapsedTime(&ms[i], ctx->work.phase[i], ctx->work.phase[i + 1]), "phase elapsed time");
  return GLASS_OK;
}

static void apply_mixed_tol(glass_gpu_ctx *ctx) {
  const double t = ctx->mixed_tol;
  ctx->work.fb_e1 = t > 0 ? (float)(kMixedErrKa / t) : 0.f;
  ctx->work.fb_e2 = t > 0 ? (float)(kMixedErrKs / t) : 0.f;
}

extern "C" int glass_gpu_set_mixed_tolerance(glass_gpu_ctx *ctx, double tol) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "glass_gpu_set_mixed_tolerance: null context");
  if (!(tol == tol)) return set_err(GLASS_ERR_ARG, "glass_gpu_set_mixed_tolerance: NaN tolerance");
  if (tol != ctx->mixed_tol) clear_host_graphs(ctx);  // the estimate's scale is a kernel argument in the graphs
  ctx->mixed_tol = tol;
  apply_mixed_tol(ctx);
  return GLASS_OK;
}

extern "C" int glass_gpu_set_mixed_tolerance_scale(glass_gpu_ctx *ctx, int n, const double *scale) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "glass_gpu_set_mixed_tolerance_scale: null context");
  if (n < 0 || (n > 0 && !scale)) return set_err(GLASS_ERR_ARG, "glass_gpu_set_mixed_tolerance_scale: bad array");
  std::vector<float> inv((size_t)n);
  for (int i = 0; i < n; i++) {
    if (!(scale[i] > 0) || !isfinite(scale[i]))
      return set_err(GLASS_ERR_ARG, "glass_gpu_set_mixed_tolerance_scale: scales must be finite and positive");
    inv[i] = (float)(1.0 / scale[i]);
  }
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  FdWorkDev &w = ctx->work;
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "tolerance scale sync");
  if (n > w.fb_nscale_cap) {
    clear_host_graphs(ctx);  // the graphs hold the array's address
    cudaFree(w.fb_inv_scale);
    w.fb_inv_scale = nullptr;
    w.fb_nscale_cap = 0;
    GLASS_CUDA(cudaMalloc(&w.fb_inv_scale, sizeof(float) * (size_t)n), "cudaMalloc(tolerance scale)");
    w.fb_nscale_cap = n;
  }
  if (n > 0)
    GLASS_CUDA(cudaMemcpy(w.fb_inv_scale, inv.data(), sizeof(float) * (size_t)n, cudaMemcpyHostToDevice),
               "upload tolerance scale");
  if (n != w.fb_nscale) clear_host_graphs(ctx);  // the count is a kernel argument in the graphs
  w.fb_nscale = n;
  return GLASS_OK;
}

// Launch-shape parameters of the mixed path by name (the autotuner's knobs).
static int *tuning_slot(glass_gpu_ctx *ctx, const char *key, int *lo, int *hi) {
  FdWorkDev::Tuning &t = ctx->work.tune;
  struct Knob {
    const char *name;
    int *slot, lo, hi;
  } knobs[] = {{"slow_block", &t.slow_block, 128, 512},
               {"slow_ctas_per_sm", &t.slow_ctas_per_sm, 0, 16},
               {"spec_ctas_per_sm", &t.spec_ctas_per_sm, 0, 8},
               {"plan_per_cta", &t.plan_per_cta, 0, 32}};
  for (const Knob &k : knobs)
    if (!strcmp(key, k.name)) {
      *lo = k.lo;
      *hi = k.hi;
      return k.slot;
    }
  return nullptr;
}

// The checked build's failed-check sites since the last call (0 in a build
// without checks, which returns 0 from glass_gpu_checked_build).
extern "C" int glass_gpu_checked_build(void) { return kCheckedBuild ? 1 : 0; }

extern "C" int glass_gpu_check_status(glass_gpu_ctx *ctx, unsigned int *word) {
  if (!ctx || !word) return set_err(GLASS_ERR_ARG, "check_status: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "check_status sync");
  *word = check_status_all();
  return GLASS_OK;
}

extern "C" int glass_gpu_set_tuning(glass_gpu_ctx *ctx, const char *key, int value) {
  if (!ctx || !key) return set_err(GLASS_ERR_ARG, "glass_gpu_set_tuning: null argument");
  int lo = 0, hi = 0;
  int *slot = tuning_slot(ctx, key, &lo, &hi);
  if (!slot) return set_err(GLASS_ERR_ARG, "glass_gpu_set_tuning: unknown parameter %s", key);
  if (value < lo || value > hi || (!strcmp(key, "slow_block") && value != 128 && value != 256 && value != 512))
    return set_err(GLASS_ERR_ARG, "glass_gpu_set_tuning: value out of range for %s", key);
  if (*slot != value) clear_host_graphs(ctx);  // launch shapes are baked into recorded graphs
  *slot = value;
  return GLASS_OK;
}

extern "C" int glass_gpu_get_tuning(glass_gpu_ctx *ctx, const char *key, int *value) {
  if (!ctx || !key || !value) return set_err(GLASS_ERR_ARG, "glass_gpu_get_tuning: null argument");
  int lo = 0, hi = 0;
  int *slot = tuning_slot(ctx, key, &lo, &hi);
  if (!slot) return set_err(GLASS_ERR_ARG, "glass_gpu_get_tuning: unknown parameter %s", key);
  *value = *slot;
  return GLASS_OK;
}

extern "C" int glass_gpu_mixed_reevaluated(glass_gpu_ctx *ctx, unsigned long long *count) {
  if (!ctx || !count) return set_err(GLASS_ERR_ARG, "glass_gpu_mixed_reevaluated: null argument");
  *count = 0;
  if (!ctx->work.fb_total) return GLASS_OK;
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  GLASS_CUDA(cudaMemcpyAsync(count, ctx->work.fb_total, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             ctx->stream), "read re-evaluation count");
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "read re-evaluation count");
  return GLASS_OK;
}

static int is_pow2_in_range(int n);

extern "C" int glass_gpu_set_template_size(glass_gpu_ctx *ctx, int n) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "set_template_size: null context");
  if (n != 0 && !is_pow2_in_range(n)) return set_err(GLASS_ERR_SIZE, "set_template_size: n must be 0 or a power of two in [32, 4096]");
  if (ctx->n_fixed != n) clear_host_graphs(ctx);  // n is a kernel argument in the graphs
  ctx->n_fixed = n;
  return GLASS_OK;
}

// -------------------------------------------------------------------- bank
static int format_code(const char *format) {
  if (!format) return -1;
  if (strcmp(format, "sangria") == 0) return GLASS_FMT_SANGRIA;
  if (strcmp(format, "phase") == 0) return GLASS_FMT_PHASE;
  if (strcmp(format, "frequency") == 0) return GLASS_FMT_FREQUENCY;
  return -1;
}

static double fstar_of_orbit() { return kCLIGHT / (2.0 * M_PI * kLARM); }  // utils/src/glass_lisa.c:129

extern "C" int glass_gpu_bank_upload(glass_gpu_ctx *ctx, int format, double T, double t0, int NFFT, int nseg,
                                     const int *qmin, const double *rA, const double *rE, const double *invCA,
                                     const double *invCE) {
  if (!ctx || !qmin || !rA || !rE || !invCA || !invCE) return set_err(GLASS_ERR_ARG, "bank_upload: null argument");
  if (format < 0 || format > 2) return set_err(GLASS_ERR_FORMAT, "bank_upload: unknown format");
  if (nseg < 1 || NFFT < kMinN || !(T > 0)) return set_err(GLASS_ERR_ARG, "bank_upload: bad sizes");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const size_t nb = (size_t)nseg * NFFT;
  std::vector<float4> w32(nb), w32lo(nb), g32(2 * nb), g32lo(2 * nb);
  std::vector<double> Q((size_t)nseg * (NFFT + 1)), QA((size_t)nseg * (NFFT + 1));
  std::vector<double2> w64(2 * nb), g64(4 * nb);
  const double fstar = fstar_of_orbit();
  fd_build_bank_tables(format, T, fstar, NFFT, nseg, qmin, rA, rE, invCA, invCE, w32.data(), w32lo.data(),
                       g32.data(), Q.data(), w64.data(), g64.data(), QA.data(), g32lo.data());
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "bank_upload sync");
  clear_host_graphs(ctx);
  cudaFree(ctx->bank_mem);
  ctx->bank_mem = nullptr;
  size_t off_q = sizeof(int) * ((nseg + 63) / 64 * 64);
  size_t off_w32 = off_q + sizeof(double) * Q.size();
  off_w32 = (off_w32 + 255) / 256 * 256;
  size_t off_w32lo = off_w32 + sizeof(float4) * w32.size();
  size_t off_g32 = off_w32lo + sizeof(float4) * w32lo.size();
  size_t off_w64 = off_g32 + sizeof(float4) * g32.size();
  size_t off_g64 = off_w64 + sizeof(double2) * w64.size();
  size_t off_invc = off_g64 + sizeof(double2) * g64.size();
  size_t off_rho = (off_invc + sizeof(float2) * nb + 255) / 256 * 256;
  size_t off_qa = off_rho + sizeof(double) * nb;
  size_t off_g32lo = (off_qa + sizeof(double) * QA.size() + 255) / 256 * 256;
  size_t total = off_g32lo + sizeof(float4) * g32lo.size();
  GLASS_CUDA(cudaMalloc(&ctx->bank_mem, total), "cudaMalloc(bank)");
  char *base = (char *)ctx->bank_mem;
  FdBankDev &b = ctx->bank;
  b.nseg = nseg;
  b.NFFT = NFFT;
  b.format = format;
  b.T = T;
  b.t0 = t0;
  b.fstar = fstar;
  b.qmin = (int *)base;
  b.Q = (double *)(base + off_q);
  b.w32 = (float4 *)(base + off_w32);
  b.w32lo = (float4 *)(base + off_w32lo);
  b.g32 = (float4 *)(base + off_g32);
  b.w64 = (double2 *)(base + off_w64);
  b.g64 = (double2 *)(base + off_g64);
  b.invc = (float2 *)(base + off_invc);
  b.rho = (double *)(base + off_rho);
  b.QA = (double *)(base + off_qa);
  b.g32lo = (float4 *)(base + off_g32lo);
  GLASS_CUDA(cudaMemcpy(b.qmin, qmin, sizeof(int) * nseg, cudaMemcpyHostToDevice), "upload qmin");
  GLASS_CUDA(cudaMemcpy(b.Q, Q.data(), sizeof(double) * Q.size(), cudaMemcpyHostToDevice), "upload Q");
  GLASS_CUDA(cudaMemcpy(b.QA, QA.data(), sizeof(double) * QA.size(), cudaMemcpyHostToDevice), "upload QA");
  GLASS_CUDA(cudaMemcpy(b.w32, w32.data(), sizeof(float4) * w32.size(), cudaMemcpyHostToDevice), "upload w32");
  GLASS_CUDA(cudaMemcpy(b.w32lo, w32lo.data(), sizeof(float4) * w32lo.size(), cudaMemcpyHostToDevice), "upload w32lo");
  GLASS_CUDA(cudaMemcpy(b.g32, g32.data(), sizeof(float4) * g32.size(), cudaMemcpyHostToDevice), "upload g32");
  GLASS_CUDA(cudaMemcpy(b.g32lo, g32lo.data(), sizeof(float4) * g32lo.size(), cudaMemcpyHostToDevice),
             "upload g32lo");
  GLASS_CUDA(cudaMemcpy(b.w64, w64.data(), sizeof(double2) * w64.size(), cudaMemcpyHostToDevice), "upload w64");
  GLASS_CUDA(cudaMemcpy(b.g64, g64.data(), sizeof(double2) * g64.size(), cudaMemcpyHostToDevice), "upload g64");
  {
    // invC relative to the segment's first bin (only ratios are used; invC
    // itself, ~1e41, is beyond FP32 range)
    std::vector<float2> ic(nb);
    for (int sg = 0; sg < nseg; sg++)
      for (int j = 0; j < NFFT; j++) {
        size_t sj = (size_t)sg * NFFT + j, s0 = (size_t)sg * NFFT;
        ic[sj] = make_float2((float)(invCA[sj] / invCA[s0]), (float)(invCE[sj] / invCE[s0]));
      }
    GLASS_CUDA(cudaMemcpy(b.invc, ic.data(), sizeof(float2) * nb, cudaMemcpyHostToDevice), "upload invc");
    std::vector<double> rho(nb);
    for (size_t sj = 0; sj < nb; sj++) rho[sj] = invCA[sj] / invCE[sj];
    GLASS_CUDA(cudaMemcpy(b.rho, rho.data(), sizeof(double) * nb, cudaMemcpyHostToDevice), "upload rho");
  }
  ctx->h_qmin.assign(qmin, qmin + nseg);
  ctx->h_invCA.assign(invCA, invCA + nb);
  ctx->h_invCE.assign(invCE, invCE + nb);
  if (!ctx->tab_ready || ctx->tab_T != T || ctx->tab_t0 != t0) {
    GLASS_CUDA(fd_build_orbit_tables(ctx->tab, T, t0, ctx->stream), "orbit tables");
    GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "orbit tables sync");
    ctx->tab_ready = true;
    ctx->tab_T = T;
    ctx->tab_t0 = t0;
  }
  return GLASS_OK;
}

extern "C" int glass_gpu_bank_set_residual(glass_gpu_ctx *ctx, int seg, const double *rA, const double *rE) {
  if (!ctx || !rA || !rE) return set_err(GLASS_ERR_ARG, "bank_set_residual: null argument");
  FdBankDev &b = ctx->bank;
  if (!b.nseg) return set_err(GLASS_ERR_STATE, "bank_set_residual: no bank");
  if (seg < 0 || seg >= b.nseg) return set_err(GLASS_ERR_ARG, "bank_set_residual: segment out of range");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const int NFFT = b.NFFT;
  std::vector<float4> w32(NFFT), w32lo(NFFT), g32(2 * NFFT);
  std::vector<double> Q(NFFT + 1), QA(NFFT + 1);
  std::vector<double2> w64(2 * NFFT), g64(4 * NFFT);
  fd_build_bank_tables(b.format, b.T, b.fstar, NFFT, 1, &ctx->h_qmin[seg], rA, rE,
                       ctx->h_invCA.data() + (size_t)seg * NFFT, ctx->h_invCE.data() + (size_t)seg * NFFT,
                       w32.data(), w32lo.data(), g32.data(), Q.data(), w64.data(), g64.data(), QA.data());
  size_t sj = (size_t)seg * NFFT;
  GLASS_CUDA(cudaMemcpyAsync(b.w32 + sj, w32.data(), sizeof(float4) * NFFT, cudaMemcpyHostToDevice, ctx->stream),
             "residual w32");
  GLASS_CUDA(cudaMemcpyAsync(b.w32lo + sj, w32lo.data(), sizeof(float4) * NFFT, cudaMemcpyHostToDevice, ctx->stream),
             "residual w32lo");
  GLASS_CUDA(cudaMemcpyAsync(b.Q + (size_t)seg * (NFFT + 1), Q.data(), sizeof(double) * (NFFT + 1),
                             cudaMemcpyHostToDevice, ctx->stream), "residual Q");
  GLASS_CUDA(cudaMemcpyAsync(b.QA + (size_t)seg * (NFFT + 1), QA.data(), sizeof(double) * (NFFT + 1),
                             cudaMemcpyHostToDevice, ctx->stream), "residual QA");
  GLASS_CUDA(cudaMemcpyAsync(b.w64 + 2 * sj, w64.data(), sizeof(double2) * 2 * NFFT, cudaMemcpyHostToDevice,
                             ctx->stream), "residual w64");
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "residual sync");
  return GLASS_OK;
}

static int is_pow2_in_range(int n) { return n >= kMinN && n <= kMaxN && (n & (n - 1)) == 0; }

// --------------------------------------------------------------- batched
// Scratch for a batch: per-proposal constants, size lists and the slow-part
// series (4 complex series of N <= NFFT samples per proposal), sized for the
// worst case so that a batch never allocates once the context has seen a batch
// of that size (required for CUDA-graph capture of glass_gpu_dlogl_batch).
static int ensure_work(glass_gpu_ctx *ctx, int nitems) {
  FdWorkDev &w = ctx->work;
  size_t series = fd_series_bytes(nitems, ctx->bank.NFFT, GLASS_PREC_FP64);
  size_t gseries = fd_grad_series_bytes(nitems, ctx->bank.NFFT);
  if (gseries > series) series = gseries;
  if (nitems <= w.cap && series <= w.series_bytes) return GLASS_OK;
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "work sync");
  clear_host_graphs(ctx);
  cudaFree(w.items64);
  cudaFree(w.itemsmix);
  cudaFree(w.itemsgrad);
  cudaFree(w.bin_count);
  cudaFree(w.bin_list);
  cudaFree(w.series);
  cudaFree(w.series2);
  cudaFree(w.hp_list);
  w.hp_list = nullptr;
  w.hp_count = nullptr;
  w.fb_count = nullptr;
  w.items64 = nullptr;
  w.itemsmix = nullptr;
  w.itemsgrad = nullptr;
  w.bin_count = nullptr;
  w.bin_list = nullptr;
  w.series = nullptr;
  w.series2 = nullptr;
  w.cap = 0;
  w.series_bytes = 0;
  int cap = nitems < 1024 ? 1024 : nitems;
  series = fd_series_bytes(cap, ctx->bank.NFFT, GLASS_PREC_FP64);
  gseries = fd_grad_series_bytes(cap, ctx->bank.NFFT);
  if (gseries > series) series = gseries;
  GLASS_CUDA(cudaMalloc(&w.items64, sizeof(ItemF64) * (size_t)cap), "cudaMalloc(items64)");
  GLASS_CUDA(cudaMalloc(&w.itemsmix, sizeof(ItemMix) * (size_t)cap), "cudaMalloc(itemsmix)");
  GLASS_CUDA(cudaMalloc(&w.itemsgrad, sizeof(ItemGrad) * (size_t)cap), "cudaMalloc(itemsgrad)");
  GLASS_CUDA(cudaMalloc(&w.bin_count, sizeof(int) * kFdCounts), "cudaMalloc(bin_count)");
  GLASS_CUDA(cudaMemset(w.bin_count, 0, sizeof(int) * kFdCounts), "cudaMemset(bin_count)");
  w.fb_count = w.bin_count + kNumBins;
  w.hp_count = w.bin_count + kNumBins + 6;
  GLASS_CUDA(cudaMalloc(&w.hp_list, sizeof(int) * (size_t)kNumBins * cap), "cudaMalloc(hp_list)");
  if (!w.fb_total) {
    GLASS_CUDA(cudaMalloc(&w.fb_total, sizeof(unsigned long long)), "cudaMalloc(fb_total)");
    GLASS_CUDA(cudaMemset(w.fb_total, 0, sizeof(unsigned long long)), "cudaMemset(fb_total)");
  }
  apply_mixed_tol(ctx);
  w.counts_zero = true;
  GLASS_CUDA(cudaMalloc(&w.bin_list, sizeof(int) * (size_t)kNumBins * cap), "cudaMalloc(bin_list)");
  GLASS_CUDA(cudaMalloc(&w.series, series), "cudaMalloc(series)");
  GLASS_CUDA(cudaMalloc(&w.series2, series), "cudaMalloc(series2)");
  w.cap = cap;
  w.series_bytes = series;
  return GLASS_OK;
}

extern "C" int glass_gpu_dlogl_batch(glass_gpu_ctx *ctx, int precision, int nitems, const int *item_seg,
                                     const double *params, const double *term_x, double *dlogl, double *term_y,
                                     double *hh, int *status) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "dlogl_batch: null context");
  if (nitems < 0) return set_err(GLASS_ERR_ARG, "dlogl_batch: negative item count");
  if (nitems == 0) return GLASS_OK;
  if (!item_seg || !params || !dlogl) return set_err(GLASS_ERR_ARG, "dlogl_batch: null argument");
  if (precision != GLASS_PREC_FP64 && precision != GLASS_PREC_MIXED)
    return set_err(GLASS_ERR_ARG, "dlogl_batch: unknown precision");
  if (!ctx->bank.nseg) return set_err(GLASS_ERR_STATE, "dlogl_batch: no segment bank uploaded");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  if ((rc = ensure_work(ctx, nitems))) return rc;
  int nl = 0;
  if (ctx->n_fixed > ctx->bank.NFFT) return set_err(GLASS_ERR_SIZE, "dlogl_batch: template size above NFFT");
  cudaError_t e = fd_dlogl_launch(ctx->bank, ctx->tab, ctx->work, precision, nitems, item_seg, params, term_x, dlogl,
                                  term_y, hh, status, ctx->n_fixed, ctx->num_sms, ctx->stream, &nl);
  ctx->last_launches = nl;
  if (e != cudaSuccess) return cuda_err(e, "dlogl_batch launch");
  return GLASS_OK;
}

extern "C" int glass_gpu_dlogl_batch_channels(glass_gpu_ctx *ctx, int precision, int nitems, const int *item_seg,
                                              const double *params, const double *term_x, double *dlogl,
                                              double *term_y, double *hh, int *status, double *term_ch) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "dlogl_batch_channels: null context");
  if (nitems < 0) return set_err(GLASS_ERR_ARG, "dlogl_batch_channels: negative item count");
  if (nitems == 0) return GLASS_OK;
  if (!item_seg || !params || !dlogl || !term_ch) return set_err(GLASS_ERR_ARG, "dlogl_batch_channels: null argument");
  if (precision != GLASS_PREC_FP64 && precision != GLASS_PREC_MIXED)
    return set_err(GLASS_ERR_ARG, "dlogl_batch_channels: unknown precision");
  if (!ctx->bank.nseg) return set_err(GLASS_ERR_STATE, "dlogl_batch_channels: no segment bank uploaded");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  if ((rc = ensure_work(ctx, nitems))) return rc;
  if (ctx->n_fixed > ctx->bank.NFFT) return set_err(GLASS_ERR_SIZE, "dlogl_batch_channels: template size above NFFT");
  int nl = 0;
  cudaError_t e = fd_dlogl_launch(ctx->bank, ctx->tab, ctx->work, precision, nitems, item_seg, params, term_x, dlogl,
                                  term_y, hh, status, ctx->n_fixed, ctx->num_sms, ctx->stream, &nl, term_ch);
  ctx->last_launches = nl;
  if (e != cudaSuccess) return cuda_err(e, "dlogl_batch_channels launch");
  return GLASS_OK;
}

static int ensure_stage(glass_gpu_ctx *ctx, size_t bytes) {
  if (bytes <= ctx->d_stage_cap) return GLASS_OK;
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "stage sync");
  clear_host_graphs(ctx);
  cudaFree(ctx->d_stage);
  ctx->d_stage = nullptr;
  GLASS_CUDA(cudaMalloc(&ctx->d_stage, bytes), "cudaMalloc(stage)");
  ctx->d_stage_cap = bytes;
  return GLASS_OK;
}

static int ensure_host_stage(glass_gpu_ctx *ctx, size_t bytes) {
  if (bytes <= ctx->h_stage_cap) return GLASS_OK;
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "host stage sync");
  clear_host_graphs(ctx);
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  ctx->h_stage = nullptr;
  ctx->h_stage_cap = 0;
  GLASS_CUDA(cudaMallocHost(&ctx->h_stage, bytes), "cudaMallocHost(stage)");
  ctx->h_stage_cap = bytes;
  return GLASS_OK;
}

// Copy-in, the batch, copy-out on the context's stream; stage layout (device
// and pinned host alike): inputs params (8n doubles) | term_x (n doubles) |
// item_seg (n ints), then at out_off the outputs dlogl | term_y | hh (n
// doubles each) | status (n ints).
// Direct host access.  The pointer block is re-read on every launch: the
// first threads of each gather CTA load it (ld.global.cv) into shared memory
// and CTA 0 leaves a device copy for the scatter kernel; the caller's arrays
// are read the same way, since both change between replays of one graph, and
// the outputs are written through (st.global.wt).
__device__ __forceinline__ void host_io_load_block(const HostIo *io, HostIo *s, HostIo *d_io) {
  const unsigned long long *w = reinterpret_cast<const unsigned long long *>(io);
  unsigned long long *sw = reinterpret_cast<unsigned long long *>(s);
  constexpr int kWords = sizeof(HostIo) / sizeof(unsigned long long);
  if (threadIdx.x < kWords) {
    const unsigned long long v = __ldcv(w + threadIdx.x);
    sw[threadIdx.x] = v;
    if (blockIdx.x == 0) reinterpret_cast<unsigned long long *>(d_io)[threadIdx.x] = v;
  }
  __syncthreads();
}

// params (8n doubles), term_x (n, when given), item_seg (n ints) into the
// device stage: one element per thread over a flat index (16-byte pairs of
// params where the caller's array allows), so that each thread waits for one
// host-memory round trip, not one per array
__global__ void host_gather_kernel(const HostIo *io, HostIo *d_io, int n, double *d_params, double *d_tx,
                                   int *d_seg) {
  __shared__ HostIo h;
  host_io_load_block(io, &h, d_io);
  const bool v2 = (reinterpret_cast<unsigned long long>(h.params) & 15) == 0;
  const long long np = v2 ? 4LL * n : 8LL * n;  // params elements
  const long long tot = np + 2LL * n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += stride) {
    if (i < np) {
      if (v2)
        reinterpret_cast<double2 *>(d_params)[i] = __ldcv(reinterpret_cast<const double2 *>(h.params) + i);
      else
        d_params[i] = __ldcv(h.params + i);
    } else if (i < np + n) {
      if (h.term_x) d_tx[i - np] = __ldcv(h.term_x + (i - np));
    } else {
      d_seg[i - np - n] = __ldcv(h.item_seg + (i - np - n));
    }
  }
}

// dlogl, term_y, hh (n doubles each) and status (n ints) to the caller's
// arrays, one element per thread; the three optional ones are skipped when NULL
__global__ void host_scatter_kernel(const HostIo *d_io, int n, const double *d_dl, const double *d_ty,
                                    const double *d_hh, const int *d_st) {
  const HostIo h = *d_io;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < 4LL * n; i += stride) {
    const int q = (int)(i / n);
    const long long j = i - (long long)q * n;
    if (q == 0) {
      __stwt(h.dlogl + j, d_dl[j]);
    } else if (q == 1) {
      if (h.term_y) __stwt(h.term_y + j, d_ty[j]);
    } else if (q == 2) {
      if (h.hh) __stwt(h.hh + j, d_hh[j]);
    } else if (h.status) {
      __stwt(h.status + j, d_st[j]);
    }
  }
}

static int host_copy_grid(const glass_gpu_ctx *ctx, long long elems) {
  const long long b = (elems + 255) / 256;
  return (int)std::max(1LL, std::min(b, 4LL * ctx->num_sms));
}

// gather, the batch, scatter on the context's stream (same stage layout as
// dlogl_host_enqueue below)
static int dlogl_direct_enqueue(glass_gpu_ctx *ctx, int precision, int nitems, bool has_tx, size_t out_off) {
  const size_t nd = (size_t)nitems;
  char *d = (char *)ctx->d_stage;
  double *d_params = (double *)d, *d_tx = d_params + 8 * nd;
  int *d_seg = (int *)(d_tx + nd);
  double *d_dl = (double *)(d + out_off), *d_ty = d_dl + nd, *d_hh = d_ty + nd;
  int *d_st = (int *)(d_hh + nd);
  cudaStream_t s = ctx->stream;
  // the device copy of the pointer block sits after the outputs
  HostIo *d_io = (HostIo *)(d + out_off + ((sizeof(double) * 3 * nd + sizeof(int) * nd + 15) / 16) * 16);
  host_gather_kernel<<<host_copy_grid(ctx, 6LL * nitems), 256, 0, s>>>(ctx->h_io, d_io, nitems, d_params, d_tx,
                                                                       d_seg);
  GLASS_CUDA(cudaGetLastError(), "host_gather_kernel launch");
  int rc = glass_gpu_dlogl_batch(ctx, precision, nitems, d_seg, d_params, has_tx ? d_tx : nullptr, d_dl, d_ty, d_hh,
                                 d_st);
  if (rc) return rc;
  host_scatter_kernel<<<host_copy_grid(ctx, 4LL * nitems), 256, 0, s>>>(d_io, nitems, d_dl, d_ty, d_hh, d_st);
  GLASS_CUDA(cudaGetLastError(), "host_scatter_kernel launch");
  ctx->last_launches += 2;
  return GLASS_OK;
}

static int dlogl_host_enqueue(glass_gpu_ctx *ctx, int precision, int nitems, bool has_tx, size_t in_bytes,
                              size_t out_off, size_t out_bytes) {
  const size_t nd = (size_t)nitems;
  char *d = (char *)ctx->d_stage;
  char *h = (char *)ctx->h_stage;
  double *d_params = (double *)d, *d_tx = d_params + 8 * nd;
  int *d_seg = (int *)(d_tx + nd);
  double *d_dl = (double *)(d + out_off), *d_ty = d_dl + nd, *d_hh = d_ty + nd;
  int *d_st = (int *)(d_hh + nd);
  cudaStream_t s = ctx->stream;
  GLASS_CUDA(cudaMemcpyAsync(d, h, in_bytes, cudaMemcpyHostToDevice, s), "H2D batch inputs");
  int rc = glass_gpu_dlogl_batch(ctx, precision, nitems, d_seg, d_params, has_tx ? d_tx : nullptr, d_dl, d_ty, d_hh,
                                 d_st);
  if (rc) return rc;
  GLASS_CUDA(cudaMemcpyAsync(h + out_off, d + out_off, out_bytes, cudaMemcpyDeviceToHost, s), "D2H batch outputs");
  return GLASS_OK;
}

extern "C" int glass_gpu_dlogl_batch_host(glass_gpu_ctx *ctx, int precision, int nitems, const int *item_seg,
                                          const double *params, const double *term_x, double *dlogl,
                                          double *term_y, double *hh, int *status) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "dlogl_batch_host: null context");
  if (nitems < 0) return set_err(GLASS_ERR_ARG, "dlogl_batch_host: negative item count");
  if (nitems == 0) return GLASS_OK;
  if (!item_seg || !params || !dlogl) return set_err(GLASS_ERR_ARG, "dlogl_batch_host: null argument");
  if (precision != GLASS_PREC_FP64 && precision != GLASS_PREC_MIXED)
    return set_err(GLASS_ERR_ARG, "dlogl_batch_host: unknown precision");
  if (!ctx->bank.nseg) return set_err(GLASS_ERR_STATE, "dlogl_batch_host: no segment bank uploaded");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const size_t nd = (size_t)nitems;
  const bool has_tx = term_x != nullptr;
  const size_t in_bytes = sizeof(double) * 9 * nd + sizeof(int) * nd;
  const size_t out_off = (in_bytes + 255) / 256 * 256;
  const size_t out_bytes = sizeof(double) * 3 * nd + sizeof(int) * nd;
  const size_t bytes = out_off + out_bytes;
  cudaStream_t s = ctx->stream;
  if (ctx->host_direct) {
    // + the device copy of the pointer block
    if ((rc = ensure_stage(ctx, out_off + (out_bytes + 15) / 16 * 16 + sizeof(HostIo)))) return rc;
    if ((rc = ensure_work(ctx, nitems))) return rc;
    if (!ctx->h_io) GLASS_CUDA(cudaMallocHost(&ctx->h_io, sizeof(HostIo)), "cudaMallocHost(host io)");
    // the previous call synchronised, so no kernel reads the block now
    HostIo *io = ctx->h_io;
    io->params = params;
    io->term_x = term_x;
    io->item_seg = item_seg;
    io->dlogl = dlogl;
    io->term_y = term_y;
    io->hh = hh;
    io->status = status;
    const long long key = ((long long)nitems << 4) | (1LL << 3) | ((long long)precision << 1) | (has_tx ? 1 : 0);
    auto it = ctx->host_graphs.find(key);
    if (it != ctx->host_graphs.end() && !ctx->work.phase_timing) {
      GLASS_CUDA(cudaGraphLaunch(it->second, s), "dlogl_batch_host graph launch");
      ctx->last_launches = 5;
    } else {
      if ((rc = dlogl_direct_enqueue(ctx, precision, nitems, has_tx, out_off))) return rc;
      GLASS_CUDA(cudaStreamSynchronize(s), "dlogl_batch_host sync");
      if (!ctx->work.phase_timing && ctx->host_graphs.size() < 64) {
        const int nl = ctx->last_launches;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
          const int rc2 = dlogl_direct_enqueue(ctx, precision, nitems, has_tx, out_off);
          const cudaError_t e2 = cudaStreamEndCapture(s, &g);
          if (rc2 == GLASS_OK && e2 == cudaSuccess && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess)
            ctx->host_graphs[key] = ge;
          if (g) cudaGraphDestroy(g);
        }
        cudaGetLastError();
        ctx->last_launches = nl;
      }
    }
    GLASS_CUDA(cudaStreamSynchronize(s), "dlogl_batch_host sync");
    return GLASS_OK;
  }
  // buffers first, so that nothing is reallocated while a graph is recorded
  if ((rc = ensure_stage(ctx, bytes))) return rc;
  if ((rc = ensure_host_stage(ctx, bytes))) return rc;
  if ((rc = ensure_work(ctx, nitems))) return rc;
  char *h = (char *)ctx->h_stage;
  memcpy(h, params, sizeof(double) * 8 * nd);
  if (has_tx) memcpy(h + sizeof(double) * 8 * nd, term_x, sizeof(double) * nd);
  memcpy(h + sizeof(double) * 9 * nd, item_seg, sizeof(int) * nd);
  const long long key = ((long long)nitems << 4) | ((long long)precision << 1) | (has_tx ? 1 : 0);
  auto it = ctx->host_graphs.find(key);
  if (it != ctx->host_graphs.end() && !ctx->work.phase_timing) {
    GLASS_CUDA(cudaGraphLaunch(it->second, s), "dlogl_batch_host graph launch");
    ctx->last_launches = 3;
  } else {
    if ((rc = dlogl_host_enqueue(ctx, precision, nitems, has_tx, in_bytes, out_off, out_bytes))) return rc;
    GLASS_CUDA(cudaStreamSynchronize(s), "dlogl_batch_host sync");
    if (!ctx->work.phase_timing && ctx->host_graphs.size() < 64) {
      // record the sequence for the next calls of this shape (a stream that
      // cannot be captured keeps the direct path)
      const int nl = ctx->last_launches;
      cudaGraph_t g = nullptr;
      cudaGraphExec_t ge = nullptr;
      if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const int rc2 = dlogl_host_enqueue(ctx, precision, nitems, has_tx, in_bytes, out_off, out_bytes);
        const cudaError_t e2 = cudaStreamEndCapture(s, &g);
        if (rc2 == GLASS_OK && e2 == cudaSuccess && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess)
          ctx->host_graphs[key] = ge;
        if (g) cudaGraphDestroy(g);
      }
      cudaGetLastError();
      ctx->last_launches = nl;
    }
  }
  GLASS_CUDA(cudaStreamSynchronize(s), "dlogl_batch_host sync");
  const char *o = h + out_off;
  memcpy(dlogl, o, sizeof(double) * nd);
  if (term_y) memcpy(term_y, o + sizeof(double) * nd, sizeof(double) * nd);
  if (hh) memcpy(hh, o + sizeof(double) * 2 * nd, sizeof(double) * nd);
  if (status) memcpy(status, o + sizeof(double) * 3 * nd, sizeof(int) * nd);
  return GLASS_OK;
}

extern "C" int glass_gpu_grad_fisher_batch(glass_gpu_ctx *ctx, int nitems, const int *item_seg,
                                           const double *params, int fisher_mode, double *term_y, double *grad,
                                           double *fisher, int *status) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "grad_fisher_batch: null context");
  if (nitems < 0) return set_err(GLASS_ERR_ARG, "grad_fisher_batch: negative item count");
  if (nitems == 0) return GLASS_OK;
  if (!item_seg || !params || !term_y || !grad) return set_err(GLASS_ERR_ARG, "grad_fisher_batch: null argument");
  const int n_fixed = ctx->n_fixed;
  if (n_fixed > kMaxN || n_fixed > ctx->bank.NFFT)
    return set_err(GLASS_ERR_SIZE, "grad_fisher_batch: template size above min(4096, NFFT)");
  if (fisher_mode != 0 && fisher_mode != 1) return set_err(GLASS_ERR_ARG, "grad_fisher_batch: unknown fisher_mode");
  if (!ctx->bank.nseg) return set_err(GLASS_ERR_STATE, "grad_fisher_batch: no segment bank uploaded");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  if ((rc = ensure_work(ctx, nitems))) return rc;
  int nl = 0;
  cudaError_t e = fd_grad_launch(ctx->bank, ctx->tab, ctx->work, nitems, item_seg, params, n_fixed, fisher_mode,
                                 term_y, grad, fisher, status, ctx->num_sms, ctx->stream, &nl);
  ctx->last_launches = nl;
  if (e != cudaSuccess) return cuda_err(e, "grad_fisher_batch launch");
  return GLASS_OK;
}

extern "C" int glass_gpu_grad_fisher_batch_host(glass_gpu_ctx *ctx, int nitems, const int *item_seg,
                                                const double *params, int fisher_mode, double *term_y,
                                                double *grad, double *fisher, int *status) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "grad_fisher_batch_host: null context");
  if (nitems < 0) return set_err(GLASS_ERR_ARG, "grad_fisher_batch_host: negative item count");
  if (nitems == 0) return GLASS_OK;
  if (!item_seg || !params || !term_y || !grad) return set_err(GLASS_ERR_ARG, "grad_fisher_batch_host: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  size_t nd = (size_t)nitems;
  size_t bytes = sizeof(double) * nd * (8 + 1 + 8 + 64) + sizeof(int) * nd * 2 + 256;
  if ((rc = ensure_stage(ctx, bytes))) return rc;
  double *d_params = (double *)ctx->d_stage;
  double *d_ty = d_params + 8 * nd;
  double *d_g = d_ty + nd;
  double *d_f = d_g + 8 * nd;
  int *d_seg = (int *)(d_f + 64 * nd);
  int *d_st = d_seg + nd;
  cudaStream_t s = ctx->stream;
  GLASS_CUDA(cudaMemcpyAsync(d_params, params, sizeof(double) * 8 * nd, cudaMemcpyHostToDevice, s), "H2D params");
  GLASS_CUDA(cudaMemcpyAsync(d_seg, item_seg, sizeof(int) * nd, cudaMemcpyHostToDevice, s), "H2D item_seg");
  rc = glass_gpu_grad_fisher_batch(ctx, nitems, d_seg, d_params, fisher_mode, d_ty, d_g, fisher ? d_f : nullptr,
                                   d_st);
  if (rc) return rc;
  GLASS_CUDA(cudaMemcpyAsync(term_y, d_ty, sizeof(double) * nd, cudaMemcpyDeviceToHost, s), "D2H term_y");
  GLASS_CUDA(cudaMemcpyAsync(grad, d_g, sizeof(double) * 8 * nd, cudaMemcpyDeviceToHost, s), "D2H grad");
  if (fisher) GLASS_CUDA(cudaMemcpyAsync(fisher, d_f, sizeof(double) * 64 * nd, cudaMemcpyDeviceToHost, s), "D2H fisher");
  if (status) GLASS_CUDA(cudaMemcpyAsync(status, d_st, sizeof(int) * nd, cudaMemcpyDeviceToHost, s), "D2H status");
  GLASS_CUDA(cudaStreamSynchronize(s), "grad_fisher_batch_host sync");
  return GLASS_OK;
}

// ------------------------------------------------------------ F-statistic
// Scratch of the F-statistic batches: cells per launch sequence bounded so
// that the filter series (16 N complex doubles per cell at the segment's
// largest filter size) stay within kFsSeriesBudget.
static constexpr size_t kFsSeriesBudget = (size_t)2 << 30;

static int ensure_fs_work(glass_gpu_ctx *ctx, int ncells) {
  int maxN = fs_max_size(ctx->bank.NFFT);
  if (maxN > kMaxN) maxN = kMaxN;
  const size_t per_cell = (size_t)16 * maxN * sizeof(double2);
  size_t chunk = kFsSeriesBudget / per_cell;
  if (chunk < 256) chunk = 256;
  size_t want = 256;
  while (want < (size_t)ncells && want < chunk) want *= 2;
  if (want > chunk) want = chunk;
  FsWorkDev &w = ctx->fsw;
  if (w.mem && (size_t)w.cap >= want && w.series_bytes >= (size_t)w.cap * per_cell) return GLASS_OK;
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "fstat work sync");
  GLASS_CUDA(fs_work_alloc(w, (int)want, ctx->bank.NFFT), "cudaMalloc(fstat work)");
  return GLASS_OK;
}

extern "C" int glass_gpu_fstat_batch(glass_gpu_ctx *ctx, int ncells, const int *cell_seg, const double *cells,
                                     double *logl, double *fparams, int *status) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "fstat_batch: null context");
  if (ncells < 0) return set_err(GLASS_ERR_ARG, "fstat_batch: negative cell count");
  if (ncells == 0) return GLASS_OK;
  if (!cell_seg || !cells || !logl) return set_err(GLASS_ERR_ARG, "fstat_batch: null argument");
  if (!ctx->bank.nseg) return set_err(GLASS_ERR_STATE, "fstat_batch: no segment bank uploaded");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  if ((rc = ensure_fs_work(ctx, ncells))) return rc;
  int nl = 0;
  cudaError_t e = fs_launch(ctx->bank, ctx->tab, ctx->bank.rho, ctx->fsw, ncells, cell_seg, 0, cells, logl, fparams,
                            status, ctx->num_sms, ctx->stream, &nl);
  ctx->last_launches = nl;
  if (e != cudaSuccess) return cuda_err(e, "fstat_batch launch");
  return GLASS_OK;
}

extern "C" int glass_gpu_fstat_batch_host(glass_gpu_ctx *ctx, int ncells, const int *cell_seg, const double *cells,
                                          double *logl, double *fparams, int *status) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "fstat_batch_host: null context");
  if (ncells < 0) return set_err(GLASS_ERR_ARG, "fstat_batch_host: negative cell count");
  if (ncells == 0) return GLASS_OK;
  if (!cell_seg || !cells || !logl) return set_err(GLASS_ERR_ARG, "fstat_batch_host: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const size_t nd = (size_t)ncells;
  if ((rc = ensure_stage(ctx, sizeof(double) * nd * (4 + 1 + 4) + sizeof(int) * nd * 2 + 256))) return rc;
  double *d_cells = (double *)ctx->d_stage;
  double *d_logl = d_cells + 4 * nd;
  double *d_fp = d_logl + nd;
  int *d_seg = (int *)(d_fp + 4 * nd);
  int *d_st = d_seg + nd;
  cudaStream_t s = ctx->stream;
  GLASS_CUDA(cudaMemcpyAsync(d_cells, cells, sizeof(double) * 4 * nd, cudaMemcpyHostToDevice, s), "H2D cells");
  GLASS_CUDA(cudaMemcpyAsync(d_seg, cell_seg, sizeof(int) * nd, cudaMemcpyHostToDevice, s), "H2D cell_seg");
  rc = glass_gpu_fstat_batch(ctx, ncells, d_seg, d_cells, d_logl, fparams ? d_fp : nullptr, d_st);
  if (rc) return rc;
  GLASS_CUDA(cudaMemcpyAsync(logl, d_logl, sizeof(double) * nd, cudaMemcpyDeviceToHost, s), "D2H logl");
  if (fparams)
    GLASS_CUDA(cudaMemcpyAsync(fparams, d_fp, sizeof(double) * 4 * nd, cudaMemcpyDeviceToHost, s), "D2H fparams");
  if (status) GLASS_CUDA(cudaMemcpyAsync(status, d_st, sizeof(int) * nd, cudaMemcpyDeviceToHost, s), "D2H status");
  GLASS_CUDA(cudaStreamSynchronize(s), "fstat_batch_host sync");
  return GLASS_OK;
}

// ucb/src/glass_ucb_waveform.c:307-314 (ucb_fdot)
static double host_ucb_fdot(double Mc, double f0) {
  double M = Mc * 4.92569043916e-6;  // TSUN, utils/src/glass_constants.h:60
  return 19.2 * pow(pow(M_PI, 8) * pow(M, 5) * pow(f0, 11), 1. / 3.);
}

extern "C" int glass_gpu_fstat_proposal_host(glass_gpu_ctx *ctx, int seg, int n_theta, int n_phi, double *tensor,
                                             double *info) {
  if (!ctx || !tensor || !info) return set_err(GLASS_ERR_ARG, "fstat_proposal_host: null argument");
  const FdBankDev &b = ctx->bank;
  if (!b.nseg) return set_err(GLASS_ERR_STATE, "fstat_proposal_host: no segment bank uploaded");
  if (seg < 0 || seg >= b.nseg) return set_err(GLASS_ERR_ARG, "fstat_proposal_host: segment out of range");
  if (n_theta < 1 || n_phi < 1) return set_err(GLASS_ERR_ARG, "fstat_proposal_host: empty sky grid");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  // the segment's frequency range as the reference holds it
  // (utils/src/glass_data.c:1077-1078, 2065-2066) and the grid of
  // setup_fstatistic_proposal (ucb/src/glass_ucb_proposal.c:927-943)
  const double T = b.T;
  const int qmin = ctx->h_qmin[seg];
  double fmin = (double)qmin / T;
  while ((int)(fmin * T) < qmin) fmin = nextafter(fmin, INFINITY);
  const double fmax = fmin + b.NFFT / T;
  FsGrid G;
  G.n_f = (int)((fmax - fmin) * T);
  G.n_theta = n_theta;
  G.n_phi = n_phi;
  G.fmin = fmin;
  G.d_f = (int)((fmax - fmin) * T) / (double)G.n_f / T;
  G.d_theta = 2. / (double)n_theta;
  G.d_phi = kPI2 / (double)n_phi;
  if (G.n_f < 1) return set_err(GLASS_ERR_ARG, "fstat_proposal_host: empty frequency grid");
  const long long nll = (long long)G.n_f * n_theta * n_phi;
  if (nll > (1LL << 28)) return set_err(GLASS_ERR_ARG, "fstat_proposal_host: grid too large");
  const int n = (int)nll;
  // chirp-mass scan values per frequency row (:1099-1100, :1142)
  std::vector<double> fdot_tab((size_t)G.n_f * kFsScan);
  const double dMc = (1.1 - 0.1) / kFsScan;
  for (int i = 0; i < G.n_f; i++) {
    double f = fmin + i * G.d_f;
    f += G.d_f / 2;
    for (int s = 0; s < kFsScan; s++) fdot_tab[(size_t)i * kFsScan + s] = host_ucb_fdot(0.1 + s * dMc, f);
  }
  if ((rc = ensure_fs_work(ctx, n))) return rc;
  cudaStream_t st = ctx->stream;
  // scratch: grid cells, logL at fdot = 0, scan bookkeeping, density
  char *mem = nullptr;
  const size_t n_d = (size_t)n;
  size_t off_logl0 = sizeof(double) * 4 * n_d;
  size_t off_tensor = off_logl0 + sizeof(double) * n_d;
  size_t off_fdot = off_tensor + sizeof(double) * n_d;
  size_t off_pos = off_fdot + sizeof(double) * fdot_tab.size();
  size_t off_active = off_pos + sizeof(int) * n_d;
  size_t off_count = off_active + sizeof(int) * n_d;
  size_t total = off_count + 256;
  GLASS_CUDA(cudaMalloc(&mem, total), "cudaMalloc(fstat grid)");
  struct Free {
    char *&p;
    ~Free() { cudaFree(p); }
  } guard{mem};
  double *d_cells = (double *)mem, *d_logl0 = (double *)(mem + off_logl0), *d_tensor = (double *)(mem + off_tensor);
  double *d_fdot = (double *)(mem + off_fdot);
  int *d_pos = (int *)(mem + off_pos), *d_active = (int *)(mem + off_active), *d_count = (int *)(mem + off_count);
  GLASS_CUDA(cudaMemcpyAsync(d_fdot, fdot_tab.data(), sizeof(double) * fdot_tab.size(), cudaMemcpyHostToDevice, st),
             "H2D fdot table");
  GLASS_CUDA(fs_grid_cells(G, 0, n, d_cells, st), "fstat grid cells");
  int nl = 0, nl2 = 0;
  GLASS_CUDA(fs_launch(b, ctx->tab, b.rho, ctx->fsw, n, nullptr, seg, d_cells, d_logl0, nullptr, nullptr,
                       ctx->num_sms, st, &nl), "fstat grid launch");
  GLASS_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int), st), "fstat scan count");
  GLASS_CUDA(fs_scan_mark(d_logl0, n, d_count, d_active, d_pos, st), "fstat scan mark");
  int nact = 0;
  GLASS_CUDA(cudaMemcpyAsync(&nact, d_count, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H scan count");
  GLASS_CUDA(cudaStreamSynchronize(st), "fstat scan sync");
  double *d_scan = nullptr;
  char *smem = nullptr;
  struct Free2 {
    char *&p;
    ~Free2() { cudaFree(p); }
  } guard2{smem};
  if (nact > 0) {
    const size_t ns = (size_t)nact * kFsScan;
    GLASS_CUDA(cudaMalloc(&smem, sizeof(double) * 5 * ns), "cudaMalloc(fstat scan)");
    double *d_scells = (double *)smem;
    d_scan = d_scells + 4 * ns;
    GLASS_CUDA(fs_scan_cells(G, d_active, 0, (int)ns, d_fdot, d_scells, st), "fstat scan cells");
    GLASS_CUDA(fs_launch(b, ctx->tab, b.rho, ctx->fsw, (int)ns, nullptr, seg, d_scells, d_scan, nullptr, nullptr,
                         ctx->num_sms, st, &nl2), "fstat scan launch");
  }
  GLASS_CUDA(fs_finalize(d_logl0, d_pos, d_scan, n, d_tensor, st), "fstat finalize");
  ctx->last_launches = nl + nl2 + 4 + (nact > 0 ? 1 : 0);
  GLASS_CUDA(cudaMemcpyAsync(tensor, d_tensor, sizeof(double) * n_d, cudaMemcpyDeviceToHost, st), "D2H tensor");
  GLASS_CUDA(cudaStreamSynchronize(st), "fstat proposal sync");
  // normalisation and maximum in the reference's order (:1154-1181)
  double norm = 0.0;
  for (size_t c = 0; c < n_d; c++) norm += tensor[c];
  norm = (G.n_f * n_theta * n_phi) / norm;
  double maxp = -1.e60;
  for (size_t c = 0; c < n_d; c++) {
    tensor[c] *= norm;
    if (tensor[c] > maxp) maxp = tensor[c];
  }
  info[0] = G.n_f;
  info[1] = norm;
  info[2] = maxp;
  info[3] = nact;
  return GLASS_OK;
}

// --------------------------------------------- the UCB sampler's noise step
// noise_model_mcmc (ucb/src/glass_ucb_sampler.c:29-73) scales each channel's
// noise by eta (generate_noise_model, ucb/src/glass_ucb_model.c:336-346) and
// compares (logL + logLnorm) at eta_y with eta_x for the chain's unchanged
// residual r = d - h: logL = -sum |r|^2 / (C eta') per channel
// (gaussian_log_likelihood, utils/src/glass_model.c:726-774, with
// eta' = sqrt(eta eta) as :342 forms it) and logLnorm = -sum log(C eta')
// (:788-803).  With S_c = sum |r_c|^2 / C_c over the segment (the bank's
// residual power Q minus the chain template's per-channel term):
//   d = -S_A (1/eta'_yA - 1/eta'_xA) - S_E (1/eta'_yE - 1/eta'_xE)
//       - NFFT (log eta'_yA - log eta'_xA + log eta'_yE - log eta'_xE).
__global__ void noise_eta_kernel(int n, const int *item_seg, const double *term_ch, const double *Q, const double *QA,
                                 int NFFT, int nseg, const double *eta_x, const double *eta_y, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int seg = item_seg[i];
  if (seg < 0 || seg >= nseg) {
    out[i] = __longlong_as_double(0x7ff8000000000000ULL);
    return;
  }
  const size_t e = (size_t)seg * (NFFT + 1) + NFFT;
  const double qa = QA[e], qe = Q[e] - QA[e];
  const double SA = qa - term_ch[2 * (size_t)i], SE = qe - term_ch[2 * (size_t)i + 1];
  const double xa = sqrt(eta_x[2 * i] * eta_x[2 * i]), xe = sqrt(eta_x[2 * i + 1] * eta_x[2 * i + 1]);
  const double ya = sqrt(eta_y[2 * i] * eta_y[2 * i]), ye = sqrt(eta_y[2 * i + 1] * eta_y[2 * i + 1]);
  const double dl = -(SA / ya - SA / xa) - (SE / ye - SE / xe);
  const double dn = -(double)NFFT * ((log(ya) - log(xa)) + (log(ye) - log(xe)));
  out[i] = dl + dn;
}

extern "C" int glass_gpu_noise_eta_batch(glass_gpu_ctx *ctx, int precision, int n, const int *item_seg,
                                         const double *params, const double *eta_x, const double *eta_y,
                                         double *dlogl_noise, int *status) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "noise_eta_batch: null context");
  if (n < 0) return set_err(GLASS_ERR_ARG, "noise_eta_batch: negative chain count");
  if (n == 0) return GLASS_OK;
  if (!item_seg || !params || !eta_x || !eta_y || !dlogl_noise) return set_err(GLASS_ERR_ARG, "noise_eta_batch: null argument");
  if (!ctx->bank.nseg) return set_err(GLASS_ERR_STATE, "noise_eta_batch: no segment bank uploaded");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  // scratch: dlogl, term_y, hh, term_ch (2 per chain)
  const size_t nd = (size_t)n;
  if (ctx->eta_cap < nd) {
    GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "noise eta scratch sync");
    cudaFree(ctx->eta_scratch);
    ctx->eta_scratch = nullptr;
    ctx->eta_cap = 0;
    GLASS_CUDA(cudaMalloc(&ctx->eta_scratch, sizeof(double) * nd * 5), "cudaMalloc(noise eta scratch)");
    ctx->eta_cap = nd;
  }
  double *scratch = ctx->eta_scratch;
  rc = glass_gpu_dlogl_batch_channels(ctx, precision, n, item_seg, params, nullptr, scratch, scratch + nd,
                                      scratch + 2 * nd, status, scratch + 3 * nd);
  if (rc == GLASS_OK) {
    noise_eta_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, item_seg, scratch + 3 * nd, ctx->bank.Q,
                                                                ctx->bank.QA, ctx->bank.NFFT, ctx->bank.nseg, eta_x,
                                                                eta_y, dlogl_noise);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_err(e, "noise_eta_kernel");
    else ctx->last_launches += 1;
  }
  return rc;
}

extern "C" int glass_gpu_noise_eta_batch_host(glass_gpu_ctx *ctx, int precision, int n, const int *item_seg,
                                              const double *params, const double *eta_x, const double *eta_y,
                                              double *dlogl_noise, int *status) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "noise_eta_batch_host: null context");
  if (n < 0) return set_err(GLASS_ERR_ARG, "noise_eta_batch_host: negative chain count");
  if (n == 0) return GLASS_OK;
  if (!item_seg || !params || !eta_x || !eta_y || !dlogl_noise)
    return set_err(GLASS_ERR_ARG, "noise_eta_batch_host: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const size_t nd = (size_t)n;
  if ((rc = ensure_stage(ctx, sizeof(double) * nd * (8 + 2 + 2 + 1) + sizeof(int) * nd * 2 + 256))) return rc;
  double *d_params = (double *)ctx->d_stage, *d_ex = d_params + 8 * nd, *d_ey = d_ex + 2 * nd, *d_out = d_ey + 2 * nd;
  int *d_seg = (int *)(d_out + nd), *d_st = d_seg + nd;
  cudaStream_t s = ctx->stream;
  GLASS_CUDA(cudaMemcpyAsync(d_params, params, sizeof(double) * 8 * nd, cudaMemcpyHostToDevice, s), "H2D params");
  GLASS_CUDA(cudaMemcpyAsync(d_ex, eta_x, sizeof(double) * 2 * nd, cudaMemcpyHostToDevice, s), "H2D eta_x");
  GLASS_CUDA(cudaMemcpyAsync(d_ey, eta_y, sizeof(double) * 2 * nd, cudaMemcpyHostToDevice, s), "H2D eta_y");
  GLASS_CUDA(cudaMemcpyAsync(d_seg, item_seg, sizeof(int) * nd, cudaMemcpyHostToDevice, s), "H2D item_seg");
  rc = glass_gpu_noise_eta_batch(ctx, precision, n, d_seg, d_params, d_ex, d_ey, d_out, d_st);
  if (rc) return rc;
  GLASS_CUDA(cudaMemcpyAsync(dlogl_noise, d_out, sizeof(double) * nd, cudaMemcpyDeviceToHost, s), "D2H dlogl_noise");
  if (status) GLASS_CUDA(cudaMemcpyAsync(status, d_st, sizeof(int) * nd, cudaMemcpyDeviceToHost, s), "D2H status");
  GLASS_CUDA(cudaStreamSynchronize(s), "noise_eta_batch_host sync");
  return GLASS_OK;
}

// ------------------------------------------------------- noise likelihood
// The SGWB response rows of the context's grids (Fourier bins, wavelet layer
// centres) from its response table; freed when no template is set.
static int sgwb_build_rows(glass_gpu_ctx *ctx) {
  struct Grid {
    double **rsg;
    std::vector<double> f;
  };
  std::vector<Grid> grids;
  if (ctx->noise.tab) {
    Grid g{&ctx->noise.rsg, std::vector<double>(ctx->noise.N)};
    for (int n = 0; n < ctx->noise.N; n++) g.f[n] = ctx->noise.fmin + (double)n / ctx->noise.T;
    grids.push_back(std::move(g));
  }
  if (ctx->noise_wv.mem) {
    Grid g{&ctx->noise_wv.rsg, std::vector<double>(ctx->noise_wv.Nlayer)};
    for (int j = 0; j < ctx->noise_wv.Nlayer; j++) g.f[j] = (double)(ctx->noise_wv.lmin + j) * ctx->noise_wv.df;
    grids.push_back(std::move(g));
  }
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "sgwb rows sync");
  for (Grid &g : grids) {
    cudaFree(*g.rsg);
    *g.rsg = nullptr;
    if (ctx->sgwb_type < 0) continue;
    const int N = (int)g.f.size();
    std::vector<double> R((size_t)6 * N);
    if (noise_sgwb_rows((int)(ctx->sgwb_resp.size() / 7), ctx->sgwb_resp.data(), N, g.f.data(), R.data()))
      return set_err(GLASS_ERR_ARG, "noise_sgwb_setup: response table needs 10..3000 rows with f, XX, YY, ZZ > 0");
    GLASS_CUDA(cudaMalloc(g.rsg, sizeof(double) * R.size()), "cudaMalloc(sgwb response)");
    GLASS_CUDA(cudaMemcpy(*g.rsg, R.data(), sizeof(double) * R.size(), cudaMemcpyHostToDevice), "upload sgwb response");
  }
  return GLASS_OK;
}

extern "C" int glass_gpu_noise_sgwb_setup(glass_gpu_ctx *ctx, int type, int nresp, const double *resp) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "noise_sgwb_setup: null context");
  if (type < -1 || type >= kSgwbTypes) return set_err(GLASS_ERR_ARG, "noise_sgwb_setup: template is -1, 0, 1 or 2");
  if (type >= 0 && (!resp || nresp < 10 || nresp > 3000))
    return set_err(GLASS_ERR_ARG, "noise_sgwb_setup: response table needs 10..3000 rows");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  ctx->sgwb_type = type;
  if (type >= 0)
    ctx->sgwb_resp.assign(resp, resp + 7 * (size_t)nresp);
  else
    ctx->sgwb_resp.clear();
  rc = sgwb_build_rows(ctx);
  if (rc) ctx->sgwb_type = -1;
  return rc;
}

extern "C" int glass_gpu_noise_setup(glass_gpu_ctx *ctx, double T, int qmin, int NFFT, const double *X,
                                     const double *Y, const double *Z) {
  if (!ctx || !X || !Y || !Z) return set_err(GLASS_ERR_ARG, "noise_setup: null argument");
  if (!(T > 0) || NFFT < 1 || qmin < 1) return set_err(GLASS_ERR_ARG, "noise_setup: bad grid (T > 0, NFFT >= 1, qmin >= 1)");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const double fmin = (double)qmin / T;  // floor(fmin T)/T (utils/src/glass_data.c:2065)
  std::vector<double> tab((size_t)kNoiseTabRows * NFFT);
  noise_build_table(T, fmin, NFFT, X, Y, Z, tab.data());
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "noise_setup sync");
  NoiseDev &nd = ctx->noise;
  cudaFree(nd.tab);
  nd.tab = nullptr;
  GLASS_CUDA(cudaMalloc(&nd.tab, sizeof(double) * tab.size()), "cudaMalloc(noise table)");
  GLASS_CUDA(cudaMemcpy(nd.tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice), "upload noise table");
  nd.nch = 3;
  nd.N = NFFT;
  nd.T = T;
  nd.fmin = fmin;
  cudaFree(nd.partial);
  nd.partial = nullptr;
  nd.partial_models = 0;
  return sgwb_build_rows(ctx);
}

extern "C" int glass_gpu_noise_setup_channels(glass_gpu_ctx *ctx, int nchannel, double T, int qmin, int NFFT,
                                              const double *d0, const double *d1, const double *d2) {
  if (nchannel == 3) return glass_gpu_noise_setup(ctx, T, qmin, NFFT, d0, d1, d2);
  if (!ctx) return set_err(GLASS_ERR_ARG, "noise_setup_channels: null context");
  if (nchannel != 1 && nchannel != 2) return set_err(GLASS_ERR_ARG, "noise_setup_channels: one, two or three channels");
  if (!d0 || (nchannel == 2 && !d1)) return set_err(GLASS_ERR_ARG, "noise_setup_channels: null argument");
  // qmin >= 1: at f = 0 the reference's one- and two-channel branch writes
  // covariance entries of three channels
  if (!(T > 0) || NFFT < 1 || qmin < 1)
    return set_err(GLASS_ERR_ARG, "noise_setup_channels: bad grid (T > 0, NFFT >= 1, qmin >= 1)");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const double fmin = (double)qmin / T;
  std::vector<double> tab((size_t)kNoiseTabRows * NFFT);
  noise_build_table_ch(T, fmin, NFFT, nchannel, d0, d1, tab.data());
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "noise_setup_channels sync");
  NoiseDev &nd = ctx->noise;
  cudaFree(nd.tab);
  nd.tab = nullptr;
  GLASS_CUDA(cudaMalloc(&nd.tab, sizeof(double) * tab.size()), "cudaMalloc(noise table)");
  GLASS_CUDA(cudaMemcpy(nd.tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice), "upload noise table");
  nd.nch = nchannel;
  nd.N = NFFT;
  nd.T = T;
  nd.fmin = fmin;
  cudaFree(nd.partial);
  nd.partial = nullptr;
  nd.partial_models = 0;
  return sgwb_build_rows(ctx);
}

extern "C" int glass_gpu_noise_logl_batch_sgwb(glass_gpu_ctx *ctx, int nprop, const double *inst, const double *sgal,
                                               const double *sgwb, double *logl) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "noise_logl_batch: null context");
  if (nprop < 0) return set_err(GLASS_ERR_ARG, "noise_logl_batch: negative model count");
  if (nprop == 0) return GLASS_OK;
  if (!inst || !logl) return set_err(GLASS_ERR_ARG, "noise_logl_batch: null argument");
  NoiseDev &nd = ctx->noise;
  if (!nd.tab) return set_err(GLASS_ERR_STATE, "noise_logl_batch: no data set (glass_gpu_noise_setup)");
  if (sgwb && nd.nch != 3)  // generate_sgwb_model stops for Nchannel 1 or 2
    return set_err(GLASS_ERR_ARG, "noise_logl_batch: the SGWB covariance needs three channels");
  if (sgwb && (ctx->sgwb_type < 0 || !nd.rsg))
    return set_err(GLASS_ERR_STATE, "noise_logl_batch: no SGWB template set (glass_gpu_noise_sgwb_setup)");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  if (nprop > nd.partial_models) {
    int want = nd.partial_models > 0 ? nd.partial_models : 64;
    while (want < nprop) want *= 2;
    GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "noise partial sync");
    cudaFree(nd.partial);
    nd.partial = nullptr;
    nd.partial_models = 0;
    GLASS_CUDA(cudaMalloc(&nd.partial, sizeof(double) * (size_t)want * noise_chunks(nd.N)), "cudaMalloc(noise partial)");
    nd.partial_models = want;
  }
  int nl = 0;
  cudaError_t e = noise_logl_launch(nd, nprop, inst, sgal, ctx->sgwb_type, sgwb, logl, ctx->stream, &nl);
  ctx->last_launches = nl;
  if (e != cudaSuccess) return cuda_err(e, "noise_logl_batch launch");
  return GLASS_OK;
}

extern "C" int glass_gpu_noise_logl_batch(glass_gpu_ctx *ctx, int nprop, const double *inst, const double *sgal,
                                          double *logl) {
  return glass_gpu_noise_logl_batch_sgwb(ctx, nprop, inst, sgal, nullptr, logl);
}

extern "C" int glass_gpu_noise_logl_batch_sgwb_host(glass_gpu_ctx *ctx, int nprop, const double *inst,
                                                    const double *sgal, const double *sgwb, double *logl) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "noise_logl_batch_host: null context");
  if (nprop < 0) return set_err(GLASS_ERR_ARG, "noise_logl_batch_host: negative model count");
  if (nprop == 0) return GLASS_OK;
  if (!inst || !logl) return set_err(GLASS_ERR_ARG, "noise_logl_batch_host: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const size_t nd = (size_t)nprop;
  if ((rc = ensure_stage(ctx, sizeof(double) * nd * (12 + 5 + 4 + 1) + 256))) return rc;
  double *d_inst = (double *)ctx->d_stage, *d_sgal = d_inst + 12 * nd, *d_sgwb = d_sgal + 5 * nd,
         *d_logl = d_sgwb + 4 * nd;
  cudaStream_t s = ctx->stream;
  GLASS_CUDA(cudaMemcpyAsync(d_inst, inst, sizeof(double) * 12 * nd, cudaMemcpyHostToDevice, s), "H2D inst");
  if (sgal) GLASS_CUDA(cudaMemcpyAsync(d_sgal, sgal, sizeof(double) * 5 * nd, cudaMemcpyHostToDevice, s), "H2D sgal");
  if (sgwb) GLASS_CUDA(cudaMemcpyAsync(d_sgwb, sgwb, sizeof(double) * 4 * nd, cudaMemcpyHostToDevice, s), "H2D sgwb");
  rc = glass_gpu_noise_logl_batch_sgwb(ctx, nprop, d_inst, sgal ? d_sgal : nullptr, sgwb ? d_sgwb : nullptr, d_logl);
  if (rc) return rc;
  GLASS_CUDA(cudaMemcpyAsync(logl, d_logl, sizeof(double) * nd, cudaMemcpyDeviceToHost, s), "D2H logl");
  GLASS_CUDA(cudaStreamSynchronize(s), "noise_logl_batch_host sync");
  return GLASS_OK;
}

extern "C" int glass_gpu_noise_logl_batch_host(glass_gpu_ctx *ctx, int nprop, const double *inst, const double *sgal,
                                               double *logl) {
  return glass_gpu_noise_logl_batch_sgwb_host(ctx, nprop, inst, sgal, nullptr, logl);
}

// ------------------------------------------------------ spline noise model
extern "C" int glass_gpu_spline_noise_setup(glass_gpu_ctx *ctx, int nchannel, double T, int qmin, int NFFT,
                                            const double *transfer, const double *d0, const double *d1) {
  if (!ctx || !transfer || !d0 || (nchannel == 2 && !d1))
    return set_err(GLASS_ERR_ARG, "spline_noise_setup: null argument");
  if (nchannel < 1 || nchannel > 2) return set_err(GLASS_ERR_ARG, "spline_noise_setup: one or two channels");
  if (!(T > 0) || NFFT < 1 || qmin < 0) return set_err(GLASS_ERR_ARG, "spline_noise_setup: bad grid");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const size_t N = (size_t)NFFT;
  std::vector<double> tab((2 + nchannel) * N);
  const double fmin = (double)qmin / T;
  for (size_t n = 0; n < N; n++) {
    tab[n] = fmin + (double)n / T;  // the model's grid (noise/src/glass_noise_model.c:1349)
    tab[N + n] = transfer[n];
    for (int c = 0; c < nchannel; c++) {
      const double *d = c == 0 ? d0 : d1;
      tab[(2 + c) * N + n] = d[2 * n] * d[2 * n] + d[2 * n + 1] * d[2 * n + 1];
    }
  }
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "spline_noise_setup sync");
  SplineNoiseDev &sd = ctx->spline_noise;
  cudaFree(sd.tab);
  sd.tab = nullptr;
  GLASS_CUDA(cudaMalloc(&sd.tab, sizeof(double) * tab.size()), "cudaMalloc(spline noise table)");
  GLASS_CUDA(cudaMemcpy(sd.tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice),
             "upload spline noise table");
  sd.nch = nchannel;
  sd.N = NFFT;
  return GLASS_OK;
}

extern "C" int glass_gpu_spline_noise_logl_batch(glass_gpu_ctx *ctx, int nprop, int kmax, const int *nknots,
                                                 const double *knot_f, const double *knot_C, double *logl) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "spline_noise_logl_batch: null context");
  if (nprop < 0) return set_err(GLASS_ERR_ARG, "spline_noise_logl_batch: negative model count");
  if (nprop == 0) return GLASS_OK;
  if (!nknots || !knot_f || !knot_C || !logl) return set_err(GLASS_ERR_ARG, "spline_noise_logl_batch: null argument");
  if (kmax < 2 || kmax > kSplineMaxKnots)
    return set_err(GLASS_ERR_ARG, "spline_noise_logl_batch: kmax must be 2 .. %s", std::to_string(kSplineMaxKnots).c_str());
  if (!ctx->spline_noise.tab) return set_err(GLASS_ERR_STATE, "spline_noise_logl_batch: no data (glass_gpu_spline_noise_setup)");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  int nl = 0;
  cudaError_t e = spline_noise_launch(ctx->spline_noise, nprop, kmax, nknots, knot_f, knot_C, logl, ctx->stream, &nl);
  ctx->last_launches = nl;
  if (e != cudaSuccess) return cuda_err(e, "spline_noise_logl_batch launch");
  return GLASS_OK;
}

extern "C" int glass_gpu_spline_noise_logl_batch_host(glass_gpu_ctx *ctx, int nprop, int kmax, const int *nknots,
                                                      const double *knot_f, const double *knot_C, double *logl) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "spline_noise_logl_batch_host: null context");
  if (nprop < 0) return set_err(GLASS_ERR_ARG, "spline_noise_logl_batch_host: negative model count");
  if (nprop == 0) return GLASS_OK;
  if (!nknots || !knot_f || !knot_C || !logl)
    return set_err(GLASS_ERR_ARG, "spline_noise_logl_batch_host: null argument");
  if (kmax < 2 || kmax > kSplineMaxKnots)
    return set_err(GLASS_ERR_ARG, "spline_noise_logl_batch_host: kmax must be 2 .. %s",
                   std::to_string(kSplineMaxKnots).c_str());
  if (!ctx->spline_noise.tab)
    return set_err(GLASS_ERR_STATE, "spline_noise_logl_batch_host: no data (glass_gpu_spline_noise_setup)");
  const int nch = ctx->spline_noise.nch;
  for (int p = 0; p < nprop; p++) {  // knot counts in range, frequencies increasing
    if (nknots[p] < 2 || nknots[p] > kmax)
      return set_err(GLASS_ERR_ARG, "spline_noise_logl_batch_host: model %s has a knot count outside 2 .. kmax",
                     std::to_string(p).c_str());
    for (int k = 1; k < nknots[p]; k++)
      if (!(knot_f[(size_t)p * kmax + k] > knot_f[(size_t)p * kmax + k - 1]))
        return set_err(GLASS_ERR_ARG, "spline_noise_logl_batch_host: model %s's knot frequencies do not increase",
                       std::to_string(p).c_str());
  }
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const size_t nd = (size_t)nprop, km = (size_t)kmax;
  const size_t bytes = sizeof(double) * nd * (km * (1 + nch) + 1) + sizeof(int) * nd;
  if ((rc = ensure_stage(ctx, bytes))) return rc;
  double *d_f = (double *)ctx->d_stage, *d_C = d_f + nd * km, *d_l = d_C + nd * km * nch;
  int *d_n = (int *)(d_l + nd);
  cudaStream_t s = ctx->stream;
  GLASS_CUDA(cudaMemcpyAsync(d_f, knot_f, sizeof(double) * nd * km, cudaMemcpyHostToDevice, s), "H2D knot_f");
  GLASS_CUDA(cudaMemcpyAsync(d_C, knot_C, sizeof(double) * nd * km * nch, cudaMemcpyHostToDevice, s), "H2D knot_C");
  GLASS_CUDA(cudaMemcpyAsync(d_n, nknots, sizeof(int) * nd, cudaMemcpyHostToDevice, s), "H2D nknots");
  rc = glass_gpu_spline_noise_logl_batch(ctx, nprop, kmax, d_n, d_f, d_C, d_l);
  if (rc) return rc;
  GLASS_CUDA(cudaMemcpyAsync(logl, d_l, sizeof(double) * nd, cudaMemcpyDeviceToHost, s), "D2H logl");
  GLASS_CUDA(cudaStreamSynchronize(s), "spline_noise_logl_batch_host sync");
  return GLASS_OK;
}

extern "C" int glass_gpu_noise_wavelet_setup(glass_gpu_ctx *ctx, int NF, int NT, double df, int lmin, int Nlayer,
                                             int Q, const double *X, const double *Y, const double *Z,
                                             const double *mod) {
  if (!ctx || !X || !Y || !Z) return set_err(GLASS_ERR_ARG, "noise_wavelet_setup: null argument");
  if (NF < 1 || NT < 1 || Nlayer < 1 || lmin < 0 || !(df > 0) || Q < 1 || Q > NT)
    return set_err(GLASS_ERR_ARG, "noise_wavelet_setup: bad grid (NF, NT, Nlayer >= 1, lmin >= 0, df > 0, 1 <= Q <= NT)");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const int Nc = NT / Q;
  const size_t Npix = (size_t)Nlayer * Nc;
  std::vector<double> tab((size_t)kNoiseTabRows * Nlayer), P(6 * Npix);
  noise_wv_build(NT, df, lmin, Nlayer, Q, X, Y, Z, tab.data(), P.data());
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "noise_wavelet_setup sync");
  NoiseWvDev &w = ctx->noise_wv;
  cudaFree(w.mem);
  cudaFree(w.partial);
  cudaFree(w.rsg);
  w = NoiseWvDev{};
  const size_t bytes = sizeof(double) * (tab.size() + P.size() + 6 * (size_t)Nc);
  GLASS_CUDA(cudaMalloc(&w.mem, bytes), "cudaMalloc(noise wavelet)");
  w.tab = (double *)w.mem;
  w.P = w.tab + tab.size();
  w.mod = w.P + P.size();
  GLASS_CUDA(cudaMemcpy(w.tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice), "upload noise wv table");
  GLASS_CUDA(cudaMemcpy(w.P, P.data(), sizeof(double) * P.size(), cudaMemcpyHostToDevice), "upload noise wv stats");
  if (mod)
    GLASS_CUDA(cudaMemcpy(w.mod, mod, sizeof(double) * 6 * Nc, cudaMemcpyHostToDevice), "upload modulation");
  w.NF = NF;
  w.NT = NT;
  w.lmin = lmin;
  w.Nlayer = Nlayer;
  w.Q = Q;
  w.Ncoarse = Nc;
  w.df = df;
  w.has_mod = mod != nullptr;
  return sgwb_build_rows(ctx);
}

extern "C" int glass_gpu_noise_wavelet_logl_batch_sgwb(glass_gpu_ctx *ctx, int mode, int nprop, const double *inst,
                                                       const double *sgal, const double *sgwb, double *logl) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "noise_wavelet_logl_batch: null context");
  if (nprop < 0) return set_err(GLASS_ERR_ARG, "noise_wavelet_logl_batch: negative model count");
  if (mode < 0 || mode > 2) return set_err(GLASS_ERR_ARG, "noise_wavelet_logl_batch: mode is 0, 1 or 2");
  if (nprop == 0) return GLASS_OK;
  if (!inst || !logl || (mode && !sgal)) return set_err(GLASS_ERR_ARG, "noise_wavelet_logl_batch: null argument");
  NoiseWvDev &w = ctx->noise_wv;
  if (!w.mem) return set_err(GLASS_ERR_STATE, "noise_wavelet_logl_batch: no data set (glass_gpu_noise_wavelet_setup)");
  if (mode == 2 && !w.has_mod) return set_err(GLASS_ERR_STATE, "noise_wavelet_logl_batch: mode 2 needs the modulation");
  if (sgwb && (ctx->sgwb_type < 0 || !w.rsg))
    return set_err(GLASS_ERR_STATE, "noise_wavelet_logl_batch: no SGWB template set (glass_gpu_noise_sgwb_setup)");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  if (mode == 2 && nprop > w.partial_models) {
    int want = w.partial_models > 0 ? w.partial_models : 64;
    while (want < nprop) want *= 2;
    GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "noise wv partial sync");
    cudaFree(w.partial);
    w.partial = nullptr;
    w.partial_models = 0;
    GLASS_CUDA(cudaMalloc(&w.partial, sizeof(double) * (size_t)want * noise_wv_chunks(w)), "cudaMalloc(noise wv partial)");
    w.partial_models = want;
  }
  int nl = 0;
  cudaError_t e = noise_wv_logl_launch(w, mode, nprop, inst, sgal, ctx->sgwb_type, sgwb, logl, ctx->stream, &nl);
  ctx->last_launches = nl;
  if (e != cudaSuccess) return cuda_err(e, "noise_wavelet_logl_batch launch");
  return GLASS_OK;
}

extern "C" int glass_gpu_noise_wavelet_logl_batch(glass_gpu_ctx *ctx, int mode, int nprop, const double *inst,
                                                  const double *sgal, double *logl) {
  return glass_gpu_noise_wavelet_logl_batch_sgwb(ctx, mode, nprop, inst, sgal, nullptr, logl);
}

extern "C" int glass_gpu_noise_wavelet_logl_batch_sgwb_host(glass_gpu_ctx *ctx, int mode, int nprop,
                                                            const double *inst, const double *sgal,
                                                            const double *sgwb, double *logl) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "noise_wavelet_logl_batch_host: null context");
  if (nprop < 0) return set_err(GLASS_ERR_ARG, "noise_wavelet_logl_batch_host: negative model count");
  if (nprop == 0) return GLASS_OK;
  if (!inst || !logl) return set_err(GLASS_ERR_ARG, "noise_wavelet_logl_batch_host: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const size_t nd = (size_t)nprop;
  if ((rc = ensure_stage(ctx, sizeof(double) * nd * (12 + 5 + 4 + 1) + 256))) return rc;
  double *d_inst = (double *)ctx->d_stage, *d_sgal = d_inst + 12 * nd, *d_sgwb = d_sgal + 5 * nd,
         *d_logl = d_sgwb + 4 * nd;
  cudaStream_t s = ctx->stream;
  GLASS_CUDA(cudaMemcpyAsync(d_inst, inst, sizeof(double) * 12 * nd, cudaMemcpyHostToDevice, s), "H2D inst");
  if (sgal) GLASS_CUDA(cudaMemcpyAsync(d_sgal, sgal, sizeof(double) * 5 * nd, cudaMemcpyHostToDevice, s), "H2D sgal");
  if (sgwb) GLASS_CUDA(cudaMemcpyAsync(d_sgwb, sgwb, sizeof(double) * 4 * nd, cudaMemcpyHostToDevice, s), "H2D sgwb");
  rc = glass_gpu_noise_wavelet_logl_batch_sgwb(ctx, mode, nprop, d_inst, sgal ? d_sgal : nullptr,
                                               sgwb ? d_sgwb : nullptr, d_logl);
  if (rc) return rc;
  GLASS_CUDA(cudaMemcpyAsync(logl, d_logl, sizeof(double) * nd, cudaMemcpyDeviceToHost, s), "D2H logl");
  GLASS_CUDA(cudaStreamSynchronize(s), "noise_wavelet_logl_batch_host sync");
  return GLASS_OK;
}

extern "C" int glass_gpu_noise_wavelet_logl_batch_host(glass_gpu_ctx *ctx, int mode, int nprop, const double *inst,
                                                       const double *sgal, double *logl) {
  return glass_gpu_noise_wavelet_logl_batch_sgwb_host(ctx, mode, nprop, inst, sgal, nullptr, logl);
}

// ------------------------------------------------------ on-device sampler
extern "C" int glass_gpu_rand_r_fill(glass_gpu_ctx *ctx, int n, int count, unsigned int *seed, int *out) {
  if (!ctx || !seed || !out || n < 0 || count < 0) return set_err(GLASS_ERR_ARG, "rand_r_fill: bad argument");
  if (n == 0 || count == 0) return GLASS_OK;
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  GLASS_CUDA(rand_r_fill_launch(n, count, seed, out, ctx->stream), "rand_r_fill");
  return GLASS_OK;
}

extern "C" int glass_gpu_mh_accept(glass_gpu_ctx *ctx, int n, const double *temperature, const double *dlogl,
                                   const double *logPx, const double *logPy, const double *logQxy,
                                   const double *logQyx, const double *snr, unsigned int *seed, double *logL_x,
                                   double *params_x, const double *params_y, int *accepted) {
  if (!ctx || n < 0) return set_err(GLASS_ERR_ARG, "mh_accept: bad argument");
  if (n == 0) return GLASS_OK;
  if (!temperature || !dlogl || !logPx || !logPy || !logQxy || !logQyx || !seed || !logL_x || !params_x || !params_y)
    return set_err(GLASS_ERR_ARG, "mh_accept: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  MhArgs a{n, temperature, dlogl, logPx, logPy, logQxy, logQyx, snr, logL_x, params_x, params_y, seed, accepted};
  GLASS_CUDA(mh_accept_launch(a, ctx->stream), "mh_accept");
  ctx->last_launches = 1;
  return GLASS_OK;
}

extern "C" int glass_gpu_ptmcmc(glass_gpu_ctx *ctx, int nens, int NC, const double *temperature, const double *logL,
                                const double *logLnorm, int *index, unsigned int *seed, double *acceptance) {
  if (!ctx || nens < 0 || NC < 1) return set_err(GLASS_ERR_ARG, "ptmcmc: bad argument");
  if (nens == 0) return GLASS_OK;
  if (!temperature || !logL || !index || !seed || !acceptance) return set_err(GLASS_ERR_ARG, "ptmcmc: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  PtArgs a{nens, NC, temperature, logL, logLnorm, index, seed, acceptance};
  GLASS_CUDA(ptmcmc_launch(a, ctx->stream), "ptmcmc");
  ctx->last_launches = 1;
  return GLASS_OK;
}

extern "C" int glass_gpu_fisher_draw(glass_gpu_ctx *ctx, int n, const double *params_x, const double *evec,
                                     const double *evalue, unsigned int *seed, double *params_y, double *logQ,
                                     int *status) {
  if (!ctx || n < 0) return set_err(GLASS_ERR_ARG, "fisher_draw: bad argument");
  if (n == 0) return GLASS_OK;
  if (!params_x || !evec || !evalue || !seed || !params_y) return set_err(GLASS_ERR_ARG, "fisher_draw: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  FisherDrawArgs a{n, params_x, evec, evalue, seed, params_y, logQ, status};
  GLASS_CUDA(fisher_draw_launch(a, ctx->stream), "fisher_draw");
  ctx->last_launches = 1;
  return GLASS_OK;
}

extern "C" int glass_gpu_sym_eigen8(glass_gpu_ctx *ctx, int n, const double *matrix, double *evec, double *evalue) {
  if (!ctx || n < 0) return set_err(GLASS_ERR_ARG, "sym_eigen8: bad argument");
  if (n == 0) return GLASS_OK;
  if (!matrix || !evec || !evalue) return set_err(GLASS_ERR_ARG, "sym_eigen8: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  GLASS_CUDA(sym_eigen8_launch(n, matrix, evec, evalue, ctx->stream), "sym_eigen8");
  ctx->last_launches = 1;
  return GLASS_OK;
}

static int prior_args(const char *who, glass_gpu_ctx *ctx, int n, const double *prior, int prior_stride,
                      const double *logPV, double *params, double *out, PriorArgs &a) {
  if (!ctx || n < 0 || (prior_stride != 0 && prior_stride != 1)) return set_err(GLASS_ERR_ARG, "%s: bad argument", who);
  if (n > 0 && (!prior || !logPV || !params || !out)) return set_err(GLASS_ERR_ARG, "%s: null argument", who);
  a = PriorArgs{};
  a.n = n;
  a.prior = prior;
  a.logPV = logPV;
  a.stride = prior_stride;
  a.params = params;
  a.out = out;
  return ctx_activate(ctx);
}

extern "C" int glass_gpu_prior_draw(glass_gpu_ctx *ctx, int n, const double *prior, int prior_stride,
                                    const double *logPV, unsigned int *seed, double *params, double *logQ) {
  PriorArgs a;
  int rc = prior_args("prior_draw", ctx, n, prior, prior_stride, logPV, params, logQ, a);
  if (rc || n == 0) return rc;
  if (!seed) return set_err(GLASS_ERR_ARG, "prior_draw: null seed");
  a.seed = seed;
  GLASS_CUDA(prior_draw_launch(a, ctx->stream), "prior_draw");
  ctx->last_launches = 1;
  return GLASS_OK;
}

extern "C" int glass_gpu_ucb_prior(glass_gpu_ctx *ctx, int n, double *params, const double *prior, int prior_stride,
                                   const double *logPV, const double *skyhist, double dcostheta, double dphi, int nphi,
                                   double *logP) {
  PriorArgs a;
  int rc = prior_args("ucb_prior", ctx, n, prior, prior_stride, logPV, params, logP, a);
  if (rc || n == 0) return rc;
  if (skyhist && !(dcostheta > 0 && dphi > 0 && nphi > 0)) return set_err(GLASS_ERR_ARG, "ucb_prior: bad sky grid");
  a.skyhist = skyhist;
  a.dcostheta = dcostheta;
  a.dphi = dphi;
  a.nphi = nphi;
  GLASS_CUDA(ucb_prior_launch(a, ctx->stream), "ucb_prior");
  ctx->last_launches = 1;
  return GLASS_OK;
}

// ------------------------------------------- trans-dimensional (RJ) step
extern "C" int glass_gpu_rj_propose(glass_gpu_ctx *ctx, int n, int maxsrc, const int *Nlive, const int *Neff,
                                    const double *src, const double *prior, int prior_stride, const double *logPV,
                                    const double *rjweight, const glass_gpu_fstat_grid *grid, unsigned int *seed,
                                    int *move, int *slot, int *kind, double *params_y, double *logQxy, double *logQyx,
                                    double *logPy, int *status) {
  if (!ctx || n < 0 || maxsrc < 1 || (prior_stride != 0 && prior_stride != 1))
    return set_err(GLASS_ERR_ARG, "rj_propose: bad argument");
  if (n == 0) return GLASS_OK;
  if (!Nlive || !Neff || !src || !prior || !logPV || !rjweight || !seed || !move || !slot || !kind || !params_y ||
      !logQxy || !logQyx || !logPy)
    return set_err(GLASS_ERR_ARG, "rj_propose: null argument");
  RjArgs a{};
  double wsum = 0.0;
  for (int k = 0; k < 9; k++) {
    if (!(rjweight[k] >= 0.0 && rjweight[k] <= 1.0)) return set_err(GLASS_ERR_ARG, "rj_propose: rj weights are 0 .. 1");
    if (k >= 2 && rjweight[k] > 0.0)
      return set_err(GLASS_ERR_ARG, "rj_propose: only the prior (0) and F-statistic (1) draws run on the device");
    a.rjw[k] = rjweight[k];
    wsum += rjweight[k];
  }
  if (!(wsum > 0.0)) return set_err(GLASS_ERR_ARG, "rj_propose: every rj weight is 0");
  if (rjweight[1] > 0.0) {
    if (!grid || !grid->tensor || grid->n_f < 1 || grid->n_theta < 1 || grid->n_phi < 1 || !(grid->maxp > 0) ||
        !(grid->d_f > 0) || !(grid->d_theta > 0) || !(grid->d_phi > 0) || !(grid->T > 0))
      return set_err(GLASS_ERR_ARG, "rj_propose: the F-statistic draw needs its grid");
    a.tensor = grid->tensor;
    a.n_f = grid->n_f;
    a.n_theta = grid->n_theta;
    a.n_phi = grid->n_phi;
    a.qmin = grid->qmin;
    a.d_f = grid->d_f;
    a.d_theta = grid->d_theta;
    a.d_phi = grid->d_phi;
    a.maxp = grid->maxp;
    a.T = grid->T;
  }
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  a.n = n;
  a.maxsrc = maxsrc;
  a.Nlive = const_cast<int *>(Nlive);
  a.Neff = Neff;
  a.src = const_cast<double *>(src);
  a.prior = prior;
  a.logPV = logPV;
  a.stride = prior_stride;
  a.seed = seed;
  a.move = move;
  a.slot = slot;
  a.kind = kind;
  a.status = status;
  a.params_y = params_y;
  a.logQxy = logQxy;
  a.logQyx = logQyx;
  a.logPy = logPy;
  GLASS_CUDA(rj_propose_launch(a, ctx->stream), "rj_propose");
  ctx->last_launches = 1;
  return GLASS_OK;
}

extern "C" int glass_gpu_rj_accept(glass_gpu_ctx *ctx, int n, int maxsrc, int *Nlive, double *src, const int *move,
                                   const int *slot, double *params_y, const double *logQxy, const double *logQyx,
                                   const double *logPy, const double *temperature, const double *dlogl,
                                   const double *hh, int dlogl_is_term, int prior_only, const double *prior,
                                   int prior_stride, const double *logPV, const double *skyhist, double dcostheta,
                                   double dphi, int nphi, unsigned int *seed, double *logL_x, int *accepted) {
  if (!ctx || n < 0 || maxsrc < 1 || (prior_stride != 0 && prior_stride != 1))
    return set_err(GLASS_ERR_ARG, "rj_accept: bad argument");
  if (n == 0) return GLASS_OK;
  if (!Nlive || !src || !move || !slot || !params_y || !logQxy || !logQyx || !logPy || !temperature || !dlogl ||
      !prior || !logPV || !seed || !logL_x)
    return set_err(GLASS_ERR_ARG, "rj_accept: null argument");
  if (dlogl_is_term && !hh) return set_err(GLASS_ERR_ARG, "rj_accept: a death's change from its term needs hh");
  if (skyhist && !(dcostheta > 0 && dphi > 0 && nphi > 0)) return set_err(GLASS_ERR_ARG, "rj_accept: bad sky grid");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  RjArgs a{};
  a.n = n;
  a.maxsrc = maxsrc;
  a.Nlive = Nlive;
  a.src = src;
  a.move = const_cast<int *>(move);
  a.slot = const_cast<int *>(slot);
  a.params_y = params_y;
  a.logQxy = const_cast<double *>(logQxy);
  a.logQyx = const_cast<double *>(logQyx);
  a.logPy = const_cast<double *>(logPy);
  a.T_chain = temperature;
  a.dlogl = dlogl;
  a.hh = hh;
  a.dlogl_is_term = dlogl_is_term ? 1 : 0;
  a.prior_only = prior_only ? 1 : 0;
  a.prior = prior;
  a.logPV = logPV;
  a.stride = prior_stride;
  a.skyhist = skyhist;
  a.dcostheta = dcostheta;
  a.dphi = dphi;
  a.nphi = nphi;
  a.seed = seed;
  a.logL_x = logL_x;
  a.accepted = accepted;
  GLASS_CUDA(rj_accept_launch(a, ctx->stream), "rj_accept");
  ctx->last_launches = 1;
  return GLASS_OK;
}

// ------------------------------------------------------- drop-in functions
// Layout of struct Orbit (utils/src/glass_lisa.h:60-109), restated so the
// drop-in ucb_waveform can read the arm length, transfer frequency and the
// orbit function the caller initialised.
struct OrbitLayout {
  char OrbitFileName[1024];
  int Norb;
  double L, fstar, ecc, R, lambda_0, kappa_0;
  double *t;
  double **x, **y, **z;
  void **dx, **dy, **dz;
  void (*orbit_function)(struct Orbit *, double, double *, double *, double *);
};

// Analytic orbits (utils/src/glass_lisa.c:77-124) evaluated on the host for the
// status-returning entry point when the caller passes no positions.
static void analytic_positions(double t, double *xyz9) {
  const double sbs[3] = {0.0, 0.866025403784439, -0.866025403784438};
  const double cbs[3] = {1.0, -0.5, -0.5};
  double alpha = kPI2 * t / kYEAR;
  double sa = sin(alpha), ca = cos(alpha);
  double R = kAU * (kLARM / (2.0 * kSQ3 * kAU));
  double sa2 = sa * sa, ca2 = ca * ca, saca = sa * ca;
  for (int i = 0; i < 3; i++) {
    xyz9[3 * i + 0] = kAU * ca + R * (saca * sbs[i] - (1. + sa2) * cbs[i]);
    xyz9[3 * i + 1] = kAU * sa + R * (saca * cbs[i] - (1. + ca2) * sbs[i]);
    xyz9[3 * i + 2] = -kSQ3 * R * (ca * cbs[i] + sa * sbs[i]);
  }
}

// Per-thread resources of the drop-in entry points: the reference calls them
// from one OpenMP thread per chain, so each thread gets its own stream and
// staging buffers.
struct LegacyThread {
  bool init = false;
  int device = 0;
  cudaStream_t stream = nullptr;
  FdTablesDev tab;  // twiddles only
  // staging: [ItemF64][OrbitSample64 x kMaxN] in, 10 kMaxN doubles out
  unsigned char *h_in = nullptr, *d_in = nullptr;
  double *h_out = nullptr, *d_out = nullptr;
  double2 *d_d6 = nullptr;
  // one CUDA graph per (size, format, channel count): copy in, three kernels, copy out
  std::map<std::pair<int, double>, cudaGraphExec_t> graphs;
  ItemF64 *h_item() { return reinterpret_cast<ItemF64 *>(h_in); }
  OrbitSample64 *h_pos() { return reinterpret_cast<OrbitSample64 *>(h_in + kPosOffset); }
  static constexpr size_t kPosOffset = (sizeof(ItemF64) + 255) / 256 * 256;
  ~LegacyThread() {
    if (!init) return;
    cudaSetDevice(device);
    cudaStreamSynchronize(stream);
    for (auto &g : graphs) cudaGraphExecDestroy(g.second);
    cudaFreeHost(h_in);
    cudaFreeHost(h_out);
    cudaFree(d_in);
    cudaFree(d_out);
    cudaFree(d_d6);
    cudaFree(tab.base);
    cudaStreamDestroy(stream);
  }
};
static thread_local LegacyThread g_legacy;

static int legacy_init() {
  LegacyThread &L = g_legacy;
  if (L.init) {
    GLASS_CUDA(cudaSetDevice(L.device), "cudaSetDevice");
    return GLASS_OK;
  }
  const char *dev = getenv("GLASS_GPU_DEVICE");
  L.device = dev ? atoi(dev) : 0;
  GLASS_CUDA(cudaSetDevice(L.device), "cudaSetDevice");
  GLASS_CUDA(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking), "cudaStreamCreate");
  GLASS_CUDA(fd_build_orbit_tables(L.tab, 31457280.0, 0.0, L.stream), "twiddle tables");
  const size_t in_bytes = LegacyThread::kPosOffset + sizeof(OrbitSample64) * kMaxN;
  GLASS_CUDA(cudaMallocHost(&L.h_in, in_bytes), "cudaMallocHost");
  GLASS_CUDA(cudaMallocHost(&L.h_out, sizeof(double) * 10 * kMaxN), "cudaMallocHost");
  GLASS_CUDA(cudaMalloc(&L.d_in, in_bytes), "cudaMalloc");
  GLASS_CUDA(cudaMalloc(&L.d_out, sizeof(double) * 10 * kMaxN), "cudaMalloc");
  GLASS_CUDA(cudaMalloc(&L.d_d6, sizeof(double2) * 6 * kMaxN), "cudaMalloc");
  GLASS_CUDA(cudaStreamSynchronize(L.stream), "init sync");
  L.init = true;
  return GLASS_OK;
}

static int bin_index(int N) {
  int b = 0;
  while ((32 << b) < N) b++;
  return b;
}

// Enqueue one drop-in waveform: inputs staged in h_in, outputs to h_out.
static cudaError_t legacy_enqueue(LegacyThread &L, int fmt, double T, int BW, int NI, size_t nout) {
  cudaStream_t s = L.stream;
  const size_t in_bytes = LegacyThread::kPosOffset + sizeof(OrbitSample64) * BW;
  cudaError_t e = cudaMemcpyAsync(L.d_in, L.h_in, in_bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  e = fd_waveform_launch(reinterpret_cast<const OrbitSample64 *>(L.d_in + LegacyThread::kPosOffset),
                         reinterpret_cast<const ItemF64 *>(L.d_in), BW, fmt, NI, T, fstar_of_orbit(), L.d_d6, L.d_out,
                         L.tab.tw64[bin_index(BW)], s);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(L.h_out, L.d_out, sizeof(double) * nout, cudaMemcpyDeviceToHost, s);
}

// Shared body of the two waveform entry points; positions already in g_legacy.h_pos().
// The first call for a (size, format, channels) runs directly and records a
// CUDA graph of the sequence; later calls replay it (one launch instead of six
// API calls).  T is a kernel argument, so it is part of the key.
static int legacy_waveform_run(int fmt, double T, const double *params, int NParams, double *X, double *Y, double *Z,
                               double *A, double *E, int BW, int NI) {
  LegacyThread &L = g_legacy;
  double p[8];
  for (int k = 0; k < 8; k++) p[k] = k < NParams ? params[k] : 0.0;
  // the source's constants on the host: the same FP64 code the batched
  // plan kernels run, with the reference's operation order
  SourceGeom geo;
  source_geometry(p, NParams, T, geo);
  make_item_f64(geo, BW, *L.h_item());
  bool all = (fmt == GLASS_FMT_SANGRIA) || NI > 1;
  size_t nout = all ? 10 * (size_t)BW : 2 * (size_t)BW;
  cudaStream_t s = L.stream;
  const std::pair<int, double> key((bin_index(BW) * 4 + fmt) * 2 + (all ? 1 : 0), T);
  auto it = L.graphs.find(key);
  if (it != L.graphs.end()) {
    GLASS_CUDA(cudaGraphLaunch(it->second, s), "ucb_waveform graph launch");
  } else {
    GLASS_CUDA(legacy_enqueue(L, fmt, T, BW, NI, nout), "ucb_waveform launch");
    if (L.graphs.size() < 256) {
      // record the sequence for the next calls (the kernels' attributes are set by now)
      GLASS_CUDA(cudaStreamSynchronize(s), "ucb_waveform sync");
      cudaGraph_t g = nullptr;
      cudaGraphExec_t ge = nullptr;
      GLASS_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
      cudaError_t e = legacy_enqueue(L, fmt, T, BW, NI, nout);
      cudaError_t e2 = cudaStreamEndCapture(s, &g);
      if (e == cudaSuccess && e2 == cudaSuccess && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess) L.graphs[key] = ge;
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();  // a failed capture leaves the direct path in use
    }
  }
  GLASS_CUDA(cudaStreamSynchronize(s), "ucb_waveform sync");
  memcpy(X, L.h_out, sizeof(double) * 2 * BW);
  if (all) {
    memcpy(Y, L.h_out + 2 * BW, sizeof(double) * 2 * BW);
    memcpy(Z, L.h_out + 4 * BW, sizeof(double) * 2 * BW);
    memcpy(A, L.h_out + 6 * BW, sizeof(double) * 2 * BW);
    memcpy(E, L.h_out + 8 * BW, sizeof(double) * 2 * BW);
  }
  return GLASS_OK;
}

extern "C" int glass_ucb_waveform(const double *orbit_xyz, const char *format, double T, double t0,
                                  const double *params, int NParams, double *X, double *Y, double *Z, double *A,
                                  double *E, int BW, int NI) {
  int fmt = format_code(format);
  if (fmt < 0) return set_err(GLASS_ERR_FORMAT, "Unsupported data format %s", format ? format : "(null)");
  if (!is_pow2_in_range(BW)) return set_err(GLASS_ERR_SIZE, "ucb_waveform: BW must be a power of two in [32, 4096]");
  if (!params || !X || ((fmt == GLASS_FMT_SANGRIA || NI > 1) && (!Y || !Z || !A || !E)))
    return set_err(GLASS_ERR_ARG, "ucb_waveform: null argument");
  if (NParams < 7 || NParams > 8) return set_err(GLASS_ERR_ARG, "ucb_waveform: NParams must be 7 or 8");
  int rc = legacy_init();
  if (rc) return rc;
  LegacyThread &L = g_legacy;
  for (int n = 0; n < BW; n++) {
    double t = t0 + T * (double)n / (double)BW;  // ucb/src/glass_ucb_waveform.c:843
    double xyz[9];
    if (orbit_xyz) {
      memcpy(xyz, orbit_xyz + 9 * (size_t)n, sizeof(xyz));
    } else {
      analytic_positions(t, xyz);
    }
    OrbitSample64 &o = L.h_pos()[n];
    for (int i = 0; i < 3; i++) {
      o.x[i] = xyz[3 * i];
      o.y[i] = xyz[3 * i + 1];
      o.z[i] = xyz[3 * i + 2];
    }
    o.t = t;
  }
  return legacy_waveform_run(fmt, T, params, NParams, X, Y, Z, A, E, BW, NI);
}

extern "C" void ucb_waveform(struct Orbit *orbit, char *format, double T, double t0, double *params, int NParams,
                             double *X, double *Y, double *Z, double *A, double *E, int BW, int NI) {
  int fmt = format_code(format);
  if (fmt < 0) {
    fprintf(stderr, "Unsupported data format %s", format ? format : "(null)");  // ucb/src/glass_ucb_waveform.c:973
    exit(1);
  }
  int rc = GLASS_OK;
  if (!is_pow2_in_range(BW) || NParams < 7 || NParams > 8) {
    rc = set_err(GLASS_ERR_SIZE, "ucb_waveform: BW must be a power of two in [32, 4096] and NParams 7 or 8");
  } else if ((rc = legacy_init()) == GLASS_OK) {
    const OrbitLayout *o = reinterpret_cast<const OrbitLayout *>(orbit);
    LegacyThread &L = g_legacy;
    double x[4], y[4], z[4];
    for (int n = 0; n < BW; n++) {
      double t = t0 + T * (double)(n) / (double)BW;
      o->orbit_function(orbit, t, x, y, z);
      OrbitSample64 &s = L.h_pos()[n];
      for (int i = 0; i < 3; i++) {
        s.x[i] = x[i + 1];
        s.y[i] = y[i + 1];
        s.z[i] = z[i + 1];
      }
      s.t = t;
    }
    rc = legacy_waveform_run(fmt, T, params, NParams, X, Y, Z, A, E, BW, NI);
  }
  if (rc != GLASS_OK) {
    fprintf(stderr, "ucb_waveform (GB300): %s\n", g_err.c_str());
    exit(1);
  }
}

// ucb/src/glass_ucb_waveform.c:698-725, with AEnoise of utils/src/glass_lisa.c:1188-1198.
static double aenoise_host(double L, double fstar, double f) {
  double fonfstar = f / fstar;
  double sf = sin(fonfstar);
  double trans = sf * sf;
  double r = 1.0e-4 / f;
  double red = 1. + 16.0 * (pow((2.0e-5 / f), 10.0) + r * r);
  double w = kPI2 * f;
  double w4 = w * w * w * w;
  return (16.0 / 3.0) * trans *
         ((2.0 + cos(fonfstar)) * (kSPS + kSLOC) +
          2.0 * (3.0 + 2.0 * cos(fonfstar) + cos(2.0 * fonfstar)) * (kSLOC / 2.0 + kSACC / w4 * red)) /
         ((2.0 * L) * (2.0 * L));
}

static int pow2_above_host(double v) {
  if (!(v >= 1.0)) return 1;
  int e = ilogb(v) + 1;
  return e > 30 ? (1 << 30) : (1 << e);
}

extern "C" int ucb_bandwidth(double L, double fstar, double f, double fdot, double costheta, double A, double T,
                             int N) {
  const int Nmin = 16;
  int half = N / 2;
  int Nmax = 1;
  while (Nmax * 2 <= half) Nmax *= 2;
  if (half < 1) Nmax = 0;
  double sqT = sqrt(T);
  double sf = sin(f / fstar);
  double sn = aenoise_host(L, fstar, f);
  double sintheta = sin(acos(costheta));
  double bw = 2 * T * ((4. + kPI2 * f * (kAU / kCLIGHT) * sintheta) / kYEAR + fabs(fdot) * T);
  int DS = pow2_above_host(bw - 1);
  if (DS > Nmax) DS = Nmax;
  if (DS < Nmin) DS = Nmin;
  double SNRm = A * sqT * sf / sqrt(sn);
  int SS = pow2_above_host(SNRm - 1);
  if (SS > Nmax) SS = Nmax;
  if (SS < Nmin) SS = Nmin;
  return (DS > SS) ? DS : SS;
}

// ------------------------------------------------------------------ WDM
extern "C" int glass_wdm_window(int NF, int NT, double A, double nx, int forward, double *phif) {
  if (!phif || NF < 1 || NT < 2 || NT % 2) return set_err(GLASS_ERR_ARG, "glass_wdm_window: bad grid or null output");
  if (!(nx > 0) || !(A >= 0)) return set_err(GLASS_ERR_ARG, "glass_wdm_window: need nx > 0 and A >= 0");
  wdm_window(NF, NT, A, nx, forward != 0, phif);
  return GLASS_OK;
}

static int wdm_plan_for(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx) {
  if (precision != GLASS_PREC_FP64 && precision != GLASS_PREC_MIXED)
    return set_err(GLASS_ERR_ARG, "WDM: precision must be GLASS_PREC_FP64 or GLASS_PREC_MIXED");
  if (!(nx > 0) || !(A >= 0) || !(2 * A < M_PI / NF))
    return set_err(GLASS_ERR_ARG, "WDM: need nx > 0 and 0 <= A < pi / (2 NF)");
  if (!wdm_grid_supported(NF, NT))
    return set_err(GLASS_ERR_SIZE,
                   "WDM: unsupported grid (NT even, 8..4096, NT and NF NT/2 of the form 2^a 3^b, NF NT/2 <= 4096^2)");
  WdmPlan &P = ctx->wdm;
  if (P.base && P.precision == precision && P.NF == NF && P.NT == NT && P.A == A && P.nx == nx) return GLASS_OK;
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "WDM plan sync");
  std::vector<double> win(NT / 2 + 1);
  wdm_window(NF, NT, A, nx, true, win.data());
  GLASS_CUDA(wdm_prepare(P, precision, NF, NT, win.data(), ctx->stream), "WDM plan");
  P.A = A;
  P.nx = nx;
  return GLASS_OK;
}

extern "C" int glass_gpu_wdm_forward(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx,
                                     const double *time, double *wdm) {
  if (!ctx || !time || !wdm) return set_err(GLASS_ERR_ARG, "glass_gpu_wdm_forward: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  if ((rc = wdm_plan_for(ctx, precision, NF, NT, A, nx))) return rc;
  GLASS_CUDA(wdm_forward(ctx->wdm, time, wdm, ctx->stream), "glass_gpu_wdm_forward");
  return GLASS_OK;
}

extern "C" int glass_gpu_wdm_inverse(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx,
                                     const double *wdm, double *time) {
  if (!ctx || !time || !wdm) return set_err(GLASS_ERR_ARG, "glass_gpu_wdm_inverse: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  if ((rc = wdm_plan_for(ctx, precision, NF, NT, A, nx))) return rc;
  GLASS_CUDA(wdm_inverse(ctx->wdm, wdm, time, ctx->stream), "glass_gpu_wdm_inverse");
  return GLASS_OK;
}

extern "C" int glass_gpu_wdm_to_freq(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx,
                                     const double *wdm, double *freq) {
  if (!ctx || !wdm || !freq) return set_err(GLASS_ERR_ARG, "glass_gpu_wdm_to_freq: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  if ((rc = wdm_plan_for(ctx, precision, NF, NT, A, nx))) return rc;
  GLASS_CUDA(wdm_to_freq(ctx->wdm, wdm, freq, ctx->stream), "glass_gpu_wdm_to_freq");
  return GLASS_OK;
}

extern "C" int glass_gpu_wdm_from_freq(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx,
                                       const double *freq, double *wdm) {
  if (!ctx || !wdm || !freq) return set_err(GLASS_ERR_ARG, "glass_gpu_wdm_from_freq: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  if ((rc = wdm_plan_for(ctx, precision, NF, NT, A, nx))) return rc;
  GLASS_CUDA(wdm_from_freq(ctx->wdm, freq, wdm, ctx->stream), "glass_gpu_wdm_from_freq");
  return GLASS_OK;
}

static int wdm_host(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx, const double *in,
                    double *out, bool forward) {
  if (!ctx || !in || !out) return set_err(GLASS_ERR_ARG, "glass_gpu_wdm_*_host: null argument");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  if ((rc = wdm_plan_for(ctx, precision, NF, NT, A, nx))) return rc;
  const size_t bytes = sizeof(double) * (size_t)NF * NT;
  if (ctx->wdm_stage_cap < bytes) {
    GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "WDM stage sync");
    cudaFree(ctx->wdm_stage);
    ctx->wdm_stage = nullptr;
    ctx->wdm_stage_cap = 0;
    GLASS_CUDA(cudaMalloc(&ctx->wdm_stage, bytes), "cudaMalloc(WDM stage)");
    ctx->wdm_stage_cap = bytes;
  }
  double *d = (double *)ctx->wdm_stage;
  GLASS_CUDA(cudaMemcpyAsync(d, in, bytes, cudaMemcpyHostToDevice, ctx->stream), "WDM upload");
  GLASS_CUDA(forward ? wdm_forward(ctx->wdm, d, d, ctx->stream) : wdm_inverse(ctx->wdm, d, d, ctx->stream),
             "WDM transform");
  GLASS_CUDA(cudaMemcpyAsync(out, d, bytes, cudaMemcpyDeviceToHost, ctx->stream), "WDM download");
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "WDM sync");
  return GLASS_OK;
}

extern "C" int glass_gpu_wdm_forward_host(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx,
                                          const double *time, double *wdm) {
  return wdm_host(ctx, precision, NF, NT, A, nx, time, wdm, true);
}

extern "C" int glass_gpu_wdm_inverse_host(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx,
                                          const double *wdm, double *time) {
  return wdm_host(ctx, precision, NF, NT, A, nx, wdm, time, false);
}

extern "C" int glass_gpu_wdm_by_layers_host(glass_gpu_ctx *ctx, int NF, int NT, int jmin, int nlayers,
                                            const double *window, double *timedata) {
  if (!ctx || !window || !timedata) return set_err(GLASS_ERR_ARG, "glass_gpu_wdm_by_layers_host: null argument");
  const long long N = (long long)NT * (nlayers + 1);
  int r = (int)(N / 2);
  while (r > 1 && r % 3 == 0) r /= 3;
  while (r > 1 && r % 2 == 0) r /= 2;
  if (NT < 4 || (NT & (NT - 1)) || nlayers < 1 || r != 1 || N % 2)
    return set_err(GLASS_ERR_SIZE, "glass_gpu_wdm_by_layers_host: NT a power of two, NT (Nlayers + 1) / 2 of the "
                                   "form 2^a 3^b");
  if ((size_t)(N / 2 + NT) * sizeof(double2) > 227 * 1024)
    return set_err(GLASS_ERR_SIZE, "glass_gpu_wdm_by_layers_host: NT (Nlayers + 3) / 2 complex values must fit "
                                   "227 KB of shared memory");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  std::vector<double2> tw((size_t)N);
  wdm_unit_roots((int)N, tw.data());
  const size_t nwin = (size_t)NT / 2 + 1;
  const size_t bytes = sizeof(double2) * N + sizeof(double) * (N + nwin);
  void *mem = nullptr;
  GLASS_CUDA(cudaMallocAsync(&mem, bytes, ctx->stream), "cudaMallocAsync(by_layers)");
  double2 *d_tw = (double2 *)mem;
  double *d_data = (double *)(d_tw + N), *d_win = d_data + N;
  cudaError_t e = cudaMemcpyAsync(d_tw, tw.data(), sizeof(double2) * N, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_data, timedata, sizeof(double) * N, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_win, window, sizeof(double) * nwin, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = wdm_by_layers_launch(NF, NT, jmin, nlayers, d_win, d_tw, d_data, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(timedata, d_data, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->stream);
  cudaFreeAsync(mem, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  GLASS_CUDA(e, "wdm_by_layers");
  return GLASS_OK;
}

// ------------------------------------------------------------ wavelet-domain UCB path
static constexpr int kWvChunk = 4096;  // sources per launch sequence (bounds the work memory)

static bool smooth23_even(int x) {
  if (x < 2 || x % 2) return false;
  while (x % 3 == 0) x /= 3;
  return (x & (x - 1)) == 0;
}

extern "C" int glass_gpu_wavelet_setup(glass_gpu_ctx *ctx, double Tobs, double t0, int NF, int NT, double wdt,
                                       double wdf, double A, double nx, int kmin, int kmax, int norb,
                                       const double *orbit_t, const double *orbit_pos) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "glass_gpu_wavelet_setup: null context");
  if (!(Tobs > 0) || !(wdt > 0) || !(wdf > 0) || !(A >= 0) || !(nx > 0) || NF < 2)
    return set_err(GLASS_ERR_ARG, "glass_gpu_wavelet_setup: need Tobs, wdt, wdf, nx > 0, A >= 0, NF >= 2");
  if (!smooth23_even(NT) || NT < 8 || NT > kWvMaxNT)
    return set_err(GLASS_ERR_SIZE, "glass_gpu_wavelet_setup: NT must be even, of the form 2^a 3^b, 8..4096");
  if (kmin < 0 || kmax <= kmin || kmin % NT || kmax % NT || kmax / NT > NF + 1)
    return set_err(GLASS_ERR_ARG, "glass_gpu_wavelet_setup: need 0 <= kmin < kmax, both whole layers of the grid");
  WvGridHost h;
  h.Tobs = Tobs;
  h.t0 = t0;
  h.NF = NF;
  h.NT = NT;
  h.wdt = wdt;
  h.wdf = wdf;
  h.A = A;
  h.nx = nx;
  h.kmin = kmin;
  h.kmax = kmax;
  if (orbit_t || orbit_pos) {
    if (!orbit_t || !orbit_pos || norb < 20 || norb > kWvMaxOrb)
      return set_err(GLASS_ERR_ARG, "glass_gpu_wavelet_setup: orbit needs t and positions of 20..2048 nodes");
    h.orb_t.assign(orbit_t, orbit_t + norb);
    h.orb_pos.assign(orbit_pos, orbit_pos + (size_t)9 * norb);
    for (int i = 1; i < norb; i++)
      if (!(h.orb_t[i] > h.orb_t[i - 1])) return set_err(GLASS_ERR_ARG, "glass_gpu_wavelet_setup: orbit times must increase");
  } else {
    wv_analytic_orbit(Tobs, t0, h.orb_t, h.orb_pos);
    if ((int)h.orb_t.size() > kWvMaxOrb) return set_err(GLASS_ERR_SIZE, "glass_gpu_wavelet_setup: observation too long");
  }
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "wavelet setup sync");
  cudaFree(ctx->wv_grid_mem);
  cudaFree(ctx->wv_data_mem);
  cudaFree(ctx->wv_work_mem);
  ctx->wv_grid_mem = ctx->wv_data_mem = ctx->wv_work_mem = nullptr;
  ctx->wv_data_ready = false;
  ctx->wv = WvGridDev{};
  ctx->wvw = WvWorkDev{};
  GLASS_CUDA(wv_build_grid(h, &ctx->wv, &ctx->wv_grid_mem, ctx->stream), "wavelet grid tables");
  const size_t N = (size_t)(kmax - kmin);
  // FP64 residual and invC, per-pixel data terms, then the mixed-precision copies
  GLASS_CUDA(cudaMalloc(&ctx->wv_data_mem, sizeof(double) * 13 * N + sizeof(float) * 15 * N),
             "cudaMalloc(wavelet data)");
  {
    double *d = (double *)ctx->wv_data_mem;
    ctx->wv.res = d;
    ctx->wv.invC = d + 3 * N;
    ctx->wv.qpix = d + 12 * N;
    float *f = (float *)(d + 13 * N);
    ctx->wv.res_hi = f;
    ctx->wv.res_lo = f + 3 * N;
    ctx->wv.invC32 = f + 6 * N;
    ctx->wv.scale = 1.0;
  }
  const size_t wb = wv_work_bytes(kWvChunk, ctx->wv.norb, NT);
  GLASS_CUDA(cudaMalloc(&ctx->wv_work_mem, wb), "cudaMalloc(wavelet work)");
  wv_work_carve(ctx->wvw, ctx->wv_work_mem, kWvChunk, ctx->wv.norb, NT);
  GLASS_CUDA(cudaMemset(ctx->wvw.total, 0, sizeof(unsigned long long)), "cudaMemset(wavelet re-evaluation count)");
  return GLASS_OK;
}

extern "C" int glass_gpu_wavelet_reevaluated(glass_gpu_ctx *ctx, unsigned long long *count) {
  if (!ctx || !count) return set_err(GLASS_ERR_ARG, "glass_gpu_wavelet_reevaluated: null argument");
  *count = 0;
  if (!ctx->wvw.total) return GLASS_OK;
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  GLASS_CUDA(cudaMemcpyAsync(count, ctx->wvw.total, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream),
             "read wavelet re-evaluation count");
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "read wavelet re-evaluation count");
  return GLASS_OK;
}

extern "C" int glass_gpu_wavelet_set_data(glass_gpu_ctx *ctx, const double *rX, const double *rY, const double *rZ,
                                          const double *invC) {
  if (!ctx || !rX || !rY || !rZ || !invC) return set_err(GLASS_ERR_ARG, "glass_gpu_wavelet_set_data: null argument");
  if (!ctx->wv_grid_mem) return set_err(GLASS_ERR_STATE, "glass_gpu_wavelet_set_data: call glass_gpu_wavelet_setup first");
  int rc = ctx_activate(ctx);
  if (rc) return rc;
  const size_t N = (size_t)ctx->wv.N;
  double *d = (double *)ctx->wv_data_mem;
  GLASS_CUDA(cudaMemcpyAsync(d, rX, sizeof(double) * N, cudaMemcpyHostToDevice, ctx->stream), "upload rX");
  GLASS_CUDA(cudaMemcpyAsync(d + N, rY, sizeof(double) * N, cudaMemcpyHostToDevice, ctx->stream), "upload rY");
  GLASS_CUDA(cudaMemcpyAsync(d + 2 * N, rZ, sizeof(double) * N, cudaMemcpyHostToDevice, ctx->stream), "upload rZ");
  GLASS_CUDA(cudaMemcpyAsync(d + 3 * N, invC, sizeof(double) * 9 * N, cudaMemcpyHostToDevice, ctx->stream),
             "upload invC");
  // mixed-precision copies: residual / s (hi + lo), invC s^2, per-pixel r^T invC r
  std::vector<float> rhi, rlo, ic32;
  std::vector<double> qp;
  double scale = 1.0;
  wv_mixed_data((int)N, ctx->wv.NT, rX, rY, rZ, invC, &scale, rhi, rlo, ic32, qp);
  GLASS_CUDA(cudaMemcpyAsync((void *)ctx->wv.qpix, qp.data(), sizeof(double) * qp.size(), cudaMemcpyHostToDevice,
                             ctx->stream),
             "upload data terms");
  GLASS_CUDA(cudaMemcpyAsync((void *)ctx->wv.res_hi, rhi.data(), sizeof(float) * rhi.size(), cudaMemcpyHostToDevice,
                             ctx->stream),
             "upload residual hi");
  GLASS_CUDA(cudaMemcpyAsync((void *)ctx->wv.res_lo, rlo.data(), sizeof(float) * rlo.size(), cudaMemcpyHostToDevice,
                             ctx->stream),
             "upload residual lo");
  GLASS_CUDA(cudaMemcpyAsync((void *)ctx->wv.invC32, ic32.data(), sizeof(float) * ic32.size(),
                             cudaMemcpyHostToDevice, ctx->stream),
             "upload invC32");
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "wavelet data sync");
  ctx->wv.scale = scale;
  ctx->wv_data_ready = true;
  return GLASS_OK;
}

static int wv_check(glass_gpu_ctx *ctx, int nitems, const void *params, const char *who, bool need_data) {
  if (!ctx) return set_err(GLASS_ERR_ARG, "%s: null context", who);
  if (nitems < 0) return set_err(GLASS_ERR_ARG, "%s: negative item count", who);
  if (nitems > 0 && !params) return set_err(GLASS_ERR_ARG, "%s: null params", who);
  if (!ctx->wv_grid_mem) return set_err(GLASS_ERR_STATE, "%s: call glass_gpu_wavelet_setup first", who);
  if (need_data && !ctx->wv_data_ready) return set_err(GLASS_ERR_STATE, "%s: call glass_gpu_wavelet_set_data first", who);
  return ctx_activate(ctx);
}

static int wv_precision_ok(int precision, const char *who) {
  if (precision != GLASS_PREC_FP64 && precision != GLASS_PREC_MIXED)
    return set_err(GLASS_ERR_ARG, "%s: precision must be GLASS_PREC_FP64 or GLASS_PREC_MIXED", who);
  return GLASS_OK;
}

extern "C" int glass_gpu_wavelet_dlogl_batch(glass_gpu_ctx *ctx, int precision, int nitems, const double *params,
                                             const double *term_x, double *dlogl, double *term_y, double *hh,
                                             int *status) {
  int rc = wv_precision_ok(precision, "glass_gpu_wavelet_dlogl_batch");
  if (rc) return rc;
  rc = wv_check(ctx, nitems, params, "glass_gpu_wavelet_dlogl_batch", true);
  if (rc) return rc;
  ctx->last_launches = 0;
  for (int off = 0; off < nitems; off += kWvChunk) {
    const int n = std::min(kWvChunk, nitems - off);
    GLASS_CUDA(wv_waveform_launch(ctx->wv, ctx->wvw, precision, n, params + 8 * (size_t)off,
                                  status ? status + off : nullptr, ctx->stream, &ctx->last_launches),
               "wavelet waveform launch");
    GLASS_CUDA(wv_dlogl_launch(ctx->wv, ctx->wvw, precision, n, term_x ? term_x + off : nullptr,
                               dlogl ? dlogl + off : nullptr,
                               term_y ? term_y + off : nullptr, hh ? hh + off : nullptr,
                               status ? status + off : nullptr, ctx->stream, &ctx->last_launches, ctx->mixed_tol),
               "wavelet dlogl launch");
  }
  return GLASS_OK;
}

static constexpr int kWvFisherChunk = kWvChunk / 16;  // sources per Fisher launch sequence (16 waveforms each)

extern "C" int glass_gpu_wavelet_fisher_batch(glass_gpu_ctx *ctx, int nitems, const double *params, int imin,
                                              int imax, double *fisher, int *status) {
  int rc = wv_check(ctx, nitems, params, "glass_gpu_wavelet_fisher_batch", true);
  if (rc) return rc;
  if (nitems > 0 && !fisher) return set_err(GLASS_ERR_ARG, "glass_gpu_wavelet_fisher_batch: null fisher");
  if (!ctx->wv_fisher_mem)
    GLASS_CUDA(cudaMalloc(&ctx->wv_fisher_mem, sizeof(double) * 8 * 16 * (size_t)kWvFisherChunk),
               "cudaMalloc(fisher parameters)");
  ctx->last_launches = 0;
  for (int off = 0; off < nitems; off += kWvFisherChunk) {
    const int n = std::min(kWvFisherChunk, nitems - off);
    GLASS_CUDA(wv_fisher_launch(ctx->wv, ctx->wvw, n, params + 8 * (size_t)off, (double *)ctx->wv_fisher_mem, imin,
                                imax, fisher + 64 * (size_t)off, status ? status + off : nullptr, ctx->stream,
                                &ctx->last_launches),
               "wavelet fisher launch");
  }
  return GLASS_OK;
}

extern "C" int glass_gpu_wavelet_fisher_batch_host(glass_gpu_ctx *ctx, int nitems, const double *params, int imin,
                                                   int imax, double *fisher, int *status) {
  int rc = wv_check(ctx, nitems, params, "glass_gpu_wavelet_fisher_batch_host", true);
  if (rc) return rc;
  if (nitems == 0) return GLASS_OK;
  if (!fisher) return set_err(GLASS_ERR_ARG, "glass_gpu_wavelet_fisher_batch_host: null fisher");
  const size_t nd = (size_t)nitems;
  const size_t bytes = sizeof(double) * 72 * nd + sizeof(int) * nd + 256;
  if ((rc = ensure_stage(ctx, bytes))) return rc;
  double *dp = (double *)ctx->d_stage, *df = dp + 8 * nd;
  int *dst = (int *)(df + 64 * nd);
  GLASS_CUDA(cudaMemcpyAsync(dp, params, sizeof(double) * 8 * nd, cudaMemcpyHostToDevice, ctx->stream), "H2D params");
  if ((rc = glass_gpu_wavelet_fisher_batch(ctx, nitems, dp, imin, imax, df, dst))) return rc;
  GLASS_CUDA(cudaMemcpyAsync(fisher, df, sizeof(double) * 64 * nd, cudaMemcpyDeviceToHost, ctx->stream),
             "D2H fisher");
  if (status)
    GLASS_CUDA(cudaMemcpyAsync(status, dst, sizeof(int) * nd, cudaMemcpyDeviceToHost, ctx->stream), "D2H status");
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "wavelet fisher sync");
  return GLASS_OK;
}

extern "C" int glass_gpu_wavelet_waveform_batch(glass_gpu_ctx *ctx, int precision, int nitems, const double *params,
                                                int *info, double *xyz, int *status) {
  int rc = wv_precision_ok(precision, "glass_gpu_wavelet_waveform_batch");
  if (rc) return rc;
  rc = wv_check(ctx, nitems, params, "glass_gpu_wavelet_waveform_batch", false);
  if (rc) return rc;
  if (precision == GLASS_PREC_MIXED && !ctx->wv_data_ready)
    return set_err(GLASS_ERR_STATE, "glass_gpu_wavelet_waveform_batch: mixed precision scales by the data's noise level; "
                                    "call glass_gpu_wavelet_set_data first");
  ctx->last_launches = 0;
  const size_t per = (size_t)3 * kWvMaxLayers * ctx->wv.NT;
  for (int off = 0; off < nitems; off += kWvChunk) {
    const int n = std::min(kWvChunk, nitems - off);
    GLASS_CUDA(wv_waveform_launch(ctx->wv, ctx->wvw, precision, n, params + 8 * (size_t)off,
                                  status ? status + off : nullptr, ctx->stream, &ctx->last_launches),
               "wavelet waveform launch");
    GLASS_CUDA(wv_export(ctx->wv, ctx->wvw, precision, n, info ? info + 4 * (size_t)off : nullptr,
                         xyz ? xyz + per * off : nullptr, ctx->stream),
               "wavelet export");
  }
  return GLASS_OK;
}

extern "C" int glass_gpu_wavelet_dlogl_batch_host(glass_gpu_ctx *ctx, int precision, int nitems, const double *params,
                                                  const double *term_x, double *dlogl, double *term_y, double *hh,
                                                  int *status) {
  int rc = wv_precision_ok(precision, "glass_gpu_wavelet_dlogl_batch_host");
  if (rc) return rc;
  rc = wv_check(ctx, nitems, params, "glass_gpu_wavelet_dlogl_batch_host", true);
  if (rc) return rc;
  if (nitems == 0) return GLASS_OK;
  const size_t n = (size_t)nitems;
  const size_t bytes = sizeof(double) * n * 12 + sizeof(int) * n + 256;
  if ((rc = ensure_stage(ctx, bytes))) return rc;
  double *dp = (double *)ctx->d_stage, *dtx = dp + 8 * n, *ddl = dtx + n, *dty = ddl + n, *dhh = dty + n;
  int *dst = (int *)(dhh + n);
  GLASS_CUDA(cudaMemcpyAsync(dp, params, sizeof(double) * 8 * n, cudaMemcpyHostToDevice, ctx->stream), "upload params");
  if (term_x)
    GLASS_CUDA(cudaMemcpyAsync(dtx, term_x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream), "upload term_x");
  if ((rc = glass_gpu_wavelet_dlogl_batch(ctx, precision, nitems, dp, term_x ? dtx : nullptr, ddl, dty, dhh, dst)))
    return rc;
  if (dlogl) GLASS_CUDA(cudaMemcpyAsync(dlogl, ddl, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream), "dl");
  if (term_y) GLASS_CUDA(cudaMemcpyAsync(term_y, dty, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream), "ty");
  if (hh) GLASS_CUDA(cudaMemcpyAsync(hh, dhh, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream), "hh");
  if (status) GLASS_CUDA(cudaMemcpyAsync(status, dst, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream), "st");
  GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "wavelet dlogl sync");
  return GLASS_OK;
}

extern "C" int glass_gpu_wavelet_waveform_batch_host(glass_gpu_ctx *ctx, int precision, int nitems, const double *params,
                                                     int *info, double *xyz, int *status) {
  int rc = wv_precision_ok(precision, "glass_gpu_wavelet_waveform_batch_host");
  if (rc) return rc;
  rc = wv_check(ctx, nitems, params, "glass_gpu_wavelet_waveform_batch_host", false);
  if (rc) return rc;
  if (nitems == 0) return GLASS_OK;
  const size_t per = (size_t)3 * kWvMaxLayers * ctx->wv.NT;
  for (int off = 0; off < nitems; off += kWvChunk) {
    const size_t n = (size_t)std::min(kWvChunk, nitems - off);
    const size_t nx = xyz ? per * n : 0;
    const size_t bytes = sizeof(double) * (8 * n + nx) + sizeof(int) * n * 5 + 256;
    if ((rc = ensure_stage(ctx, bytes))) return rc;
    double *dp = (double *)ctx->d_stage, *dx = xyz ? dp + 8 * n : nullptr;
    int *dinfo = (int *)(dp + 8 * n + nx), *dst = dinfo + 4 * n;
    GLASS_CUDA(cudaMemcpyAsync(dp, params + 8 * (size_t)off, sizeof(double) * 8 * n, cudaMemcpyHostToDevice,
                               ctx->stream),
               "upload params");
    if ((rc = glass_gpu_wavelet_waveform_batch(ctx, precision, (int)n, dp, dinfo, dx, dst))) return rc;
    if (info)
      GLASS_CUDA(cudaMemcpyAsync(info + 4 * (size_t)off, dinfo, sizeof(int) * 4 * n, cudaMemcpyDeviceToHost,
                                 ctx->stream),
                 "info");
    if (xyz)
      GLASS_CUDA(cudaMemcpyAsync(xyz + per * off, dx, sizeof(double) * per * n, cudaMemcpyDeviceToHost, ctx->stream),
                 "xyz");
    if (status)
      GLASS_CUDA(cudaMemcpyAsync(status + off, dst, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream), "status");
    GLASS_CUDA(cudaStreamSynchronize(ctx->stream), "wavelet waveform sync");
  }
  return GLASS_OK;
}

// ------------------------------------------------------------ drop-ins for the wavelet headers
static constexpr double kWaveletFilterConstant = 6.0;  // WAVELET_FILTER_CONSTANT, utils/src/glass_wavelet.h:21

// One context per host thread for the drop-in entry points (the reference's
// callers run one chain per OpenMP thread).
struct DropInThread {
  glass_gpu_ctx *ctx = nullptr;
  void *d_buf = nullptr;
  size_t d_cap = 0;
  // wavelet waveform grid cache key
  double key[14] = {0};
  bool wv_ready = false;
  std::vector<int> info;
  std::vector<double> xyz;
  ~DropInThread() {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaFree(d_buf);
    glass_gpu_destroy(ctx);
  }
};
static thread_local DropInThread g_dropin;

[[noreturn]] void dropin_fail(const char *who) {
  fprintf(stderr, "%s: %s\n", who, glass_gpu_last_error());
  exit(1);
}

glass_gpu_ctx *dropin_ctx(const char *who) {
  DropInThread &D = g_dropin;
  if (!D.ctx) {
    const char *dev = getenv("GLASS_GPU_DEVICE");
    if (glass_gpu_create(dev ? atoi(dev) : 0, &D.ctx) != GLASS_OK) dropin_fail(who);
  }
  return D.ctx;
}

static double *dropin_buf(size_t doubles, const char *who) {
  DropInThread &D = g_dropin;
  const size_t bytes = sizeof(double) * doubles;
  if (bytes > D.d_cap) {
    cudaFree(D.d_buf);
    D.d_buf = nullptr;
    D.d_cap = 0;
    cudaError_t e = cudaMalloc(&D.d_buf, bytes);
    if (e != cudaSuccess) {
      cuda_err(e, "cudaMalloc(drop-in buffer)");
      dropin_fail(who);
    }
    D.d_cap = bytes;
  }
  return (double *)D.d_buf;
}

// build_wdm_filter_freq (utils/src/glass_wavelet.c:327)
extern "C" void build_wdm_filter_freq(double *phif, int Nf, int Nt, double A, bool forward) {
  if (glass_wdm_window(Nf, Nt, A, kWaveletFilterConstant, forward ? 1 : 0, phif) != GLASS_OK)
    dropin_fail("build_wdm_filter_freq");
}

// wavelet_transform_timefreq (utils/src/glass_wavelet.c:293): in place, FP64
extern "C" void wavelet_transform_timefreq(struct Wavelets *wdm, double *timedata) {
  const WaveletsLayout *w = reinterpret_cast<const WaveletsLayout *>(wdm);
  glass_gpu_ctx *ctx = dropin_ctx("wavelet_transform_timefreq");
  if (glass_gpu_wdm_forward_host(ctx, GLASS_PREC_FP64, w->NF, w->NT, w->A, kWaveletFilterConstant, timedata,
                                 timedata) != GLASS_OK)
    dropin_fail("wavelet_transform_timefreq");
}

// wavelet_transform_timefreq_by_layers (utils/src/glass_wavelet.c:544): in
// place on the caller's NT (Nlayers + 1) samples, FP64
extern "C" void wavelet_transform_timefreq_by_layers(struct Wavelets *wdm, int jmin, int Nlayers, double *window,
                                                     double *timedata) {
  const WaveletsLayout *w = reinterpret_cast<const WaveletsLayout *>(wdm);
  glass_gpu_ctx *ctx = dropin_ctx("wavelet_transform_timefreq_by_layers");
  if (glass_gpu_wdm_by_layers_host(ctx, w->NF, w->NT, jmin, Nlayers, window, timedata) != GLASS_OK)
    dropin_fail("wavelet_transform_timefreq_by_layers");
}

static void dropin_freq(struct Wavelets *wdm, const double *in, double *out, bool to_freq, const char *who) {
  const WaveletsLayout *w = reinterpret_cast<const WaveletsLayout *>(wdm);
  glass_gpu_ctx *ctx = dropin_ctx(who);
  const size_t ND = (size_t)w->NF * w->NT;
  double *d = dropin_buf(2 * ND + 2, who);
  double *d_wdm = d, *d_freq = d + ND;
  const size_t nin = to_freq ? ND : ND + 2, nout = to_freq ? ND + 2 : ND;
  double *d_in = to_freq ? d_wdm : d_freq, *d_out = to_freq ? d_freq : d_wdm;
  cudaError_t e = cudaMemcpyAsync(d_in, in, sizeof(double) * nin, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) {
    cuda_err(e, who);
    dropin_fail(who);
  }
  int rc = to_freq ? glass_gpu_wdm_to_freq(ctx, GLASS_PREC_FP64, w->NF, w->NT, w->A, kWaveletFilterConstant, d_in, d_out)
                   : glass_gpu_wdm_from_freq(ctx, GLASS_PREC_FP64, w->NF, w->NT, w->A, kWaveletFilterConstant, d_in,
                                             d_out);
  if (rc != GLASS_OK) dropin_fail(who);
  e = cudaMemcpyAsync(out, d_out, sizeof(double) * nout, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cuda_err(e, who);
    dropin_fail(who);
  }
}

// wavelet_transform_freq (utils/src/glass_wavelet.c:410): ND/2+1 bins -> wdm
extern "C" void wavelet_transform_freq(struct Wavelets *wdm, double *freqdata, double *wdmdata) {
  dropin_freq(wdm, freqdata, wdmdata, false, "wavelet_transform_freq");
}

// wavelet_transform_inverse_freq (utils/src/glass_wavelet.c:351): wdm -> ND/2+1 bins
extern "C" void wavelet_transform_inverse_freq(struct Wavelets *wdm, double *wdmdata, double *freqdata) {
  dropin_freq(wdm, wdmdata, freqdata, true, "wavelet_transform_inverse_freq");
}

// ucb_waveform_wavelet (ucb/src/glass_ucb_waveform.c:1061): one source, host
// arrays; the orbit nodes are read from the caller's struct Orbit (t, x, y, z).
extern "C" void ucb_waveform_wavelet(struct Orbit *orbit, struct Wavelets *wdm, double Tobs, double t0,
                                     double *params, int *wavelet_list, int *Nwavelet, double *X, double *Y,
                                     double *Z) {
  static const char *who = "ucb_waveform_wavelet";
  const WaveletsLayout *w = reinterpret_cast<const WaveletsLayout *>(wdm);
  DropInThread &D = g_dropin;
  glass_gpu_ctx *ctx = dropin_wavelet_grid(orbit, wdm, Tobs, t0, who);
  const int NT = w->NT;
  const size_t per = (size_t)3 * kWvMaxLayers * NT;
  D.info.resize(4);
  D.xyz.resize(per);
  int st = 0;
  if (glass_gpu_wavelet_waveform_batch_host(ctx, GLASS_PREC_FP64, 1, params, D.info.data(), D.xyz.data(), &st) !=
      GLASS_OK)
    dropin_fail(who);
  const int jlo = D.info[2], c = D.info[3];
  if (st != 0 || c < 0) {
    set_err(GLASS_ERR_ARG, "ucb_waveform_wavelet: invalid source parameters");
    dropin_fail(who);
  }
  const int n = NT * c;
  const double *hx = D.xyz.data(), *hy = hx + kWvMaxLayers * NT, *hz = hy + kWvMaxLayers * NT;
  for (int q = 0; q < n; q++) {
    const int k = q / c + (jlo + q % c) * NT - w->kmin;
    wavelet_list[q] = k;
    X[k] = hx[q];
    Y[k] = hy[q];
    Z[k] = hz[q];
  }
  *Nwavelet = n;
}

// The calling thread's context with its wavelet grid set up for this WDM
// grid, segment and orbit (kept while they stay the same).
glass_gpu_ctx *dropin_wavelet_grid(struct Orbit *orbit, struct Wavelets *wdm, double Tobs, double t0,
                                   const char *who) {
  const WaveletsLayout *w = reinterpret_cast<const WaveletsLayout *>(wdm);
  const OrbitLayout *o = reinterpret_cast<const OrbitLayout *>(orbit);
  DropInThread &D = g_dropin;
  glass_gpu_ctx *ctx = dropin_ctx(who);
  const int norb = o->Norb;
  const double key[14] = {Tobs, t0, (double)w->NF, (double)w->NT, w->dt, w->df, w->A, (double)w->kmin,
                          (double)w->kmax, (double)norb, (double)(uintptr_t)o->t, norb > 0 ? o->t[0] : 0.0,
                          norb > 0 ? o->t[norb - 1] : 0.0, norb > 0 ? o->x[0][norb - 1] : 0.0};
  if (!D.wv_ready || memcmp(key, D.key, sizeof(key)) != 0) {
    if (norb < 20 || norb > kWvMaxOrb) {
      set_err(GLASS_ERR_ARG, "%s: orbit needs 20..2048 nodes", who);
      dropin_fail(who);
    }
    std::vector<double> pos((size_t)9 * norb);
    for (int sc = 0; sc < 3; sc++)
      for (int n = 0; n < norb; n++) {
        pos[(size_t)(3 * sc + 0) * norb + n] = o->x[sc][n];
        pos[(size_t)(3 * sc + 1) * norb + n] = o->y[sc][n];
        pos[(size_t)(3 * sc + 2) * norb + n] = o->z[sc][n];
      }
    if (glass_gpu_wavelet_setup(ctx, Tobs, t0, w->NF, w->NT, w->dt, w->df, w->A, kWaveletFilterConstant, w->kmin,
                                w->kmax, norb, o->t, pos.data()) != GLASS_OK)
      dropin_fail(who);
    memcpy(D.key, key, sizeof(key));
    D.wv_ready = true;
  }
  return ctx;
}

// Status-returning forms of the two reference variants that are not built here.
extern "C" int glass_ucb_waveform_wavelet_tab(void) {
  return set_err(GLASS_ERR_STATE,
                 "ucb_waveform_wavelet_tab: not implemented (the reference's lookup-table variant exits as not "
                 "implemented too); use ucb_waveform_wavelet");
}

extern "C" int glass_ucb_waveform_wavelet_slow(void) {
  return set_err(GLASS_ERR_STATE,
                 "ucb_waveform_wavelet_slow: not built (a debugging variant that writes files); use "
                 "ucb_waveform_wavelet");
}

// ucb/src/glass_ucb_waveform.c:1480 and :1243: report and exit, as the
// reference's lookup-table variant does
extern "C" void ucb_waveform_wavelet_tab(struct Orbit *, struct Wavelets *, double, double, double *, int *, int *,
                                         double *, double *, double *) {
  glass_ucb_waveform_wavelet_tab();
  dropin_fail("ucb_waveform_wavelet_tab");
}

extern "C" void ucb_waveform_wavelet_slow(struct Orbit *, struct Wavelets *, double, double, double *, int *, int *,
                                          double *, double *, double *) {
  glass_ucb_waveform_wavelet_slow();
  dropin_fail("ucb_waveform_wavelet_slow");
}
