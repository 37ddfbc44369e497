// Shared device/host definitions of the GB300 UCB likelihood engine.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

namespace glass {

// ------------------------------------------------------------ checked build
// With -DGLASS_GPU_CHECKS (the checked library, libglass_gb300_checks.so,
// which the test suite runs in place of compute-sanitizer) the kernels check
// their indexed accesses against the extents of the buffers they index: a
// failed check sets its site's bit in the translation unit's check word and
// skips the access, so the kernel runs to its end and the host reads the
// word (glass_gpu_check_status).  Without the flag every check is the
// constant true and compiles away.
enum : unsigned {
  kChkBankRead = 1u << 0,     // a segment bin outside the bank
  kChkSeriesRead = 1u << 1,   // a series element outside the scratch
  kChkSeriesWrite = 1u << 2,  // the same, written
  kChkItem = 1u << 3,         // a proposal index outside the batch
  kChkBinList = 1u << 4,      // a size-list slot outside its capacity
  kChkReevalList = 1u << 5,   // a re-evaluation list slot outside its capacity
  kChkOutput = 1u << 6,       // an output element outside its array
};
// Every translation unit of the checked build registers a reader of its
// check word (returns the word and clears it); check_status_all ORs them.
void register_check_reader(unsigned (*read_reset)());
unsigned check_status_all();
#ifdef GLASS_GPU_CHECKS
constexpr bool kCheckedBuild = true;
static __device__ unsigned int g_check_word;
__device__ __forceinline__ bool chk(bool ok, unsigned site) {
  if (!ok) atomicOr(&g_check_word, site);
  return ok;
}
static unsigned check_read_reset() {
  unsigned v = 0, z = 0;
  if (cudaMemcpyFromSymbol(&v, g_check_word, sizeof(v)) != cudaSuccess) v = ~0u;
  (void)cudaMemcpyToSymbol(g_check_word, &z, sizeof(z));
  return v;
}
[[maybe_unused]] static const bool g_check_registered = (register_check_reader(&check_read_reset), true);
#else
constexpr bool kCheckedBuild = false;
__device__ __forceinline__ constexpr bool chk(bool, unsigned) { return true; }
#endif

// ------------------------------------------------------ per-device launch set-up
// A kernel's dynamic shared-memory limit (cudaFuncSetAttribute) and the
// occupancy derived from it belong to the current device, and the entry points
// are called from several host threads: the set-up runs once per device, under
// a lock, and later launches on that device read the stored occupancy.
constexpr int kMaxDevices = 64;
struct LaunchSetup {
  std::mutex m;
  int occ[kMaxDevices] = {};  // 0: not yet set up on that device
};
// init(int *occ) sets the attributes and writes the occupancy (CTAs per SM).
template <typename Init>
inline cudaError_t launch_setup(LaunchSetup &s, Init init, int *occ) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  int v = __atomic_load_n(&s.occ[dev], __ATOMIC_ACQUIRE);
  if (v <= 0) {
    std::lock_guard<std::mutex> g(s.m);
    v = s.occ[dev];
    if (v <= 0) {
      if ((e = init(&v)) != cudaSuccess) return e;
      if (v < 1) v = 1;
      __atomic_store_n(&s.occ[dev], v, __ATOMIC_RELEASE);
    }
  }
  *occ = v;
  return cudaSuccess;
}

// Physical constants, identical to utils/src/glass_constants.h:31-89 and
// utils/src/glass_lisa.h:31 (the carrier phase multiplies them by ~1e5, so
// they must be the same doubles as the reference's).
constexpr double kSQ3 = 1.73205080757;
constexpr double kPI2 = 6.283185307179586;
constexpr double kPI = 3.14159265358979323846;
constexpr double kCLIGHT = 299792458.;
constexpr double kYEAR = 3.15581497632e7;
constexpr double kAU = 1.49597870700e11;
constexpr double kLARM = 2.5e9;
constexpr double kSPS = 8.321000e-23;
constexpr double kSACC = 9.000000e-30;
constexpr double kSLOC = 2.89e-24;
constexpr double kINVSQ6 = 0.408248290463863;  // utils/src/glass_lisa.c:435
constexpr double kSQRT1_2 = 0.70710678118654752440;

// Waveform sizes handled by the batched kernels: N = 32 << b, b in [0, 8).
constexpr int kNumBins = 8;
constexpr int kMinN = 32;
constexpr int kMaxN = 4096;

// ---------------------------------------------------------------- df (double-float)
// Unevaluated sum hi + lo of two floats, ~48 significant bits.  Error-free
// transformations after Knuth (two-sum) and Dekker/Ogita-Rump-Oishi (two-product
// with a fused multiply-add).
struct df {
  float hi, lo;
};

__host__ __device__ inline df df_from_double(double x) {
  float hi = (float)x;
  float lo = (float)(x - (double)hi);
  return {hi, lo};
}

__device__ __forceinline__ df two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ df quick_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}
__device__ __forceinline__ df two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  float e = __fmaf_rn(a, b, -p);
  return {p, e};
}
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  float lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return quick_two_sum(s.hi, lo);
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  float lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
  return quick_two_sum(p.hi, lo);
}
// a (double-float) times an exactly representable float b
__device__ __forceinline__ df df_mul_f(df a, float b) {
  df p = two_prod(a.hi, b);
  float lo = __fmaf_rn(a.lo, b, p.lo);
  return quick_two_sum(p.hi, lo);
}

// x reduced to [-pi, pi] and rounded to float.
__device__ __forceinline__ float df_reduce_2pi(df x) {
  const float inv2pi = 0.15915494309189535f;
  const float pi2_hi = 6.28318548202514648f;     // float(2 pi)
  const float pi2_lo = -1.7484555314695172e-07f;  // 2 pi - float(2 pi)
  float k = rintf(x.hi * inv2pi);
  df kp = two_prod(k, pi2_hi);
  df r = df_add(x, df_neg(kp));
  return __fsub_rn(__fadd_rn(r.hi, r.lo), k * pi2_lo);
}

// The same, kept as a double-float (hi in about [-pi, pi]): 2 pi is carried
// to ~1e-15 relative (hi + lo floats), so k 2 pi for the few k of a phase of
// tens of radians adds ~1e-14 rad.
__device__ __forceinline__ df df_reduce_2pi_df(df x) {
  const float inv2pi = 0.15915494309189535f;
  const float pi2_hi = 6.28318548202514648f;
  const float pi2_lo = -1.7484555314695172e-07f;
  const float k = rintf(x.hi * inv2pi);
  const df r = df_add(x, df_neg(two_prod(k, pi2_hi)));
  return df_add(r, df_neg(two_prod(k, pi2_lo)));
}

// --------------------------------------------------------- per-item constants
// Everything a waveform needs that does not depend on the sample index,
// computed once per proposal (FP64) by the plan kernel.  The antenna-pattern
// products of ucb/src/glass_ucb_waveform.c:896-897 are folded into two
// symmetric tensors per proposal,
//   Mr = DPr e+ + DCr ex,   Mi = DPi e+ + DCi ex,
// so that dplus*DPr + dcross*DCr = r.Mr.r for an arm direction r.  Symmetric
// tensors are stored as xx, xy, xz, yy, yz, zz.

// Plain-FP64 path.
struct ItemF64 {
  int seg, N, imin, pad;
  double k[3];
  double ep[6], ec[6];        // polarisation tensors e+, ex
  double DPr, DPi, DCr, DCi;  // amplitude-free polarisation factors
  double f0, fdot, phi0, dfq;  // dfq = 2 pi q / T (ucb/src/glass_ucb_waveform.c:818)
  double amp_s;               // amp / (2N)
};

// Mixed path: FP32 for everything but the carrier phase, which is carried as
// double-float values.
struct __align__(16) ItemMix {
  int seg, N, imin, pad;
  float k[4];                 // kx, ky, kz, 0
  float Mr[6], Mi[6];
  // Mr, Mi minus their float rounding: the antenna factors multiply every
  // sample of the template, so their rounding (3e-8 rms) would be a relative
  // error common to the whole template, i.e. of (h|h), which delta logL
  // carries times (h|h) for a loud template far from the data
  float Mrl[6], Mil[6];
  float fonfs0;   // f0/f*
  float fdfs;     // fdot*T/f*       : fonfs_i = fonfs0 + fdfs*(u - tau_i/T)
  float aef;      // (2/3)*fdot*T/f0 : aevol_i = 1 + aef*(u - tau_i/T)
  float w0c;      // 2 pi f0 / c
  float p7pi;     // pi*fdot*T^2 (small corrections)
  float amp_hi, amp_lo;  // amp/(2N) = amp_hi + amp_lo (gradient path)
  // amp/(2N) = m 2^e with m in [1, 2): amp_p2 = 2^e, exactly, and Mr, Mi (hi
  // and lo) hold m (DP e+ + DC ex), so the likelihood kernels scale the
  // template by a power of two, which rounds nothing
  float amp_p2;
  // k, w0c, fonfs0 minus their float rounding: they set the phase differences
  // between the arms, and so the size of the A/E combinations; a rounding
  // common to the template is a coherent phase and amplitude error
  float kl[3], w0cl, fonfs0l;
  float fdfsl, aefl;  // fdfs, aef minus their float rounding (double-float slow part)
  df eps2pi;      // 2 pi (f0 T - q)
  df beta1, beta2;  // 2 pi f0 AU/c * k_x, k_y
  df phi0;
  df p7pi_d;      // pi*fdot*T^2
};

// Gradient / Fisher path: the mixed-precision constants plus what the tangent
// templates need.  The template is h = DP H+ + DC Hx with H+, Hx the responses
// to unit plus/cross polarisation factors (ucb/src/glass_ucb_waveform.c:822-835);
// derivatives of DP, DC give the cos(iota) and psi directions.
struct __align__(16) ItemGrad {
  ItemMix m;
  float ep[6], ec[6];                 // polarisation tensors e+, ex
  float dep_c[6], dec_c[6];           // d/dcos(theta)
  float dep_p[6], dec_p[6];           // d/dphi
  float dk_c[4], dk_p[4];             // dk/dcos(theta), dk/dphi
  float DP[2], DC[2];                 // complex polarisation factors (amplitude-free)
  float dDP_i[2], dDC_i[2];           // d/dcos(iota)
  float dDP_s[2], dDC_s[2];           // d/dpsi
  float f0, fdot, invT, fstar;        // f0 (Hz), fdot (Hz/s), 1/T, f*
};

// Per-sample orbit tables, one per waveform size.  Positions of the three
// spacecraft (FP64, metres) and the sample time; and, for the mixed path,
// u = t/T and the guiding-centre angle cos/sin(2 pi t / YEAR) as double-floats.
struct OrbitSample64 {
  double x[3], y[3], z[3], t;
};
struct OrbitSampleMix {
  float u_hi, u_lo, ca_hi, ca_lo;
  float sa_hi, sa_lo, pad0, pad1;
};
// Proposal-independent geometry of one sample for the mixed slow part,
// computed in FP64 and rounded once: the spacecraft offsets from the guiding
// centre (metres), f[0..9) = x0 y0 z0 x1 y1 z1 x2 y2 z2, and the monomials of
// the three unit arms 12, 13, 23 for the quadratic forms r^T M r with M stored
// xx, xy, xz, yy, yz, zz: f[9 + 6 a ..] = x^2, 2xy, 2xz, y^2, 2yz, z^2.
struct __align__(16) GeoSampleMix {
  float f[28];
};

}  // namespace glass
