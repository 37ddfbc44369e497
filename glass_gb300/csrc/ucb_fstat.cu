// F-statistic of sky/frequency cells for sm_103a, FP64 (compiled without
// multiply-add contraction, like the FP64 likelihood path).
//
// The reference evaluates one cell at a time (get_Fstat_logL,
// ucb/src/glass_ucb_fstatistic.c:646-703): four filter waveforms by
// ucb_waveform (:231-348), their inner products with the data N^i (:350-409)
// and with each other M^ij (:411-516), M^-1 by LAPACK, logL = N^T M^-1 N / 2
// (:599-622) and the maximum-likelihood amplitude, inclination, polarisation
// and phase (:525-597, :624-644).  build_fstatistic_proposal
// (ucb/src/glass_ucb_proposal.c:1085-1182) calls it for every cell of a
// frequency x sky grid, with OpenMP over the sky rows.
//
// Here a batch of cells runs as three stages, with the cells binned by their
// filter size N = ucb_bandwidth(f0, fdot, cos theta, A = 1e-22) in 16..4096:
//   plan   one thread per cell: the per-cell geometry (shared by the four
//          filters) and the four filters' polarisation factors and phases;
//   slow   one thread per (cell, sample): the six arm series of all four
//          filters, sharing every filter-independent quantity, with each
//          filter's own arithmetic in the reference's order;
//   spec   per size, one group of N/4 threads per cell: FFT of each filter's
//          four A/E series, TDI weights and whitening per bin (the likelihood
//          path's tables), then N^i and M^ij over the segment bins
//          0 < k < NFFT, and the 4x4 solve in one lane.
// The A/E inner products of the reference weight both channels with the A
// channel's noise C[0][0]; with templates and data whitened by their own
// channel's noise, the E terms are multiplied by invC_A/invC_E per bin, which
// gives the same weights.

#include "../../include/glass_gb300.h"
#include "ucb_fd.cuh"
#include "ucb_fd_device.cuh"

namespace glass {

namespace {

constexpr int kFsBins = 9;  // N = 16 << b
constexpr int kFsSeries = 16;  // 4 filters x (A2, A1, E2, E1)

// The four filters (ucb/src/glass_ucb_fstatistic.c:262-265): amplitude 2,
// inclination pi/2, and these polarisations and phases.
__constant__ double kFsPsi[4] = {0.0, M_PI_4, 0.0, M_PI_4};
__constant__ double kFsPhase[4] = {0.0, M_PI, 3.0 * M_PI_2, M_PI_2};
// each phase as a quadrant k (phase = k pi/2 to the rounding of the double),
// and k pi/2 as a double-double hi + lo
__constant__ int kFsQuadrant[4] = {0, 2, 3, 1};
__constant__ double kFsKPio2Hi[4] = {0.0, 1.5707963267948966, 3.141592653589793, 4.71238898038469};
__constant__ double kFsKPio2Lo[4] = {0.0, 6.123233995736766e-17, 1.2246467991473532e-16, 1.8369701987210297e-16};

struct FsCell {
  ItemF64 it;        // the cell's geometry, f0, fdot, q, amp/(2N), segment, N, imin
  double DP[4][4];   // DPr, DPi, DCr, DCi of each filter
  double phi0[4];
};

struct FsPlanArgs {
  int ncells, nseg, NFFT, cap;
  int seg_const;  // segment of every cell when cell_seg is null
  double T, fstar, L;
  const int *cell_seg;
  const double *cells;
  const int *seg_qmin;
  FsCell *fc;
  int *bin_count, *bin_list;
  double *logl, *fparams;
  int *status;
};

struct FsSlowArgs {
  int cap;
  double fstar, L;
  const int *bin_count, *bin_list;
  const FsCell *fc;
  const OrbitSample64 *pos64[kNumBins];
  double2 *series;
};

struct FsSpecArgs {
  int NFFT, cap, bin;
  const int *bin_count, *bin_list;
  const FsCell *fc;
  double2 *series;
  const double2 *tw;  // twiddles of size N (size 16: every other entry of size 32's)
  int tw_stride;
  const double2 *w64, *g64;
  const double *rho;
  double *logl, *fparams;
  int *status;
};

// ------------------------------------------------------------ 4x4 algebra
// In-place inverse by Gauss-Jordan elimination with partial pivoting.
__device__ bool fs_invert4(double *m) {
  double a[4][8];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      a[i][j] = m[4 * i + j];
      a[i][4 + j] = (i == j) ? 1.0 : 0.0;
    }
  for (int c = 0; c < 4; c++) {
    int p = c;
    for (int r = c + 1; r < 4; r++)
      if (fabs(a[r][c]) > fabs(a[p][c])) p = r;
    if (a[p][c] == 0.0) return false;
    if (p != c)
      for (int j = 0; j < 8; j++) {
        double t = a[c][j];
        a[c][j] = a[p][j];
        a[p][j] = t;
      }
    const double inv = 1.0 / a[c][c];
    for (int j = 0; j < 8; j++) a[c][j] *= inv;
    for (int r = 0; r < 4; r++) {
      if (r == c) continue;
      const double f = a[r][c];
      if (f == 0.0) continue;
      for (int j = 0; j < 8; j++) a[r][j] -= f * a[c][j];
    }
  }
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) m[4 * i + j] = a[i][4 + j];
  return true;
}

// logL and the maximum-likelihood parameters from N (already times 4) and M
// (already times 4, full symmetric).  out: logL, A, iota, psi, phase.
// Returns false when M is singular but not zero.
__device__ bool fs_finish(const double *Nv, double *m, double *out) {
  // no filter bin inside the segment leaves M = 0, which LAPACK's
  // dgetrf/dgetri (utils/src/glass_math.c:501-523) leave as it is: logL = 0, a = 0
  bool any = false;
#pragma unroll
  for (int c = 0; c < 16; c++) any |= (m[c] != 0.0);
  if (any && !fs_invert4(m)) return false;
  // ucb/src/glass_ucb_fstatistic.c:612-621
  out[0] = 0.5 * (m[0] * Nv[0] * Nv[0] + 2 * m[1] * Nv[0] * Nv[1] + 2 * m[2] * Nv[0] * Nv[2] +
                  2 * m[3] * Nv[0] * Nv[3] + m[5] * Nv[1] * Nv[1] + 2 * m[6] * Nv[1] * Nv[2] +
                  2 * m[7] * Nv[1] * Nv[3] + m[10] * Nv[2] * Nv[2] + 2 * m[11] * Nv[2] * Nv[3] +
                  m[15] * Nv[3] * Nv[3]);
  // :636-643
  double a[4];
#pragma unroll
  for (int i = 0; i < 4; i++)
    a[i] = m[4 * i] * Nv[0] + m[4 * i + 1] * Nv[1] + m[4 * i + 2] * Nv[2] + m[4 * i + 3] * Nv[3];
  // :552-570
  const double a1p4 = a[0] + a[3], a2m3 = a[1] - a[2], a1m4 = a[0] - a[3], a2p3 = a[1] + a[2];
  const double Ap = sqrt(a1p4 * a1p4 + a2m3 * a2m3) + sqrt(a1m4 * a1m4 + a2p3 * a2p3);
  const double Ac = sqrt(a1p4 * a1p4 + a2m3 * a2m3) - sqrt(a1m4 * a1m4 + a2p3 * a2p3);
  double psi = atan2(Ap * a[3] - Ac * a[0], -(Ac * a[1] + Ap * a[2]));
  psi *= 0.5;
  const double sp = sin(2.0 * psi);
  const double c = (double)((sp > 0) - (sp < 0));
  out[1] = 0.5 * (Ap + sqrt(Ap * Ap - Ac * Ac));
  out[2] = acos(-Ac / (Ap + sqrt(Ap * Ap - Ac * Ac)));
  out[3] = psi;
  out[4] = atan2(c * (Ap * a[3] - Ac * a[0]), -c * (Ac * a[2] + Ap * a[1]));
  return true;
}

__device__ void fs_write(const FsPlanArgs &a, int i, const double *o, int st) {
  a.logl[i] = o[0];
  if (a.fparams)
#pragma unroll
    for (int k = 0; k < 4; k++) a.fparams[4 * (size_t)i + k] = o[1 + k];
  if (a.status) a.status[i] = st;
}

// ------------------------------------------------------------------- plan
// One thread per cell.  Filter parameters as get_filters sets them
// (ucb/src/glass_ucb_fstatistic.c:241-344): f0 T, cos theta, phi, ln 2,
// cos(pi/2), psi, phase, fdot T^2.
__global__ void __launch_bounds__(128) fs_plan_kernel(FsPlanArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int b = -1;
  if (i < a.ncells) {
    const double *x = a.cells + 4 * (size_t)i;
    const double f0 = x[0], fdot = x[1], theta = x[2], phi = x[3];
    const int seg = a.cell_seg ? a.cell_seg[i] : a.seg_const;
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    double o[5] = {nan, nan, nan, nan, nan};
    if (seg < 0 || seg >= a.nseg) {
      fs_write(a, i, o, GLASS_ITEM_BAD_SEGMENT);
    } else if (!(isfinite(f0) && isfinite(fdot) && isfinite(theta) && isfinite(phi)) || !(f0 > 0.0)) {
      fs_write(a, i, o, GLASS_ITEM_NONFINITE);
    } else {
      const double costh = cos(theta);
      const int N = bandwidth_dev(a.L, a.fstar, f0, fdot, costh, 1.e-22, a.T, a.NFFT);
      const long long q = (long long)(f0 * a.T);
      const long long qq = q - (long long)a.seg_qmin[seg];
      // filter bin i sits at segment bin qq + i - N/2 (:378, :423); bins
      // 0 < k < NFFT take part
      const long long lo = qq - N / 2, hi = lo + N - 1;
      if (N > kMaxN) {
        fs_write(a, i, o, GLASS_ITEM_NONFINITE);
      } else if (hi < 1 || lo >= a.NFFT) {
        double Nv[4] = {0, 0, 0, 0}, m[16] = {};
        fs_finish(Nv, m, o);
        fs_write(a, i, o, GLASS_ITEM_OUTSIDE);
      } else {
        FsCell c;
        double p[8];
        p[0] = f0 * a.T;
        p[1] = costh;
        p[2] = phi;
        p[3] = log(2.0);
        p[4] = cos(M_PI_2);
        p[7] = fdot * (a.T * a.T);
        for (int f = 0; f < 4; f++) {
          p[5] = kFsPsi[f];
          p[6] = kFsPhase[f];
          SourceGeom g;
          source_geometry(p, 8, a.T, g);
          if (f == 0) make_item_f64(g, N, c.it);
          c.DP[f][0] = g.DPr;
          c.DP[f][1] = g.DPi;
          c.DP[f][2] = g.DCr;
          c.DP[f][3] = g.DCi;
          c.phi0[f] = g.phi0;
        }
        c.it.seg = seg;
        c.it.N = N;
        c.it.imin = (int)lo;
        a.fc[i] = c;
        b = 31 - __clz(N) - 4;
      }
    }
  }
  // warp-aggregated binning: one atomic per distinct size per warp
  const int lane = threadIdx.x & 31;
  const unsigned active = __ballot_sync(0xffffffffu, b >= 0);
  if (b >= 0) {
    const unsigned same = __match_any_sync(active, b);
    const int first = __ffs(same) - 1;
    int base = 0;
    if (lane == first) base = atomicAdd(&a.bin_count[b], __popc(same));
    base = __shfl_sync(same, base, first);
    a.bin_list[(size_t)b * a.cap + base + __popc(same & ((1u << lane) - 1))] = i;
  }
}

// Start (in samples of one series) of size bin `bin` in the scratch: sizes in
// increasing order, cells of one size back to back, 16 series of N each.
__device__ __forceinline__ long long fs_bin_start(const int *bin_count, int bin) {
  long long acc = 0;
#pragma unroll
  for (int b = 0; b < kFsBins; b++)
    if (b < bin) acc += (long long)bin_count[b] * (16 << b);
  return acc * kFsSeries;
}

// ------------------------------------------------------------------- slow
// One thread per (cell, sample): the six arm series of the four filters
// (ucb/src/glass_ucb_waveform.c:840-922 for each filter; every quantity that
// does not depend on the filter is computed once, with the same operations),
// combined to the four A/E series and stored at [cell][filter][series][n].
__global__ void __launch_bounds__(256) fs_slow_kernel(FsSlowArgs a) {
  long long cs[kFsBins + 1];
  long long acc = 0;
#pragma unroll
  for (int b = 0; b < kFsBins; b++) {
    cs[b] = acc;
    acc += (long long)a.bin_count[b] << (b + 4);
  }
  cs[kFsBins] = acc;
  const long long total = acc;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < total; s += stride) {
    int b = 0;
#pragma unroll
    for (int bb = 1; bb < kFsBins; bb++)
      if (s >= cs[bb]) b = bb;
    const int N = 16 << b;
    const long long local = s - cs[b];
    const int slot = (int)(local >> (b + 4));
    const int n = (int)(local & (N - 1));
    const int cell = a.bin_list[(size_t)b * a.cap + slot];
    const FsCell &c = a.fc[cell];
    // size 16 samples are every other sample of size 32 (same times exactly)
    const OrbitSample64 o = b == 0 ? a.pos64[0][2 * n] : a.pos64[b - 1][n];
    const double L = a.L, fstar = a.fstar;
    double r12[3] = {(o.x[1] - o.x[0]) / L, (o.y[1] - o.y[0]) / L, (o.z[1] - o.z[0]) / L};
    double r13[3] = {(o.x[2] - o.x[0]) / L, (o.y[2] - o.y[0]) / L, (o.z[2] - o.z[0]) / L};
    double r23[3] = {(o.x[2] - o.x[1]) / L, (o.y[2] - o.y[1]) / L, (o.z[2] - o.z[1]) / L};
    const ItemF64 &it = c.it;
    const double dp12 = quad(it.ep, r12[0], r12[1], r12[2]), dc12 = quad(it.ec, r12[0], r12[1], r12[2]);
    const double dp13 = quad(it.ep, r13[0], r13[1], r13[2]), dc13 = quad(it.ec, r13[0], r13[1], r13[2]);
    const double dp23 = quad(it.ep, r23[0], r23[1], r23[2]), dc23 = quad(it.ec, r23[0], r23[1], r23[2]);
    const double kr12 = it.k[0] * r12[0] + it.k[1] * r12[1] + it.k[2] * r12[2];
    const double kr13 = it.k[0] * r13[0] + it.k[1] * r13[1] + it.k[2] * r13[2];
    const double kr23 = it.k[0] * r23[0] + it.k[1] * r23[1] + it.k[2] * r23[2];
    const double t = o.t;
    const double w0 = kPI2 * it.f0, wd = kPI * it.fdot, ae = 0.66666666666666666666 * it.fdot / it.f0;
    const double dfqt = it.dfq * t;
    double w0x[3], wdx[3], aev[3], fon[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double kdotx = (o.x[i] * it.k[0] + o.y[i] * it.k[1] + o.z[i] * it.k[2]) / kCLIGHT;
      const double xi = t - kdotx;
      fon[i] = (it.f0 + it.fdot * xi) / fstar;
      w0x[i] = w0 * xi;
      wdx[i] = wd * xi * xi;
      aev[i] = 1.0 + ae * xi;
    }
    const int ai[6] = {0, 0, 1, 1, 2, 2};
    const double dps[6] = {dp12, dp13, dp12, dp23, dp13, dp23};
    const double dcs[6] = {dc12, dc13, dc12, dc23, dc13, dc23};
    const double krs[6] = {kr12, kr13, -kr12, kr23, -kr13, -kr23};
    double arg1[6], sinc[6];
#pragma unroll
    for (int q = 0; q < 6; q++) {
      arg1[q] = 0.5 * fon[ai[q]] * (1.0 + krs[q]);
      sinc[q] = 0.25 * sin(arg1[q]) / arg1[q];
    }
    const int Nn = N;
    double2 *out = a.series + fs_bin_start(a.bin_count, b) + (long long)slot * kFsSeries * Nn + n;
    // Filter 0 (phase 0) takes sincos of its arguments x0 = arg1 - arg2.  The
    // other filters' arguments xf, rounded exactly as the reference rounds
    // them, differ from x0 by their phase k pi/2 plus ~1e-10 (the rounding of
    // w0 xi - phi0 at |w0 xi| ~ 1e6): sincos(xf) is sincos(x0) turned by the
    // quadrant k and by eps = xf - x0 - k pi/2, taken exactly (two-sum, and
    // k pi/2 as a double-double); |eps| < 1e-9, so cos eps = 1 and sin eps =
    // eps to double precision.
    double s0[6], c0[6], x0[6];
#pragma unroll 1
    for (int f = 0; f < 4; f++) {
      double arg2[3];
#pragma unroll
      for (int i = 0; i < 3; i++) {
        double a2 = w0x[i] - c.phi0[f] - dfqt;
        a2 += wdx[i];
        arg2[i] = a2;
      }
      const double DPr = c.DP[f][0], DPi = c.DP[f][1], DCr = c.DP[f][2], DCi = c.DP[f][3];
      const int k = kFsQuadrant[f];
      const double khi = kFsKPio2Hi[k], klo = kFsKPio2Lo[k];
      double2 d[6], cmb[4];
#pragma unroll
      for (int q = 0; q < 6; q++) {
        const int i = ai[q];
        const double t1r = aev[i] * (dps[q] * DPr + dcs[q] * DCr);
        const double t1i = aev[i] * (dps[q] * DPi + dcs[q] * DCi);
        const double x = arg1[q] - arg2[i];
        double s2, c2;
        if (f == 0) {
          sincos(x, &s2, &c2);
          s0[q] = s2;
          c0[q] = c2;
          x0[q] = x;
        } else {
          const double dh = x - x0[q];
          const double bb = dh - x;
          const double dl = (x - (dh - bb)) + (-x0[q] - bb);
          const double eps = ((dh - khi) + dl) - klo;
          const double rs = (k & 1) ? c0[q] : s0[q];
          const double rc = (k & 1) ? -s0[q] : c0[q];
          const double qs = (k & 2) ? -rs : rs, qc = (k & 2) ? -rc : rc;
          s2 = qs + qc * eps;
          c2 = qc - qs * eps;
        }
        d[q] = make_double2(sinc[q] * (t1r * c2 + t1i * s2), sinc[q] * (-t1r * s2 + t1i * c2));
      }
      ae_combos(d, cmb);
#pragma unroll
      for (int kk = 0; kk < 4; kk++) out[(size_t)(4 * f + kk) * Nn] = cmb[kk];
    }
  }
}

// ------------------------------------------------------------------- spec
template <int N>
struct FsCfg {
  static constexpr int GT = N / 4;
  static constexpr int CTA = GT >= 128 ? GT : 128;
  static constexpr int GPC = CTA / GT;
  static constexpr int NSER = N == 4096 ? 2 : 4;  // series in shared memory at once
  static constexpr int PASSES = 4 / NSER;
  static constexpr size_t smem = sizeof(double2) * (size_t)N * (1 + (size_t)GPC * NSER) + sizeof(double) * 32 * GPC;
};

template <int N>
__global__ void __launch_bounds__(FsCfg<N>::CTA) fs_spec_kernel(FsSpecArgs a) {
  using Cfg = FsCfg<N>;
  constexpr int GT = Cfg::GT, GPC = Cfg::GPC, NSER = Cfg::NSER, PASSES = Cfg::PASSES;
  constexpr int B = N / GT;  // bins per thread (4)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *tw = reinterpret_cast<double2 *>(smem_raw);
  double2 *bufs = tw + N;
  double *reds = reinterpret_cast<double *>(bufs + (size_t)GPC * NSER * N);
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = a.tw[(size_t)i * a.tw_stride];
  __syncthreads();
  const int count = a.bin_count[a.bin];
  double2 *ser_bin = a.series + fs_bin_start(a.bin_count, a.bin);
  const int *list = a.bin_list + (size_t)a.bin * a.cap;
  const int g = threadIdx.x / GT, lane = threadIdx.x % GT;
  double2 *buf = bufs + (size_t)g * NSER * N;
  double *red = reds + 32 * g;
  const int NFFT = a.NFFT;
  for (int base = blockIdx.x * GPC; base < count; base += gridDim.x * GPC) {
    const int slot = base + g;
    const bool valid = slot < count;
    const int sl = valid ? slot : count - 1;
    const int cell = list[sl];
    const ItemF64 &it = a.fc[cell].it;
    const int seg = it.seg, imin = it.imin;
    const double s = it.amp_s;
    double2 *ser = ser_bin + (size_t)sl * kFsSeries * N;
#pragma unroll 1
    for (int f = 0; f < 4; ++f) {
#pragma unroll 1
      for (int pass = 0; pass < PASSES; ++pass) {
#pragma unroll
        for (int q = 0; q < NSER; ++q)
#pragma unroll
          for (int r = 0; r < B; ++r)
            buf[q * N + lane + GT * r] = ser[(size_t)(4 * f + pass * NSER + q) * N + lane + GT * r];
        group_sync<GT>();
        group_fft<N, GT, NSER, 2>(buf, tw, lane);
        // template bins of this filter, in place of its A2 (A) and E2 (E) series
#pragma unroll
        for (int r = 0; r < B; ++r) {
          const int k = lane + GT * r;
          const int m = (k + N / 2) & (N - 1);  // fftshift
          const int j = imin + m;
#pragma unroll
          for (int ch = 0; ch < NSER / 2; ++ch) {
            const int chan = pass * (NSER / 2) + ch;
            double2 h = make_double2(0.0, 0.0);
            if (j > 0 && j < NFFT) {
              const size_t sj = (size_t)seg * NFFT + j;
              const double2 g2 = a.g64[4 * sj + 2 * chan], g1 = a.g64[4 * sj + 2 * chan + 1];
              h = cscale(cadd(cmul(buf[(2 * ch) * N + k], g2), cmul(buf[(2 * ch + 1) * N + k], g1)), s);
            }
            if (valid) ser[(size_t)(4 * f + 2 * chan) * N + m] = h;
          }
        }
        group_sync<GT>();
      }
    }
    // N^i and M^ij over this thread's bins (the spectra it wrote itself)
    double nacc[4] = {0, 0, 0, 0}, macc[10] = {};
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const int k = lane + GT * r;
      const int m = (k + N / 2) & (N - 1);
      const int j = imin + m;
      if (!(j > 0 && j < NFFT)) continue;
      const size_t sj = (size_t)seg * NFFT + j;
      const double2 wA = a.w64[2 * sj], wE = a.w64[2 * sj + 1];
      const double rho = a.rho[sj];
      double2 hA[4], hE[4];
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        hA[f] = ser[(size_t)(4 * f) * N + m];
        hE[f] = ser[(size_t)(4 * f + 2) * N + m];
      }
#pragma unroll
      for (int f = 0; f < 4; ++f)
        nacc[f] += (wA.x * hA[f].x + wA.y * hA[f].y) + rho * (wE.x * hE[f].x + wE.y * hE[f].y);
      int idx = 0;
#pragma unroll
      for (int f = 0; f < 4; ++f)
#pragma unroll
        for (int h = f; h < 4; ++h, ++idx)
          macc[idx] += (hA[f].x * hA[h].x + hA[f].y * hA[h].y) + rho * (hE[f].x * hE[h].x + hE[f].y * hE[h].y);
    }
#pragma unroll
    for (int f = 0; f < 4; ++f) nacc[f] = group_sum<GT>(nacc[f], red, lane);
#pragma unroll
    for (int q = 0; q < 10; ++q) macc[q] = group_sum<GT>(macc[q], red, lane);
    if (valid && lane == 0) {
      double Nv[4], m[16], o[5];
#pragma unroll
      for (int f = 0; f < 4; ++f) Nv[f] = 4.0 * nacc[f];
      int idx = 0;
#pragma unroll
      for (int f = 0; f < 4; ++f)
#pragma unroll
        for (int h = f; h < 4; ++h, ++idx) m[4 * f + h] = m[4 * h + f] = 4.0 * macc[idx];
      int st = 0;
      if (!fs_finish(Nv, m, o)) {
        const double nan = __longlong_as_double(0x7ff8000000000000ULL);
        for (int q = 0; q < 5; q++) o[q] = nan;
        st = GLASS_ITEM_NONFINITE;
      } else if (!isfinite(o[0])) {
        st = GLASS_ITEM_NONFINITE;
      }
      a.logl[cell] = o[0];
      if (a.fparams)
#pragma unroll
        for (int q = 0; q < 4; q++) a.fparams[4 * (size_t)cell + q] = o[1 + q];
      if (a.status) a.status[cell] = st;
    }
    if constexpr (GT > 32) __syncthreads();
  }
}

template <int N>
cudaError_t fs_launch_spec(const FsSpecArgs &a, int ncells, int num_sms, cudaStream_t stream) {
  using Cfg = FsCfg<N>;
  static LaunchSetup setup;
  int occ = 0;
  cudaError_t e = launch_setup(setup, [&](int *o) {
    cudaError_t r = cudaFuncSetAttribute(fs_spec_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::smem);
    if (r != cudaSuccess) return r;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, fs_spec_kernel<N>, Cfg::CTA, Cfg::smem);
  }, &occ);
  if (e != cudaSuccess) return e;
  int need = (ncells + Cfg::GPC - 1) / Cfg::GPC;
  int grid = occ * num_sms;
  if (need < grid) grid = need;
  if (grid < 1) grid = 1;
  fs_spec_kernel<N><<<grid, Cfg::CTA, Cfg::smem, stream>>>(a);
  return cudaGetLastError();
}


// ------------------------------------------------------- proposal grid
// Cell centres of the grid of build_fstatistic_proposal
// (ucb/src/glass_ucb_proposal.c:1119-1134), cell g = (i n_theta + j) n_phi + k.
__device__ __forceinline__ void fs_grid_centre(const FsGrid &G, int g, int &i, double &f, double &theta,
                                               double &phi) {
  i = g / (G.n_theta * G.n_phi);
  const int j = (g / G.n_phi) % G.n_theta, k = g % G.n_phi;
  f = G.fmin + i * G.d_f;
  f += G.d_f / 2;
  theta = acos((-1. + (double)j * G.d_theta + G.d_theta / 2));
  phi = (double)k * G.d_phi + G.d_phi / 2;
}

__global__ void fs_grid_cells_kernel(FsGrid G, int g0, int n, double *cells) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  int i;
  double f, th, ph;
  fs_grid_centre(G, g0 + c, i, f, th, ph);
  double *x = cells + 4 * (size_t)c;
  x[0] = f;
  x[1] = 0.0;
  x[2] = th;
  x[3] = ph;
}

// Cells whose fdot = 0 value exceeds 1 get the chirp-mass scan (:1136-1148):
// their grid index goes to active[], their position in it to pos[].
__global__ void fs_scan_mark_kernel(const double *logl0, int n, int *count, int *active, int *pos) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  if (logl0[g] > 1) {
    const int idx = atomicAdd(count, 1);
    active[idx] = g;
    pos[g] = idx;
  } else {
    pos[g] = -1;
  }
}

__global__ void fs_scan_cells_kernel(FsGrid G, const int *active, int c0, int n, const double *fdot_tab,
                                     double *cells) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int a = (c0 + c) / kFsScan, s = (c0 + c) % kFsScan;
  int i;
  double f, th, ph;
  fs_grid_centre(G, active[a], i, f, th, ph);
  double *x = cells + 4 * (size_t)c;
  x[0] = f;
  x[1] = fdot_tab[(size_t)i * kFsScan + s];
  x[2] = th;
  x[3] = ph;
}

// logLmax over the fdot = 0 value and the scan up to its first value below 1,
// squared (:1138-1150).
__global__ void fs_finalize_kernel(const double *logl0, const int *pos, const double *scan, int n,
                                   double *tensor) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const double v0 = logl0[g];
  double mx = v0;
  if (v0 > 1) {
    const double *sv = scan + (size_t)pos[g] * kFsScan;
    for (int s = 0; s < kFsScan; s++) {
      const double v = sv[s];
      if (v > mx) mx = v;
      if (v < 1) break;
    }
  }
  tensor[g] = mx * mx;
}

}  // namespace

// ------------------------------------------------------------------- host
size_t fs_cell_bytes() { return sizeof(FsCell); }

// Largest filter size of a segment of NFFT bins: 2^floor(log2(NFFT/2)),
// at least 16 (ucb/src/glass_ucb_waveform.c:700-701).
int fs_max_size(int NFFT) {
  int half = NFFT / 2, n = 1;
  while (n * 2 <= half) n *= 2;
  return n < 16 ? 16 : n;
}

cudaError_t fs_work_alloc(FsWorkDev &w, int cap, int NFFT) {
  const int maxN = fs_max_size(NFFT) > kMaxN ? kMaxN : fs_max_size(NFFT);
  const size_t series = (size_t)cap * kFsSeries * maxN * sizeof(double2);
  if (w.mem && cap <= w.cap && series <= w.series_bytes) return cudaSuccess;
  cudaFree(w.mem);
  w = FsWorkDev{};
  size_t off_cells = 0;
  size_t off_count = (off_cells + sizeof(FsCell) * (size_t)cap + 255) / 256 * 256;
  size_t off_list = off_count + 256;
  size_t off_series = (off_list + sizeof(int) * kFsBins * (size_t)cap + 255) / 256 * 256;
  size_t total = off_series + series;
  cudaError_t e = cudaMalloc(&w.mem, total);
  if (e != cudaSuccess) {
    w.mem = nullptr;
    return e;
  }
  char *base = (char *)w.mem;
  w.cap = cap;
  w.cells = base + off_cells;
  w.bin_count = (int *)(base + off_count);
  w.bin_list = (int *)(base + off_list);
  w.series = base + off_series;
  w.series_bytes = series;
  return cudaSuccess;
}

void fs_work_free(FsWorkDev &w) {
  cudaFree(w.mem);
  w = FsWorkDev{};
}

cudaError_t fs_launch(const FdBankDev &bank, const FdTablesDev &tab, const double *rho, FsWorkDev &w, int ncells,
                      const int *cell_seg, int seg_const, const double *cells, double *logl, double *fparams,
                      int *status, int num_sms, cudaStream_t stream, int *nlaunch) {
  cudaError_t e;
  int launches = 0;
  const int maxN = fs_max_size(bank.NFFT);
  for (int off = 0; off < ncells; off += w.cap) {
    const int n = ncells - off < w.cap ? ncells - off : w.cap;
    if ((e = cudaMemsetAsync(w.bin_count, 0, sizeof(int) * 16, stream)) != cudaSuccess) return e;
    FsPlanArgs pa;
    pa.ncells = n;
    pa.nseg = bank.nseg;
    pa.NFFT = bank.NFFT;
    pa.cap = w.cap;
    pa.T = bank.T;
    pa.fstar = bank.fstar;
    pa.L = kLARM;
    pa.cell_seg = cell_seg ? cell_seg + off : nullptr;
    pa.seg_const = seg_const;
    pa.cells = cells + 4 * (size_t)off;
    pa.seg_qmin = bank.qmin;
    pa.fc = (FsCell *)w.cells;
    pa.bin_count = w.bin_count;
    pa.bin_list = w.bin_list;
    pa.logl = logl + off;
    pa.fparams = fparams ? fparams + 4 * (size_t)off : nullptr;
    pa.status = status ? status + off : nullptr;
    fs_plan_kernel<<<(n + 127) / 128, 128, 0, stream>>>(pa);
    launches++;
    if ((e = cudaGetLastError()) != cudaSuccess) return e;

    FsSlowArgs sa;
    sa.cap = w.cap;
    sa.fstar = bank.fstar;
    sa.L = kLARM;
    sa.bin_count = w.bin_count;
    sa.bin_list = w.bin_list;
    sa.fc = (const FsCell *)w.cells;
    for (int b = 0; b < kNumBins; b++) sa.pos64[b] = tab.pos64[b];
    sa.series = (double2 *)w.series;
    {
      static LaunchSetup setup;
      int occ = 0;
      if ((e = launch_setup(setup, [&](int *o) {
             return cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, fs_slow_kernel, 256, 0);
           }, &occ)) != cudaSuccess)
        return e;
      fs_slow_kernel<<<occ * num_sms, 256, 0, stream>>>(sa);
      launches++;
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }

    FsSpecArgs ca;
    ca.NFFT = bank.NFFT;
    ca.cap = w.cap;
    ca.bin_count = w.bin_count;
    ca.bin_list = w.bin_list;
    ca.fc = (const FsCell *)w.cells;
    ca.series = (double2 *)w.series;
    ca.w64 = bank.w64;
    ca.g64 = bank.g64;
    ca.rho = rho;
    ca.logl = logl + off;
    ca.fparams = fparams ? fparams + 4 * (size_t)off : nullptr;
    ca.status = status ? status + off : nullptr;
    for (int b = 0; b < kFsBins; b++) {
      const int N = 16 << b;
      if (N > maxN || N > kMaxN) break;
      ca.bin = b;
      ca.tw = b == 0 ? tab.tw64[0] : tab.tw64[b - 1];
      ca.tw_stride = b == 0 ? 2 : 1;
      switch (N) {
        case 16: e = fs_launch_spec<16>(ca, n, num_sms, stream); break;
        case 32: e = fs_launch_spec<32>(ca, n, num_sms, stream); break;
        case 64: e = fs_launch_spec<64>(ca, n, num_sms, stream); break;
        case 128: e = fs_launch_spec<128>(ca, n, num_sms, stream); break;
        case 256: e = fs_launch_spec<256>(ca, n, num_sms, stream); break;
        case 512: e = fs_launch_spec<512>(ca, n, num_sms, stream); break;
        case 1024: e = fs_launch_spec<1024>(ca, n, num_sms, stream); break;
        case 2048: e = fs_launch_spec<2048>(ca, n, num_sms, stream); break;
        default: e = fs_launch_spec<4096>(ca, n, num_sms, stream); break;
      }
      launches++;
      if (e != cudaSuccess) return e;
    }
  }
  if (nlaunch) *nlaunch = launches;
  return cudaSuccess;
}

cudaError_t fs_grid_cells(const FsGrid &G, int g0, int n, double *cells, cudaStream_t stream) {
  fs_grid_cells_kernel<<<(n + 255) / 256, 256, 0, stream>>>(G, g0, n, cells);
  return cudaGetLastError();
}

cudaError_t fs_scan_mark(const double *logl0, int n, int *count, int *active, int *pos, cudaStream_t stream) {
  fs_scan_mark_kernel<<<(n + 255) / 256, 256, 0, stream>>>(logl0, n, count, active, pos);
  return cudaGetLastError();
}

cudaError_t fs_scan_cells(const FsGrid &G, const int *active, int c0, int n, const double *fdot_tab, double *cells,
                          cudaStream_t stream) {
  fs_scan_cells_kernel<<<(n + 255) / 256, 256, 0, stream>>>(G, active, c0, n, fdot_tab, cells);
  return cudaGetLastError();
}

cudaError_t fs_finalize(const double *logl0, const int *pos, const double *scan, int n, double *tensor,
                        cudaStream_t stream) {
  fs_finalize_kernel<<<(n + 255) / 256, 256, 0, stream>>>(logl0, pos, scan, n, tensor);
  return cudaGetLastError();
}

}  // namespace glass
