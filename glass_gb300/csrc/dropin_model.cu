// Drop-in replacements for the reference's per-source model and likelihood
// entry points, on the reference's own structures (the layouts below restate
// its headers field for field: the field order and types are the interface).
//
//   analytic_orbits           utils/src/glass_lisa.c:77-123
//   initialize_analytic_orbit utils/src/glass_lisa.c:125-134
//   map_array_to_ucb_params   ucb/src/glass_ucb_model.c:25-38
//   ucb_alignment             ucb/src/glass_ucb_waveform.c:727-736
//   add_ucb_model             ucb/src/glass_ucb_model.c:192-231
//   remove_ucb_model          ucb/src/glass_ucb_model.c:149-190
//   generate_ucb_model        ucb/src/glass_ucb_model.c:55-103
//   update_ucb_model          ucb/src/glass_ucb_model.c:271-308
//   fourier_nwip              utils/src/glass_math.c:362-380
//   snr                       utils/src/glass_math.c:403-425
//   gaussian_log_likelihood   utils/src/glass_model.c:726-774
//   matrix_eigenstuff         utils/src/glass_math.c:475-499
//   ucb_fisher                ucb/src/glass_ucb_waveform.c:364-522
//   wavelet_nwip              utils/src/glass_math.c:382-391
//   snr_wavelet               utils/src/glass_math.c:428-438
//   delta_log_likelihood      utils/src/glass_model.c:624-687
//   ucb_fisher_wavelet        ucb/src/glass_ucb_waveform.c:524-696
//
// The waveforms come from this library's GPU ucb_waveform; ucb_fisher's
// Fisher matrix for A/E data from the GPU adjoint kernels (the reference's
// eight finite-difference waveforms are not needed; its indexing of the noise
// by template bin is kept, fisher_mode 1), for X or XYZ data from forward
// differences of the GPU waveform as the reference takes them;
// ucb_fisher_wavelet's from the batched wavelet Fisher kernels
// (glass_gpu_wavelet_fisher_batch, the reference's central differences on the
// GPU waveform).  The sums over
// a segment's bins (fourier_nwip, snr, gaussian_log_likelihood, the model
// updates) work on the caller's host arrays, in the reference's order of
// operations (bit-identical): one GPU launch per call would cost more than the
// few thousand multiply-adds it replaces, and the batched engine
// (glass_gpu_dlogl_batch) is the GPU form of the whole proposal step.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "dropin.h"
#include "glass_common.cuh"

namespace {

// utils/src/glass_lisa.h:116-140
struct TDILayout {
  double *X, *Y, *Z, *A, *E, *T;
  int Nchannel;
  int N;
  double delta;
};

// utils/src/glass_data.h:337-360
struct NoiseLayout {
  int N, kmin, Nchannel, Nlayer;
  double *eta, *f;
  double ***C, ***invC;
  double *logdetC;
  double *transfer;
};

// utils/src/glass_data.h:50-97 (the fields up to the format string)
struct DataLayout {
  int N, NFFT, Nchannel, Nlayer;
  double logN;
  unsigned int cseed, nseed, iseed;
  double T, sqT, t0;
  void *wdm;
  int qmin, qmax, qpad, lmin, lmax;
  double fmin, fmax, sine_f_on_fstar;
  TDILayout *tdi, *raw, *dft, *dwt;
  NoiseLayout *noise;
  char format[16];
};

// utils/src/glass_model.h:81-121
struct SourceLayout {
  int NP;
  double *params;
  TDILayout *tdi;
  double f0, dfdt, d2fdt2, amp, psi, cosi, phiref, phi, costheta, dL, tref, m1, m2, Mchirp, Mtotal, chi1, chi2;
  int BW, qmin, qmax, imin, imax;
  double **fisher_matrix, **fisher_evectr, *fisher_evalue;
  int fisher_update_flag;
  int *list;
  int Nlist;
};

// utils/src/glass_model.h:25-60
struct ModelLayout {
  int NP, Nmax, Neff, Nlive;
  SourceLayout **source;
  NoiseLayout *noise;
  void *calibration;
  TDILayout *tdi, *residual;
  double t0;
  double **prior;
  double *logPriorVolume;
  double logL, logLnorm;
  int *list;
  int Nlist;
};

// utils/src/glass_lisa.h:60-109
struct OrbitHead {
  char OrbitFileName[1024];
  int Norb;
  double L, fstar, ecc, R, lambda_0, kappa_0;
  double *t;
  double **x, **y, **z;
  void **dx, **dy, **dz;
  void (*orbit_function)(struct Orbit *, double, double *, double *, double *);
};


constexpr int kUcbNP = 8;  // UCB_MODEL_NP, ucb/src/glass_ucb_model.h:27

int format_code(const char *f) {
  if (!strcmp(f, "sangria")) return GLASS_FMT_SANGRIA;
  if (!strcmp(f, "phase")) return GLASS_FMT_PHASE;
  if (!strcmp(f, "frequency")) return GLASS_FMT_FREQUENCY;
  return -1;
}

// One segment's noise uploaded to the calling thread's context for the
// adjoint Fisher matrix, kept while the caller's segment and noise stay the
// same (compared by value).
struct FisherBank {
  int format = -1, NFFT = 0, qmin = 0;
  double T = 0, t0 = 0;
  std::vector<double> invA, invE;
};
thread_local FisherBank g_fbank;

}  // namespace

extern "C" {

void ucb_waveform(struct Orbit *orbit, char *format, double T, double t0, double *params, int NParams, double *X,
                  double *Y, double *Z, double *A, double *E, int BW, int NI);

// Spacecraft positions of the analytic orbits (1-based arrays, as the
// reference fills them), utils/src/glass_lisa.c:77-123.
void analytic_orbits(struct Orbit *orbit, double t, double *x, double *y, double *z) {
  const OrbitHead *o = reinterpret_cast<const OrbitHead *>(orbit);
  const double alpha = glass::kPI2 * t / glass::kYEAR;
  const double sa = sin(alpha), ca = cos(alpha);
  const double sa2 = sa * sa, ca2 = ca * ca, saca = sa * ca, AUca = glass::kAU * ca, AUsa = glass::kAU * sa;
  const double sbs[3] = {0.0, 0.866025403784439, -0.866025403784438};
  const double cbs[3] = {1.0, -0.5, -0.5};
  for (int i = 0; i < 3; i++) {
    x[i + 1] = AUca + o->R * (saca * sbs[i] - (1. + sa2) * cbs[i]);
    y[i + 1] = AUsa + o->R * (saca * cbs[i] - (1. + ca2) * sbs[i]);
    z[i + 1] = -glass::kSQ3 * o->R * (ca * cbs[i] + sa * sbs[i]);
  }
}

// utils/src/glass_lisa.c:125-134
void initialize_analytic_orbit(struct Orbit *orbit) {
  OrbitHead *o = reinterpret_cast<OrbitHead *>(orbit);
  o->L = glass::kLARM;
  o->fstar = glass::kCLIGHT / (2.0 * M_PI * glass::kLARM);
  o->ecc = glass::kLARM / (2.0 * glass::kSQ3 * glass::kAU);
  o->R = glass::kAU * o->ecc;
  o->kappa_0 = 0.0;
  o->lambda_0 = 0.0;
  o->orbit_function = &analytic_orbits;
}

void map_array_to_ucb_params(struct Source *source, double *params, double T) {
  SourceLayout *s = reinterpret_cast<SourceLayout *>(source);
  s->f0 = params[0] / T;
  s->costheta = params[1];
  s->phi = params[2];
  s->amp = exp(params[3]);
  s->cosi = params[4];
  s->psi = params[5];
  s->phiref = params[6];
  s->dfdt = params[7] / (T * T);
}

void ucb_alignment(struct Orbit *orbit, struct Data *data, struct Source *source) {
  const OrbitHead *o = reinterpret_cast<const OrbitHead *>(orbit);
  const DataLayout *d = reinterpret_cast<const DataLayout *>(data);
  SourceLayout *s = reinterpret_cast<SourceLayout *>(source);
  map_array_to_ucb_params(source, s->params, d->T);
  s->BW = 2 * ucb_bandwidth(o->L, o->fstar, s->f0, s->dfdt, s->costheta, s->amp, d->T, d->NFFT);
  s->qmin = (int)(s->f0 * d->T) - s->BW / 2;
  s->qmax = s->qmin + s->BW;
  s->imin = s->qmin - d->qmin;
  s->imax = s->imin + s->BW;
}

// sign +1 adds the source's template to the model, -1 removes it
static void model_accumulate(const DataLayout *d, ModelLayout *m, const SourceLayout *s, double sign) {
  for (int i = 0; i < s->BW; i++) {
    const int j = i + s->imin;
    if (j < 0 || j >= d->NFFT) continue;
    const int ir = 2 * i, ii = ir + 1, jr = 2 * j, ji = jr + 1;
    switch (d->Nchannel) {
      case 1:
        if (sign > 0) {
          m->tdi->X[jr] += s->tdi->X[ir];
          m->tdi->X[ji] += s->tdi->X[ii];
        } else {
          m->tdi->X[jr] -= s->tdi->X[ir];
          m->tdi->X[ji] -= s->tdi->X[ii];
        }
        break;
      case 2:
        if (sign > 0) {
          m->tdi->A[jr] += s->tdi->A[ir];
          m->tdi->A[ji] += s->tdi->A[ii];
          m->tdi->E[jr] += s->tdi->E[ir];
          m->tdi->E[ji] += s->tdi->E[ii];
        } else {
          m->tdi->A[jr] -= s->tdi->A[ir];
          m->tdi->A[ji] -= s->tdi->A[ii];
          m->tdi->E[jr] -= s->tdi->E[ir];
          m->tdi->E[ji] -= s->tdi->E[ii];
        }
        break;
      case 3:
        if (sign > 0) {
          m->tdi->X[jr] += s->tdi->X[ir];
          m->tdi->X[ji] += s->tdi->X[ii];
          m->tdi->Y[jr] += s->tdi->Y[ir];
          m->tdi->Y[ji] += s->tdi->Y[ii];
          m->tdi->Z[jr] += s->tdi->Z[ir];
          m->tdi->Z[ji] += s->tdi->Z[ii];
        } else {
          m->tdi->X[jr] -= s->tdi->X[ir];
          m->tdi->X[ji] -= s->tdi->X[ii];
          m->tdi->Y[jr] -= s->tdi->Y[ir];
          m->tdi->Y[ji] -= s->tdi->Y[ii];
          m->tdi->Z[jr] -= s->tdi->Z[ir];
          m->tdi->Z[ji] -= s->tdi->Z[ii];
        }
        break;
    }
  }
}

void add_ucb_model(struct Data *data, struct Model *model, struct Source *source) {
  model_accumulate(reinterpret_cast<const DataLayout *>(data), reinterpret_cast<ModelLayout *>(model),
                   reinterpret_cast<const SourceLayout *>(source), 1.0);
}

void remove_ucb_model(struct Data *data, struct Model *model, struct Source *source) {
  model_accumulate(reinterpret_cast<const DataLayout *>(data), reinterpret_cast<ModelLayout *>(model),
                   reinterpret_cast<const SourceLayout *>(source), -1.0);
}

static void source_waveform(struct Orbit *orbit, const DataLayout *d, double t0, SourceLayout *s) {
  ucb_waveform(orbit, const_cast<char *>(d->format), d->T, t0, s->params, kUcbNP, s->tdi->X, s->tdi->Y, s->tdi->Z,
               s->tdi->A, s->tdi->E, s->BW, s->tdi->Nchannel);
}

void generate_ucb_model(struct Orbit *orbit, struct Data *data, struct Model *model, int source_id) {
  const DataLayout *d = reinterpret_cast<const DataLayout *>(data);
  ModelLayout *m = reinterpret_cast<ModelLayout *>(model);
  for (int n = 0; n < d->N; n++) m->tdi->X[n] = m->tdi->Y[n] = m->tdi->Z[n] = m->tdi->A[n] = m->tdi->E[n] = 0.0;
  for (int n = 0; n < m->Nlive; n++) {
    SourceLayout *s = m->source[n];
    if (source_id == -1 || source_id == n) {
      for (int i = 0; i < d->N; i++) s->tdi->X[i] = s->tdi->Y[i] = s->tdi->Z[i] = s->tdi->A[i] = s->tdi->E[i] = 0.0;
      map_array_to_ucb_params(reinterpret_cast<struct Source *>(s), s->params, d->T);
      ucb_alignment(orbit, data, reinterpret_cast<struct Source *>(s));
      source_waveform(orbit, d, m->t0, s);
    }
    add_ucb_model(data, model, reinterpret_cast<struct Source *>(s));
  }
}

void update_ucb_model(struct Orbit *orbit, struct Data *data, struct Model *model_x, struct Model *model_y,
                      int source_id) {
  const DataLayout *d = reinterpret_cast<const DataLayout *>(data);
  ModelLayout *mx = reinterpret_cast<ModelLayout *>(model_x), *my = reinterpret_cast<ModelLayout *>(model_y);
  SourceLayout *sx = mx->source[source_id], *sy = my->source[source_id];
  remove_ucb_model(data, model_y, reinterpret_cast<struct Source *>(sx));
  for (int i = 0; i < d->N; i++) {
    switch (d->Nchannel) {
      case 1: sy->tdi->X[i] = 0.0; break;
      case 2: sy->tdi->A[i] = sy->tdi->E[i] = 0.0; break;
      case 3: sy->tdi->X[i] = sy->tdi->Y[i] = sy->tdi->Z[i] = 0.0; break;
    }
  }
  map_array_to_ucb_params(reinterpret_cast<struct Source *>(sy), sy->params, d->T);
  ucb_alignment(orbit, data, reinterpret_cast<struct Source *>(sy));
  source_waveform(orbit, d, my->t0, sy);
  add_ucb_model(data, model_y, reinterpret_cast<struct Source *>(sy));
}

double fourier_nwip(const double *a, const double *b, const double *invC, int N) {
  double arg = 0.0;
  for (int n = 0; n < N; n++) {
    const int j = 2 * n, k = j + 1;
    const double product = a[j] * b[j] + a[k] * b[k];
    arg += product * invC[n];
  }
  return 2.0 * arg;
}

double snr(struct Source *source, struct Noise *noise) {
  const SourceLayout *s = reinterpret_cast<const SourceLayout *>(source);
  const NoiseLayout *nz = reinterpret_cast<const NoiseLayout *>(noise);
  const TDILayout *t = s->tdi;
  const int N = t->N / 2;
  double snr2 = 0.0;
  switch (t->Nchannel) {
    case 1: snr2 += fourier_nwip(t->X, t->X, nz->invC[0][0], N); break;
    case 2:
      snr2 += fourier_nwip(t->A, t->A, nz->invC[0][0], N);
      snr2 += fourier_nwip(t->E, t->E, nz->invC[1][1], N);
      break;
    case 3:
      snr2 += fourier_nwip(t->X, t->X, nz->invC[0][0], N);
      snr2 += fourier_nwip(t->Y, t->Y, nz->invC[1][1], N);
      snr2 += fourier_nwip(t->Z, t->Z, nz->invC[2][2], N);
      snr2 += fourier_nwip(t->X, t->Y, nz->invC[0][1], N) * 2.;
      snr2 += fourier_nwip(t->X, t->Z, nz->invC[0][2], N) * 2.;
      snr2 += fourier_nwip(t->Y, t->Z, nz->invC[1][2], N) * 2.;
      break;
  }
  return sqrt(snr2);
}

double gaussian_log_likelihood(struct Data *data, struct Model *model) {
  const DataLayout *d = reinterpret_cast<const DataLayout *>(data);
  ModelLayout *m = reinterpret_cast<ModelLayout *>(model);
  TDILayout *r = m->residual;
  for (int i = 0; i < d->N; i++) {
    r->X[i] = d->tdi->X[i] - m->tdi->X[i];
    r->Y[i] = d->tdi->Y[i] - m->tdi->Y[i];
    r->Z[i] = d->tdi->Z[i] - m->tdi->Z[i];
    r->A[i] = d->tdi->A[i] - m->tdi->A[i];
    r->E[i] = d->tdi->E[i] - m->tdi->E[i];
  }
  double chi2 = 0.0;
  double ***ic = m->noise->invC;
  switch (d->Nchannel) {
    case 1: chi2 += fourier_nwip(r->X, r->X, ic[0][0], d->NFFT); break;
    case 2:
      chi2 += fourier_nwip(r->A, r->A, ic[0][0], d->NFFT);
      chi2 += fourier_nwip(r->E, r->E, ic[1][1], d->NFFT);
      break;
    case 3:
      chi2 += fourier_nwip(r->X, r->X, ic[0][0], d->NFFT);
      chi2 += fourier_nwip(r->Y, r->Y, ic[1][1], d->NFFT);
      chi2 += fourier_nwip(r->Z, r->Z, ic[2][2], d->NFFT);
      chi2 += 2.0 * fourier_nwip(r->X, r->Y, ic[0][1], d->NFFT);
      chi2 += 2.0 * fourier_nwip(r->X, r->Z, ic[0][2], d->NFFT);
      chi2 += 2.0 * fourier_nwip(r->Y, r->Z, ic[1][2], d->NFFT);
      break;
    default:
      fprintf(stderr, "Unsupported number of channels in gaussian_log_likelihood()\n");
      exit(1);
  }
  return -0.5 * chi2;
}

// Eigenvalues and eigenvectors of a symmetric N x N matrix (the reference
// takes LAPACK's general solver, dgeev, on its symmetric Fisher matrices):
// cyclic Jacobi rotations (each zeroes one off-diagonal pair; sweeps until
// every off-diagonal entry is negligible against its two diagonal entries),
// eigenvector j in column j
// (evectors[i][j]), unit length.  The pairs are sorted by decreasing
// eigenvalue and each vector's largest component made positive; LAPACK's
// order and signs differ, so results compare up to order and sign.
void matrix_eigenstuff(double **matrix, double **evectors, double *evalues, int N) {
  std::vector<double> a((size_t)N * N), v((size_t)N * N);
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      a[(size_t)i * N + j] = 0.5 * (matrix[i][j] + matrix[j][i]);
      v[(size_t)i * N + j] = i == j ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 64; sweep++) {
    int rotations = 0;
    for (int p = 0; p < N; p++)
      for (int q = p + 1; q < N; q++) {
        const double apq = a[(size_t)p * N + q];
        const double app = a[(size_t)p * N + p], aqq = a[(size_t)q * N + q];
        // negligible against both diagonal entries: leaves every eigenvalue,
        // however small, at full relative accuracy
        if (!(fabs(apq) > 1e-18 * sqrt(fabs(app * aqq))) || !(fabs(apq) > 1e-300)) continue;
        rotations++;
        // rotation angle from cot 2 theta = (aqq - app) / (2 apq); the smaller root for t = tan theta
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < N; k++) {  // columns p, q
          const double akp = a[(size_t)k * N + p], akq = a[(size_t)k * N + q];
          a[(size_t)k * N + p] = c * akp - s * akq;
          a[(size_t)k * N + q] = s * akp + c * akq;
        }
        for (int k = 0; k < N; k++) {  // rows p, q
          const double apk = a[(size_t)p * N + k], aqk = a[(size_t)q * N + k];
          a[(size_t)p * N + k] = c * apk - s * aqk;
          a[(size_t)q * N + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < N; k++) {
          const double vkp = v[(size_t)k * N + p], vkq = v[(size_t)k * N + q];
          v[(size_t)k * N + p] = c * vkp - s * vkq;
          v[(size_t)k * N + q] = s * vkp + c * vkq;
        }
      }
    if (rotations == 0) break;
  }
  std::vector<int> ord(N);
  for (int j = 0; j < N; j++) ord[j] = j;
  for (int i = 1; i < N; i++)  // insertion sort, decreasing eigenvalue
    for (int j = i; j > 0 && a[(size_t)ord[j] * N + ord[j]] > a[(size_t)ord[j - 1] * N + ord[j - 1]]; j--) {
      const int t = ord[j];
      ord[j] = ord[j - 1];
      ord[j - 1] = t;
    }
  for (int j = 0; j < N; j++) {
    const int c = ord[j];
    evalues[j] = a[(size_t)c * N + c];
    int big = 0;
    for (int i = 1; i < N; i++)
      if (fabs(v[(size_t)i * N + c]) > fabs(v[(size_t)big * N + c])) big = i;
    const double sg = v[(size_t)big * N + c] < 0.0 ? -1.0 : 1.0;
    for (int i = 0; i < N; i++) evectors[i][j] = sg * v[(size_t)i * N + c];
  }
}

void ucb_fisher(struct Orbit *orbit, struct Data *data, struct Source *source, struct Noise *noise) {
  const DataLayout *d = reinterpret_cast<const DataLayout *>(data);
  SourceLayout *s = reinterpret_cast<SourceLayout *>(source);
  const NoiseLayout *nz = reinterpret_cast<const NoiseLayout *>(noise);
  double F[kUcbNP * kUcbNP];
  const int fmt = format_code(d->format);
  if (s->tdi->Nchannel == 2 && fmt >= 0 && d->NFFT >= 32 && d->NFFT <= 8192) {
    glass_gpu_ctx *ctx = dropin_ctx("ucb_fisher");
    FisherBank &B = g_fbank;
    const double *iA = nz->invC[0][0], *iE = nz->invC[1][1];
    const size_t n = (size_t)d->NFFT;
    const bool same = B.format == fmt && B.NFFT == d->NFFT && B.qmin == d->qmin && B.T == d->T && B.t0 == d->t0 &&
                      !memcmp(B.invA.data(), iA, n * sizeof(double)) && !memcmp(B.invE.data(), iE, n * sizeof(double));
    if (!same) {
      std::vector<double> zero(2 * n, 0.0);
      const int qmin = d->qmin;
      if (glass_gpu_bank_upload(ctx, fmt, d->T, d->t0, d->NFFT, 1, &qmin, zero.data(), zero.data(), iA, iE) !=
          GLASS_OK)
        dropin_fail("ucb_fisher");
      B.format = fmt;
      B.NFFT = d->NFFT;
      B.qmin = d->qmin;
      B.T = d->T;
      B.t0 = d->t0;
      B.invA.assign(iA, iA + n);
      B.invE.assign(iE, iE + n);
    }
    const int seg = 0;
    double ty, grad[kUcbNP];
    int st = 0;
    if (glass_gpu_grad_fisher_batch_host(ctx, 1, &seg, s->params, 1, &ty, grad, F, &st) != GLASS_OK)
      dropin_fail("ucb_fisher");
    if (st & GLASS_ITEM_NONFINITE)
      for (int q = 0; q < kUcbNP * kUcbNP; q++) F[q] = NAN;
  } else {
    // forward differences of the GPU waveform, step 1e-6, as the reference
    const double eps = 1.0e-6, inv = 1.0 / eps;
    const int N = d->N;
    std::vector<double> buf((size_t)5 * N), dh((size_t)kUcbNP * 3 * N, 0.0);
    double pp[kUcbNP];
    SourceLayout wp = *s;
    TDILayout tp = *s->tdi;
    tp.X = buf.data();
    tp.Y = tp.X + N;
    tp.Z = tp.Y + N;
    tp.A = tp.Z + N;
    tp.E = tp.A + N;
    wp.tdi = &tp;
    wp.params = pp;
    int BW = 0;
    for (int i = 0; i < kUcbNP; i++) {
      for (int j = 0; j < kUcbNP; j++) pp[j] = s->params[j];
      pp[i] += eps;
      if ((i == 1 || i == 4) && pp[i] > 1.0) pp[i] = 1.0;
      map_array_to_ucb_params(reinterpret_cast<struct Source *>(&wp), pp, d->T);
      std::fill(buf.begin(), buf.end(), 0.0);
      ucb_alignment(orbit, data, reinterpret_cast<struct Source *>(&wp));
      source_waveform(orbit, d, d->t0, &wp);
      BW = wp.BW;
      double *o = dh.data() + (size_t)i * 3 * N;
      for (int k = 0; k < 2 * BW; k++) {
        switch (s->tdi->Nchannel) {
          case 1: o[k] = (tp.X[k] - s->tdi->X[k]) * inv; break;
          case 2:
            o[k] = (tp.A[k] - s->tdi->A[k]) * inv;
            o[N + k] = (tp.E[k] - s->tdi->E[k]) * inv;
            break;
          default:
            o[k] = (tp.X[k] - s->tdi->X[k]) * inv;
            o[N + k] = (tp.Y[k] - s->tdi->Y[k]) * inv;
            o[2 * N + k] = (tp.Z[k] - s->tdi->Z[k]) * inv;
        }
      }
    }
    double ***ic = nz->invC;
    for (int i = 0; i < kUcbNP; i++)
      for (int j = i; j < kUcbNP; j++) {
        const double *xi = dh.data() + (size_t)i * 3 * N, *xj = dh.data() + (size_t)j * 3 * N;
        double f;
        if (s->tdi->Nchannel == 1) {
          f = fourier_nwip(xi, xj, ic[0][0], BW);
        } else if (s->tdi->Nchannel == 2) {
          f = fourier_nwip(xi, xj, ic[0][0], BW);
          f += fourier_nwip(xi + N, xj + N, ic[1][1], BW);
        } else {
          f = fourier_nwip(xi, xj, ic[0][0], BW);
          f += fourier_nwip(xi + N, xj + N, ic[1][1], BW);
          f += fourier_nwip(xi + 2 * N, xj + 2 * N, ic[2][2], BW);
          f += fourier_nwip(xi, xj + N, ic[0][1], BW);
          f += fourier_nwip(xi, xj + 2 * N, ic[0][2], BW);
          f += fourier_nwip(xi + N, xj + 2 * N, ic[1][2], BW);
          f += fourier_nwip(xi + N, xj, ic[1][0], BW);
          f += fourier_nwip(xi + 2 * N, xj, ic[2][0], BW);
          f += fourier_nwip(xi + 2 * N, xj + N, ic[2][1], BW);
        }
        F[i * kUcbNP + j] = F[j * kUcbNP + i] = f;
      }
  }
  for (int i = 0; i < kUcbNP; i++)
    for (int j = i; j < kUcbNP; j++) {
      double f = F[i * kUcbNP + j];
      if (f != f) {  // ucb/src/glass_ucb_waveform.c:500-510
        fprintf(stderr, "WARNING: nan matrix element in ucb_fisher (GB300), fisher_matrix[%i][%i]\n", i, j);
        f = 10.0;
      }
      s->fisher_matrix[i][j] = s->fisher_matrix[j][i] = f;
    }
  matrix_eigenstuff(s->fisher_matrix, s->fisher_evectr, s->fisher_evalue, kUcbNP);
}

double wavelet_nwip(const double *a, const double *b, const double *invC, const int *list, int N) {
  double arg = 0.0;
  for (int n = 0; n < N; n++) {
    const int k = list[n];
    arg += a[k] * b[k] * invC[k];
  }
  return arg;
}

double snr_wavelet(struct Source *source, struct Noise *noise) {
  const SourceLayout *s = reinterpret_cast<const SourceLayout *>(source);
  double ***ic = reinterpret_cast<const NoiseLayout *>(noise)->invC;
  const TDILayout *t = s->tdi;
  const int *l = s->list, n = s->Nlist;
  double snr2 = 0.0;
  snr2 += wavelet_nwip(t->X, t->X, ic[0][0], l, n);
  snr2 += wavelet_nwip(t->Y, t->Y, ic[1][1], l, n);
  snr2 += wavelet_nwip(t->Z, t->Z, ic[2][2], l, n);
  snr2 += wavelet_nwip(t->X, t->Y, ic[0][1], l, n) * 2;
  snr2 += wavelet_nwip(t->X, t->Z, ic[0][2], l, n) * 2;
  snr2 += wavelet_nwip(t->Y, t->Z, ic[1][2], l, n) * 2;
  return sqrt(snr2);
}

}  // extern "C"

namespace {
// The nine XYZ cross terms of (a|h) over a pixel list, in the reference's
// order: XX, YY, ZZ, XY, XZ, YZ, YX, ZX, ZY (utils/src/glass_model.c:641-683).
double xyz_nwip9(const TDILayout *a, const TDILayout *h, double ***ic, const int *l, int n) {
  double r = 0.0;
  r += wavelet_nwip(a->X, h->X, ic[0][0], l, n);
  r += wavelet_nwip(a->Y, h->Y, ic[1][1], l, n);
  r += wavelet_nwip(a->Z, h->Z, ic[2][2], l, n);
  r += wavelet_nwip(a->X, h->Y, ic[0][1], l, n);
  r += wavelet_nwip(a->X, h->Z, ic[0][2], l, n);
  r += wavelet_nwip(a->Y, h->Z, ic[1][2], l, n);
  r += wavelet_nwip(a->Y, h->X, ic[1][0], l, n);
  r += wavelet_nwip(a->Z, h->X, ic[2][0], l, n);
  r += wavelet_nwip(a->Z, h->Y, ic[2][1], l, n);
  return r;
}
}  // namespace

extern "C" {

// The sparse-pixel likelihood difference of two wavelet-domain models: each
// model's (d|h) and (h|h) over its own pixel list with its own noise; the
// (d|d) terms cancel.
double delta_log_likelihood(struct Data *data, struct Model *model_x, struct Model *model_y) {
  const DataLayout *d = reinterpret_cast<const DataLayout *>(data);
  const ModelLayout *mx = reinterpret_cast<const ModelLayout *>(model_x);
  const ModelLayout *my = reinterpret_cast<const ModelLayout *>(model_y);
  double ***icx = mx->noise->invC, ***icy = my->noise->invC;
  const double dh_x = xyz_nwip9(d->tdi, mx->tdi, icx, mx->list, mx->Nlist);
  const double hh_x = xyz_nwip9(mx->tdi, mx->tdi, icx, mx->list, mx->Nlist);
  const double dh_y = xyz_nwip9(d->tdi, my->tdi, icy, my->list, my->Nlist);
  const double hh_y = xyz_nwip9(my->tdi, my->tdi, icy, my->list, my->Nlist);
  const double logLx = -0.5 * (hh_x - 2.0 * dh_x);
  const double logLy = -0.5 * (hh_y - 2.0 * dh_y);
  return logLy - logLx;
}

// The wavelet-domain Fisher matrix of one source: the batched GPU kernels
// (central differences of the FP64 wavelet waveform with the reference's step
// and clamping, the nine XYZ cross terms per pixel inside the time window
// imin < t < imax), then the eigen-decomposition, and the reference's
// regularisation when an eigenvalue is not positive: 0.1 added to the
// diagonal and the decomposition redone; still not positive: report, exit.
void ucb_fisher_wavelet(struct Orbit *orbit, struct Data *data, struct Source *source, struct Noise *noise) {
  static const char *who = "ucb_fisher_wavelet";
  const DataLayout *d = reinterpret_cast<const DataLayout *>(data);
  SourceLayout *s = reinterpret_cast<SourceLayout *>(source);
  const NoiseLayout *nz = reinterpret_cast<const NoiseLayout *>(noise);
  struct Wavelets *wdm = reinterpret_cast<struct Wavelets *>(d->wdm);
  const WaveletsLayout *w = reinterpret_cast<const WaveletsLayout *>(d->wdm);
  const int N = w->kmax - w->kmin;
  if (N != d->N) {
    fprintf(stderr, "%s: data->N (%d) is not the grid's kmax - kmin (%d)\n", who, d->N, N);
    exit(1);
  }
  glass_gpu_ctx *ctx = dropin_wavelet_grid(orbit, wdm, d->T, d->t0, who);
  // the noise the Fisher matrix is weighted with, as invC[(3 i + j) N + k]
  thread_local std::vector<double> resid, icv;
  resid.assign((size_t)3 * N, 0.0);
  icv.resize((size_t)9 * N);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) memcpy(&icv[(size_t)(3 * i + j) * N], nz->invC[i][j], sizeof(double) * (size_t)N);
  if (glass_gpu_wavelet_set_data(ctx, resid.data(), resid.data() + N, resid.data() + 2 * N, icv.data()) != GLASS_OK)
    dropin_fail(who);
  double F[kUcbNP * kUcbNP];
  int st = 0;
  if (glass_gpu_wavelet_fisher_batch_host(ctx, 1, s->params, w->imin, w->imax, F, &st) != GLASS_OK)
    dropin_fail(who);
  if (st != 0) {
    fprintf(stderr, "%s: invalid perturbed parameters (status %d)\n", who, st);
    exit(1);
  }
  for (int i = 0; i < kUcbNP; i++)
    for (int j = 0; j < kUcbNP; j++) s->fisher_matrix[i][j] = F[i * kUcbNP + j];
  matrix_eigenstuff(s->fisher_matrix, s->fisher_evectr, s->fisher_evalue, kUcbNP);
  bool bad = false;
  for (int i = 0; i < kUcbNP; i++) {
    const double e = s->fisher_evalue[i];
    if (e <= 0 || e != e) {
      fprintf(stderr, "WARNING: bad eigenvalue in ucb_fisher_wavelet (GB300): fisher_evalue[%i] = %lg\n", i, e);
      bad = true;
    }
  }
  if (!bad) return;
  fprintf(stderr, "WARNING: try regularization FIM and re-inverting\n");
  for (int i = 0; i < kUcbNP; i++) s->fisher_matrix[i][i] += 1.0e-1;
  matrix_eigenstuff(s->fisher_matrix, s->fisher_evectr, s->fisher_evalue, kUcbNP);
  for (int i = 0; i < kUcbNP; i++) {
    const double e = s->fisher_evalue[i];
    if (e <= 0 || e != e) {
      fprintf(stderr, "ERROR: bad eigenvalue in ucb_fisher_wavelet (GB300): fisher_evalue[%i] = %lg\n", i, e);
      exit(1);
    }
  }
}

}  // extern "C"
