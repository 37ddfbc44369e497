/*
 * glass_oracle_noise.c -- CPU restatement of the GLASS noise-model likelihood
 * (the noise module's instrument and galactic-foreground covariance and its
 * XYZ Gaussian likelihood).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the CUDA noise likelihood, called
 * from tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.  The
 * product library never links it.  Pinned to the reference's own functions
 * through tests/golden/noise.npz (tests/golden/make_golden.py).
 *
 * Same order of operations as the reference where it matters for rounding.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_CLIGHT 299792458.
#define ORC_PI2 6.283185307179586
#define ORC_LARM 2.5e9

/* utils/src/glass_lisa.c:1258-1262 */
static double orc_noise_transfer_function(double x)
{
    double sinx = sin(x);
    return sinx * sinx;
}

/* utils/src/glass_galaxy.c:40-44 */
static double orc_galaxy_foreground(double f, double A, double f1, double alpha, double fk, double f2)
{
    return A * pow(f, -7. / 3.) * exp(-pow(f / f1, alpha)) * 0.5 * (1. + tanh((fk - f) / f2));
}

/* Covariance of one bin (the instrument part of
 * noise/src/glass_noise_model.c:389-546 and the foreground of :612-654). */
static void orc_noise_cov_bin(double f, const double *sacc, const double *soms, int gal, double Amp, double f1,
                              double alpha, double fk, double f2, double C[3][3])
{
    const double fstar = ORC_CLIGHT / (2.0 * M_PI * ORC_LARM);
    const double acc_units = 2.81837551648e-19;
    const double oms_units = 4.39256635604e-16;
    const double acc_fmax = 0.01;
    const double s12 = sacc[0], s21 = sacc[1], s23 = sacc[2], s32 = sacc[3], s13 = sacc[4], s31 = sacc[5];
    const double o12 = soms[0], o21 = soms[1], o23 = soms[2], o32 = soms[3], o13 = soms[4], o31 = soms[5];
    memset(C, 0, 9 * sizeof(double));
    if (f != 0.0) {
        double x = f / fstar, f2f = f * f;
        double cosx = cos(x);
        double tdi = orc_noise_transfer_function(x);
        double acc_tf = 0.0;
        if (f < acc_fmax) acc_tf = acc_units / f2f * (1.0 + pow(0.4e-3 / f, 2)) * (1.0 + pow(f / 8.0e-3, 4));
        double oms_tf = oms_units * f2f * (1.0 + pow(2.0e-3 / f, 4));
        tdi *= -8.0;
        double A12 = 0, A21 = 0, A23 = 0, A32 = 0, A13 = 0, A31 = 0;
        if (f < acc_fmax) {
            A12 = s12 * acc_tf; A21 = s21 * acc_tf; A23 = s23 * acc_tf;
            A32 = s32 * acc_tf; A13 = s13 * acc_tf; A31 = s31 * acc_tf;
        }
        double O12 = o12 * oms_tf, O21 = o21 * oms_tf, O23 = o23 * oms_tf;
        double O32 = o32 * oms_tf, O13 = o13 * oms_tf, O31 = o31 * oms_tf;
        double c00 = 0., c11 = 0., c22 = 0., c01 = 0., c02 = 0., c12 = 0.;
        c00 += (O12 + O21 + O13 + O31) * .25;
        c11 += (O23 + O32 + O21 + O12) * .25;
        c22 += (O31 + O13 + O32 + O23) * .25;
        c01 += (O12 + O21) * .5;
        c02 += (O13 + O31) * .5;
        c12 += (O32 + O23) * .5;
        if (f < acc_fmax) {
            c00 += ((A12 + A13) + ((A21 + A31)) * cosx * cosx);
            c11 += ((A23 + A21) + ((A32 + A12)) * cosx * cosx);
            c22 += ((A31 + A32) + ((A13 + A23)) * cosx * cosx);
            c01 += 2. * (A12 + A21);
            c02 += 2. * (A13 + A31);
            c12 += 2. * (A32 + A23);
        }
        c00 *= -2. * tdi;
        c11 *= -2. * tdi;
        c22 *= -2. * tdi;
        c01 *= tdi * cosx;
        c02 *= tdi * cosx;
        c12 *= tdi * cosx;
        C[0][0] = c00 / 4.0; C[1][1] = c11 / 4.0; C[2][2] = c22 / 4.0;
        C[0][1] = C[1][0] = c01 / 4.0;
        C[0][2] = C[2][0] = c02 / 4.0;
        C[1][2] = C[2][1] = c12 / 4.0;
        if (gal) {
            double fs = ORC_CLIGHT / (ORC_PI2 * ORC_LARM);
            double xg = f / fs;
            double t = 4. * xg * xg * sin(xg) * sin(xg);
            double Sgal = (f > f1 * 10) ? 0.0 : orc_galaxy_foreground(f, Amp, f1, alpha, fk, f2);
            double d = t * Sgal / 4.0, o = -0.5 * t * Sgal / 4.0;
            C[0][0] += d; C[1][1] += d; C[2][2] += d;
            C[0][1] += o; C[0][2] += o; C[1][2] += o;
            C[1][0] += o; C[2][0] += o; C[2][1] += o;
        }
    }
}

/* ------------------------------------------- one- and two-channel forms */
/* The instrument covariance of generate_instrument_noise_model's case 1
 * (Michelson X: XYZnoise_FF) and case 2 (A, E: AEnoise_FF;
 * utils/src/glass_lisa.c:1121-1145) with the link levels sacc12, soms12
 * (noise/src/glass_noise_model.c:450-461), normalised by 4; plus the
 * foreground's case 1 / case 2 (:635-641) added as
 * generate_full_covariance_matrix does; the diagonal inverse
 * (invert_noise_covariance_matrix, utils/src/glass_math.c:248-258) and
 * noise_log_likelihood (noise/src/glass_noise_model.c:1104-1134).  d0 = X
 * (one channel) or A, d1 = E; 2 N doubles each; f = fmin + n/T > 0. */
double orc_noise_logl_ch(int nch, double T, double fmin, int N, const double *d0, const double *d1,
                         const double *sacc, const double *soms, const double *sgal)
{
    const double fstar = ORC_CLIGHT / (2.0 * M_PI * ORC_LARM);
    const double acc_units = 2.81837551648e-19;
    const double oms_units = 4.39256635604e-16;
    const double acc_fmax = 0.01;
    double Amp = 0, f1 = 0, alpha = 0, fk = 0, f2g = 0;
    if (sgal) {
        Amp = exp(sgal[0]); f1 = exp(sgal[1]); alpha = sgal[2]; fk = exp(sgal[3]); f2g = exp(sgal[4]);
    }
    double *C = malloc(sizeof(double) * (size_t)N);
    for (int n = 0; n < N; n++) {
        double f = fmin + (double)n / T;
        double x = f / fstar, f2 = f * f;
        double acc_tf = (f < acc_fmax) ? acc_units / f2 * (1.0 + pow(0.4e-3 / f, 2)) * (1.0 + pow(f / 8.0e-3, 4)) : 0.0;
        double oms_tf = oms_units * f2 * (1.0 + pow(2.0e-3 / f, 4));
        double Spm = sacc[0] * acc_tf, Sop = soms[0] * oms_tf;
        double cosx = cos(x), c;
        if (nch == 1)
            c = 16. * orc_noise_transfer_function(x) * (2. * (1.0 + cosx * cosx) * Spm + Sop);
        else
            c = 8. * orc_noise_transfer_function(x) * (2. * Spm * (3. + 2. * cosx + cos(2. * x)) + Sop * (2. + cosx));
        c /= 4.0;
        if (sgal) {
            double fs = ORC_CLIGHT / (ORC_PI2 * ORC_LARM);
            double xg = f / fs;
            double t = 4. * xg * xg * sin(xg) * sin(xg);
            double Sgal = (f > f1 * 10) ? 0.0 : orc_galaxy_foreground(f, Amp, f1, alpha, fk, f2g);
            c += (nch == 1 ? Sgal : 1.5 * t * Sgal) / 4.0;
        }
        C[n] = c;
    }
    double logL = 0.0;
    for (int ch = 0; ch < nch; ch++) {
        const double *d = ch == 0 ? d0 : d1;
        double arg = 0.0;
        for (int n = 0; n < N; n++) arg += (d[2 * n] * d[2 * n] + d[2 * n + 1] * d[2 * n + 1]) * (1. / C[n]);
        logL += -0.5 * (2.0 * arg);
    }
    for (int n = 0; n < N; n++) logL -= (nch == 2) ? log(C[n]) + log(C[n]) : log(C[n]);
    free(C);
    return logL;
}

void orc_noise_logl_ch_batch(int nch, double T, double fmin, int N, const double *d0, const double *d1, int nprop,
                             const double *inst, const double *sgal, double *logl)
{
    for (int p = 0; p < nprop; p++)
        logl[p] = orc_noise_logl_ch(nch, T, fmin, N, d0, d1, inst + 12 * (size_t)p, inst + 12 * (size_t)p + 6,
                                    sgal ? sgal + 5 * (size_t)p : NULL);
}

/* ------------------------------------------------------- natural splines */
/* spline_coefficients (utils/src/glass_math.c:98-178): natural cubic spline
 * through (x[i], y[i]), i < n, coefficients c0..c3 of interval i. */
static void orc_nat_spline(int n, const double *x, const double *y, double *c0, double *c1, double *c2, double *c3)
{
    double *h = calloc(n, sizeof(double)), *al = calloc(n, sizeof(double));
    double *l = calloc(n, sizeof(double)), *z = calloc(n, sizeof(double)), *mu = calloc(n, sizeof(double));
    h[0] = x[1] - x[0];
    for (int i = 1; i < n - 1; i++) {
        h[i] = x[i + 1] - x[i];
        al[i] = 3.0 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1]);
    }
    l[0] = l[n - 1] = 1.0;
    for (int i = 1; i < n - 1; i++) {
        l[i] = 2.0 * (x[i + 1] - x[i - 1]) - h[i - 1] * mu[i - 1];
        mu[i] = h[i] / l[i];
        z[i] = (al[i] - h[i - 1] * z[i - 1]) / l[i];
    }
    c0[n - 1] = y[n - 1];
    c1[n - 1] = c2[n - 1] = c3[n - 1] = 0.0;
    for (int i = n - 2; i >= 0; i--) {
        c0[i] = y[i];
        c2[i] = z[i] - mu[i] * c2[i + 1];
        c1[i] = (c0[i + 1] - c0[i]) / h[i] - h[i] * (c2[i + 1] + 2.0 * c2[i]) / 3.0;
        c3[i] = (c2[i + 1] - c2[i]) / (3.0 * h[i]);
    }
    free(h); free(al); free(l); free(z); free(mu);
}

/* binary_search (utils/src/glass_math.c:443-473) on distinct knots: the
 * largest i with x[i] <= v (0 below the first knot, where the reference's
 * lookup is undefined). */
static int orc_knot_below(int n, const double *x, double v)
{
    int lo = 0, hi = n - 1;
    if (v <= x[0]) return 0;
    if (v >= x[n - 1]) return n - 1;
    while (hi - lo > 1) {
        int mid = (lo + hi) / 2;
        if (x[mid] <= v) lo = mid; else hi = mid;
    }
    return lo;
}

/* ----------------------------------------------------- spline noise model */
/* The noise module's one- and two-channel spline noise model for one model:
 * per channel c the natural cubic spline through the control points
 * (kf[k], kC[c K + k]), k < K, evaluated at f = fmin + n/T with the
 * binary-search lookup (CubicSplineGLASS, utils/src/glass_math.c:855-868),
 * plus transfer[n] (generate_spline_noise_model,
 * noise/src/glass_noise_model.c:366-387), inverted per channel
 * (invert_noise_covariance_matrix's one- and two-channel branches,
 * utils/src/glass_math.c:248-258), and noise_log_likelihood
 * (noise/src/glass_noise_model.c:1104-1134): -1/2 fourier_nwip per channel
 * minus the log-determinants.  d0, d1: 2 NFFT doubles (X; or A, E). */
double orc_spline_noise_logl(int nch, int NFFT, double T, double fmin, const double *d0, const double *d1,
                             const double *transfer, int K, const double *kf, const double *kC)
{
    double *c0 = malloc(sizeof(double) * K), *c1 = malloc(sizeof(double) * K);
    double *c2 = malloc(sizeof(double) * K), *c3 = malloc(sizeof(double) * K);
    double *C = malloc(sizeof(double) * (size_t)nch * NFFT);
    for (int c = 0; c < nch; c++) {
        orc_nat_spline(K, kf, kC + (size_t)c * K, c0, c1, c2, c3);
        for (int n = 0; n < NFFT; n++) {
            double f = fmin + (double)n / T;
            int j = orc_knot_below(K, kf, f);
            double d = f - kf[j];
            C[(size_t)c * NFFT + n] = (c0[j] + c1[j] * d + c2[j] * d * d + c3[j] * d * d * d) + transfer[n];
        }
    }
    double logL = 0.0;
    for (int c = 0; c < nch; c++) {
        const double *dd = c == 0 ? d0 : d1;
        double arg = 0.0;
        for (int n = 0; n < NFFT; n++) {
            double product = dd[2 * n] * dd[2 * n] + dd[2 * n + 1] * dd[2 * n + 1];
            arg += product * (1. / C[(size_t)c * NFFT + n]);
        }
        logL += -0.5 * (2.0 * arg);
    }
    for (int n = 0; n < NFFT; n++) {
        double ld = log(C[n]);
        if (nch == 2) ld += log(C[(size_t)NFFT + n]);
        logL -= ld;
    }
    free(c0); free(c1); free(c2); free(c3); free(C);
    return logL;
}

/* Batched: knots kf[p kmax + k], kC[(p nch + c) kmax + k], k < nknots[p]. */
void orc_spline_noise_logl_batch(int nch, int NFFT, double T, double fmin, const double *d0, const double *d1,
                                 const double *transfer, int nprop, int kmax, const int *nknots, const double *kf,
                                 const double *kC, double *logl)
{
    double *cc = malloc(sizeof(double) * (size_t)nch * kmax);
    for (int p = 0; p < nprop; p++) {
        int K = nknots[p];
        for (int c = 0; c < nch; c++)
            memcpy(cc + (size_t)c * K, kC + ((size_t)p * nch + c) * kmax, sizeof(double) * K);
        logl[p] = orc_spline_noise_logl(nch, NFFT, T, fmin, d0, d1, transfer, K, kf + (size_t)p * kmax, cc);
    }
    free(cc);
}

/* ------------------------------------------------------------------ SGWB */
/* utils/src/glass_constants.h:81-86 */
#define ORC_H0 (70 * 3.24078e-20)
#define ORC_HSCALE (3 * ORC_H0 * ORC_H0 / (4 * M_PI * M_PI))
#define ORC_CGOR0 (1.6e-5 / (0.7 * 0.7))

/* glass_erfc (utils/src/glass_math.c:1310-1320): Abramowitz & Stegun 7.1.26 */
static double orc_erfc(double x)
{
    double ax = fabs(x);
    double t = 1.0 / (1.0 + 0.3275911 * ax);
    double poly = ((((1.061405429 * t - 1.453152027) * t + 1.421413741) * t - 0.284496736) * t + 0.254829592) * t;
    double y = poly * exp(-ax * ax);
    return (x < 0.0) ? (2.0 - y) : y;
}

/* sgwb_powerlaw, sgwb_lognormal, sgwb_phase_transition
 * (noise/src/glass_noise_model.c:725-776), in their operation order */
double orc_sgwb_psd(int type, double f, const double *p)
{
    double prefactor = ORC_HSCALE / (f * f * f);
    if (type == 0) {
        double A = pow(10.0, p[0]);
        return prefactor * A * pow(f / 25.0, p[1]);
    }
    if (type == 1) {
        double A = pow(10.0, p[0]), fst = pow(10.0, p[1]), D = pow(10.0, p[2]);
        double ft = f / fst;
        if (D < 9.0) {
            double logft = log(ft);
            double logK = logft + 1.5 * D * D;
            double sqrtpi = sqrt(M_PI);
            double half_log32 = 0.5 * log(1.5);
            double D2 = D * D;
            double t1 = 4.0 / 5.0 / sqrtpi * ft * ft * ft * exp(9.0 * D2 / 4.0) / D *
                        ((logK * logK + 0.5 * D2) * orc_erfc((logK + half_log32) / D) -
                         D / sqrtpi * exp(-(logK + half_log32) * (logK + half_log32) / D2) * (logK - half_log32));
            double t2 = 0.0659 / D2 * ft * ft * exp(D2) *
                        exp(-(logft + D2 - 0.5 * log(4.0 / 3.0)) * (logft + D2 - 0.5 * log(4.0 / 3.0)) / D2);
            double t3 = (1.0 / 3.0) * sqrt(2.0) / sqrtpi * pow(ft, -4) * exp(8.0 * D2) / D *
                        exp(-logft * logft / (2.0 * D2)) * orc_erfc((4.0 * D2 - logft + log(4.0)) / (D * sqrt(2.0)));
            return prefactor * ORC_CGOR0 * A * A * (t1 + t2 + t3);
        }
        return prefactor * ORC_CGOR0 * A * A * 0.783 / 1e3;
    }
    double rb = p[0], b = p[1], Ap = pow(10.0, p[2]), fp = pow(10.0, p[3]);
    double rb4 = rb * rb * rb * rb;
    double m = (9 * rb4 + b) / (rb4 + 1);
    double sv = f / fp;
    double s4 = sv * sv * sv * sv;
    double s9 = s4 * s4 * sv;
    double M = s9 * pow((1 + rb4) / (rb4 + s4), (9 - b) / 4) * pow((b + 4) / (b + 4 - m + m * sv * sv), (b + 4) / 2);
    return Ap * M * prefactor;
}

/* The response R6[e N + n] (xx, yy, zz, xy, xz, yz) at f[n]: natural cubic
 * splines over log f of log XX, log YY, log ZZ and asinh(XY / 1e-7), ...
 * (alloc_pop_sgwb_response, noise/src/glass_noise_model.c:134-189), evaluated
 * as generate_sgwb_model does (:808-820); 0 at f = 0.  resp[7 i ..] = f, XX,
 * YY, ZZ, XY, XZ, YZ. */
void orc_sgwb_response(int nresp, const double *resp, int N, const double *f, double *R6)
{
    const double ascale = 1e-7;
    double *x = malloc(sizeof(double) * nresp), *y = malloc(sizeof(double) * nresp);
    double *h = calloc(nresp, sizeof(double)), *al = calloc(nresp, sizeof(double));
    double *l = calloc(nresp, sizeof(double)), *z = calloc(nresp, sizeof(double)), *mu = calloc(nresp, sizeof(double));
    double *c0 = malloc(sizeof(double) * nresp), *c1 = malloc(sizeof(double) * nresp);
    double *c2 = malloc(sizeof(double) * nresp), *c3 = malloc(sizeof(double) * nresp);
    for (int i = 0; i < nresp; i++) x[i] = log(resp[7 * i]);
    for (int e = 0; e < 6; e++) {
        for (int i = 0; i < nresp; i++) {
            double v = resp[7 * i + 1 + e];
            y[i] = e < 3 ? log(v) : asinh(v / ascale);
        }
        /* spline_coefficients (utils/src/glass_math.c:98-178) */
        h[0] = x[1] - x[0];
        for (int i = 1; i < nresp - 1; i++) {
            h[i] = x[i + 1] - x[i];
            al[i] = 3.0 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1]);
        }
        l[0] = l[nresp - 1] = 1.0;
        mu[0] = z[0] = 0.0;
        for (int i = 1; i < nresp - 1; i++) {
            l[i] = 2.0 * (x[i + 1] - x[i - 1]) - h[i - 1] * mu[i - 1];
            mu[i] = h[i] / l[i];
            z[i] = (al[i] - h[i - 1] * z[i - 1]) / l[i];
        }
        c0[nresp - 1] = y[nresp - 1];
        c1[nresp - 1] = c2[nresp - 1] = c3[nresp - 1] = 0.0;
        for (int i = nresp - 2; i >= 0; i--) {
            c0[i] = y[i];
            c2[i] = z[i] - mu[i] * c2[i + 1];
            c1[i] = (c0[i + 1] - c0[i]) / h[i] - h[i] * (c2[i + 1] + 2.0 * c2[i]) / 3.0;
            c3[i] = (c2[i + 1] - c2[i]) / (3.0 * h[i]);
        }
        for (int n = 0; n < N; n++) {
            if (f[n] == 0.0) {
                R6[(size_t)e * N + n] = 0.0;
                continue;
            }
            double v = log(f[n]);
            /* even_sampled_search (utils/src/glass_math.c:393-402) */
            int j = (int)floor((v - x[0]) / (x[1] - x[0]));
            if (j < 0) j = 0;
            if (j > nresp - 1) j = nresp - 1;
            double d = v - x[j];
            double s = c0[j] + c1[j] * d + c2[j] * d * d + c3[j] * d * d * d;
            R6[(size_t)e * N + n] = e < 3 ? exp(s) : ascale * sinh(s);
        }
    }
    free(x); free(y); free(h); free(al); free(l); free(z); free(mu);
    free(c0); free(c1); free(c2); free(c3);
}

/*
 * One noise model on the XYZ frequency grid f_n = fmin + n/T, n < N:
 *  - instrument covariance (noise/src/glass_noise_model.c:389-546, three
 *    channels): link levels sacc[6], soms[6] in the reference's array order
 *    (12, 21, 23, 32, 13, 31; :24-44);
 *  - plus, if sgal is given, the galactic foreground (:612-654 with
 *    map_array_to_foreground_params :67-74), added entry by entry
 *    (generate_full_covariance_matrix :894-907);
 *  - inverse and log-determinant (utils/src/glass_math.c:240-289, the
 *    three-channel branch with signed_log_div :236-238);
 *  - my_noise_log_likelihood (noise/src/glass_noise_model.c:1243-1273).
 * X, Y, Z: 2N doubles each (re/im).  Returns logL.
 */
double orc_noise_logl_sgwb(double T, double fmin, int N, const double *X, const double *Y, const double *Z,
                           const double *sacc, const double *soms, const double *sgal, int sg_type,
                           const double *sgwb, const double *R6);

double orc_noise_logl(double T, double fmin, int N, const double *X, const double *Y, const double *Z,
                      const double *sacc, const double *soms, const double *sgal)
{
    return orc_noise_logl_sgwb(T, fmin, N, X, Y, Z, sacc, soms, sgal, -1, NULL, NULL);
}

/* orc_noise_logl with, when sgwb is given, the background of template
 * sg_type added last (noise_instrument_model_mcmc's order,
 * noise/src/glass_noise_sampler.c:559-568): C += R(f) S(f), the response
 * R6 (6 rows of N, orc_sgwb_response) at the grid's bins. */
double orc_noise_logl_sgwb(double T, double fmin, int N, const double *X, const double *Y, const double *Z,
                           const double *sacc, const double *soms, const double *sgal, int sg_type,
                           const double *sgwb, const double *R6)
{
    double Amp = 0, f1 = 0, alpha = 0, fk = 0, f2 = 0;
    if (sgal) {
        Amp = exp(sgal[0]);
        f1 = exp(sgal[1]);
        alpha = sgal[2];
        fk = exp(sgal[3]);
        f2 = exp(sgal[4]);
    }
    const double log2pi = log(2 * M_PI);
    double logL = 0.0;
    for (int n = 0; n < N; n++) {
        double f = fmin + (double)n / T;
        double C[3][3];
        orc_noise_cov_bin(f, sacc, soms, sgal != NULL, Amp, f1, alpha, fk, f2, C);
        double cxx = C[0][0], cyy = C[1][1], czz = C[2][2], cxy = C[0][1], cxz = C[0][2], cyz = C[1][2];
        if (sgwb && f != 0.0) {
            double S = orc_sgwb_psd(sg_type, f, sgwb);
            cxx += R6[n] * S;
            cyy += R6[(size_t)N + n] * S;
            czz += R6[2 * (size_t)N + n] * S;
            cxy += R6[3 * (size_t)N + n] * S;
            cxz += R6[4 * (size_t)N + n] * S;
            cyz += R6[5 * (size_t)N + n] * S;
        }
        double d1 = cxx;
        double d2 = cyy - cxy * cxy / d1;
        double tt = cyz - cxy * cxz / d1;
        double d3 = (czz - cxz * cxz / d1) - (tt * tt) / d2;
        double logdetC = log(d1) + log(d2) + log(d3);
#define ORC_SLD(num) copysign(exp(log(fabs(num)) - logdetC), (num))
        double ixx = ORC_SLD(cyy * czz - cyz * cyz);
        double iyy = ORC_SLD(czz * cxx - cxz * cxz);
        double izz = ORC_SLD(cxx * cyy - cxy * cxy);
        double ixy = ORC_SLD(cxz * cyz - czz * cxy);
        double ixz = ORC_SLD(cxy * cyz - cxz * cyy);
        double iyz = ORC_SLD(cxy * cxz - cxx * cyz);
#undef ORC_SLD
        double rex = X[2 * n], imx = X[2 * n + 1];
        double rey = Y[2 * n], imy = Y[2 * n + 1];
        double rez = Z[2 * n], imz = Z[2 * n + 1];
        double xx = rex * rex + imx * imx;
        double yy = rey * rey + imy * imy;
        double zz = rez * rez + imz * imz;
        double xy = rex * rey + imx * imy;
        double xz = rex * rez + imx * imz;
        double yz = rey * rez + imy * imz;
        logL -= 0.5 * xx * ixx * 2;
        logL -= 0.5 * yy * iyy * 2;
        logL -= 0.5 * zz * izz * 2;
        logL -= xy * ixy * 2;
        logL -= xz * ixz * 2;
        logL -= yz * iyz * 2;
        logL -= logdetC;
    }
    logL -= 3 * N * log2pi;
    return logL;
}

/* Batched form with the background: sgwb[4 p ..] of template sg_type. */
void orc_noise_logl_sgwb_batch(double T, double fmin, int N, const double *X, const double *Y, const double *Z,
                               int nprop, const double *inst, const double *sgal, int sg_type, const double *sgwb,
                               int nresp, const double *resp, double *logl, int nthreads)
{
    double *f = malloc(sizeof(double) * N), *R6 = malloc(sizeof(double) * 6 * (size_t)N);
    for (int n = 0; n < N; n++) f[n] = fmin + (double)n / T;
    orc_sgwb_response(nresp, resp, N, f, R6);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int p = 0; p < nprop; p++)
        logl[p] = orc_noise_logl_sgwb(T, fmin, N, X, Y, Z, inst + 12 * (size_t)p, inst + 12 * (size_t)p + 6,
                                      sgal ? sgal + 5 * (size_t)p : NULL, sg_type, sgwb + 4 * (size_t)p, R6);
    free(f);
    free(R6);
}

/* Batched form: inst[12 p ..] = sacc[6], soms[6]; sgal[5 p ..] or NULL. */
void orc_noise_logl_batch(double T, double fmin, int N, const double *X, const double *Y, const double *Z, int nprop,
                          const double *inst, const double *sgal, double *logl, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int p = 0; p < nprop; p++)
        logl[p] = orc_noise_logl(T, fmin, N, X, Y, Z, inst + 12 * (size_t)p, inst + 12 * (size_t)p + 6,
                                 sgal ? sgal + 5 * (size_t)p : NULL);
}

/* The covariance of every bin: C6[6 n ..] = xx, yy, zz, xy, xz, yz (for
 * drawing synthetic data with the model's own statistics). */
void orc_noise_covariance(double T, double fmin, int N, const double *sacc, const double *soms, const double *sgal,
                          double *C6)
{
    double Amp = 0, f1 = 0, alpha = 0, fk = 0, f2 = 0;
    if (sgal) {
        Amp = exp(sgal[0]);
        f1 = exp(sgal[1]);
        alpha = sgal[2];
        fk = exp(sgal[3]);
        f2 = exp(sgal[4]);
    }
    for (int n = 0; n < N; n++) {
        double C[3][3];
        orc_noise_cov_bin(fmin + (double)n / T, sacc, soms, sgal != NULL, Amp, f1, alpha, fk, f2, C);
        double *o = C6 + 6 * (size_t)n;
        o[0] = C[0][0]; o[1] = C[1][1]; o[2] = C[2][2]; o[3] = C[0][1]; o[4] = C[0][2]; o[5] = C[1][2];
    }
}

/* ------------------------------------------------------ wavelet domain */

/* invert_noise_covariance_matrix's three-channel branch
 * (utils/src/glass_math.c:259-286): inverse entries ixx, iyy, izz, ixy, ixz,
 * iyz and the log-determinant. */
static void orc_invert3(const double *c6, double *i6, double *logdet)
{
    double cxx = c6[0], cyy = c6[1], czz = c6[2], cxy = c6[3], cxz = c6[4], cyz = c6[5];
    double d1 = cxx;
    double d2 = cyy - cxy * cxy / d1;
    double tt = cyz - cxy * cxz / d1;
    double d3 = (czz - cxz * cxz / d1) - (tt * tt) / d2;
    double ld = log(d1) + log(d2) + log(d3);
#define ORC_SLD(num) copysign(exp(log(fabs(num)) - ld), (num))
    i6[0] = ORC_SLD(cyy * czz - cyz * cyz);
    i6[1] = ORC_SLD(czz * cxx - cxz * cxz);
    i6[2] = ORC_SLD(cxx * cyy - cxy * cxy);
    i6[3] = ORC_SLD(cxz * cyz - czz * cxy);
    i6[4] = ORC_SLD(cxy * cyz - cxz * cyy);
    i6[5] = ORC_SLD(cxy * cxz - cxx * cyz);
#undef ORC_SLD
    *logdet = ld;
}

/*
 * The noise module's coarse-grained wavelet-domain likelihood for one noise
 * model (noise/src/glass_noise_model.c:1211-1241), on layers lmin ..
 * lmin + Nlayer - 1 of an NF x NT grid (layer width df) coarsened by Q in
 * time:
 *  - instrument variance per layer: the Fourier model at the layer centre
 *    (lmin + k) df over ND = NF NT (generate_instrument_noise_model_wavelet,
 *    :561-610);
 *  - mode 1 (stationary foreground): the foreground at the layer centre with
 *    the off-diagonals' -1/2 undone, over ND (generate_galactic_foreground_
 *    model_wavelet :656-722), added as generate_full_stationary_covariance_
 *    matrix_coarse does (:983-1029: diagonal +, off-diagonal - 1/2);
 *  - mode 2 (modulated foreground): the same foreground times the modulation
 *    of coarse cell q, mod[6 Ncoarse] = XX, YY, ZZ, XY, XZ, YZ, entry by entry
 *    (generate_full_dynamic_covariance_matrix_coarse :923-981);
 *  - mode 0: instrument only;
 *  - inverse per pixel, and the per-pixel Wishart sum with the cells'
 *    sample (cross-)covariances P[6][Nlayer Ncoarse] (coarse_grain_wavelet_data
 *    :1057-1102, cell k = q + j Ncoarse), minus 3/2 Nlayer NT log 2 pi.
 * inst: sacc[6], soms[6]; sgal: 5 (unused in mode 0).
 */
double orc_noise_wavelet_logl_sgwb(int NF, int NT, double df, int lmin, int Nlayer, int Q, const double *P, int mode,
                                   const double *mod, const double *inst, const double *sgal, int sg_type,
                                   const double *sgwb, const double *R6);

double orc_noise_wavelet_logl(int NF, int NT, double df, int lmin, int Nlayer, int Q, const double *P, int mode,
                              const double *mod, const double *inst, const double *sgal)
{
    return orc_noise_wavelet_logl_sgwb(NF, NT, df, lmin, Nlayer, Q, P, mode, mod, inst, sgal, -1, NULL, NULL);
}

/* With the background (generate_sgwb_model_wavelet,
 * noise/src/glass_noise_model.c:843-892: the Fourier model at the layer
 * centre over ND, zero in the DC layer) added last to every cell's
 * covariance (:964-971, :1012-1019); R6: 6 rows of Nlayer at the layer
 * centres. */
double orc_noise_wavelet_logl_sgwb(int NF, int NT, double df, int lmin, int Nlayer, int Q, const double *P, int mode,
                                   const double *mod, const double *inst, const double *sgal, int sg_type,
                                   const double *sgwb, const double *R6)
{
    const int Ncoarse = NT / Q;
    const double inv_ND = 1.0 / (double)(NF * NT);
    const double log2pi = log(2 * M_PI);
    double Amp = 0, f1 = 0, alpha = 0, fk = 0, f2 = 0;
    if (mode) {
        Amp = exp(sgal[0]);
        f1 = exp(sgal[1]);
        alpha = sgal[2];
        fk = exp(sgal[3]);
        f2 = exp(sgal[4]);
    }
    const size_t Npix = (size_t)Nlayer * Ncoarse;
    const double *Pxx = P, *Pyy = P + Npix, *Pzz = P + 2 * Npix, *Pxy = P + 3 * Npix, *Pxz = P + 4 * Npix,
                 *Pyz = P + 5 * Npix;
    const double Qd = (double)Q;
    double logL = 0.0;
    for (int j = 0; j < Nlayer; j++) {
        const double f = (double)(lmin + j) * df;
        double Ci[3][3], Cg[3][3];
        orc_noise_cov_bin(f, inst, inst + 6, 0, 0, 0, 0, 0, 0, Ci);
        double inst6[6] = {Ci[0][0] * inv_ND, Ci[1][1] * inv_ND, Ci[2][2] * inv_ND,
                           Ci[0][1] * inv_ND, Ci[0][2] * inv_ND, Ci[1][2] * inv_ND};
        double conf6[6] = {0, 0, 0, 0, 0, 0};
        if (mode) {
            /* the foreground of generate_galactic_foreground_model alone */
            double fs = ORC_CLIGHT / (ORC_PI2 * ORC_LARM);
            double xg = f / fs;
            double t = 4. * xg * xg * sin(xg) * sin(xg);
            double Sgal = (f > f1 * 10) ? 0.0 : orc_galaxy_foreground(f, Amp, f1, alpha, fk, f2);
            memset(Cg, 0, sizeof(Cg));
            double dg = t * Sgal / 4.0, og = -0.5 * t * Sgal / 4.0;
            if (lmin + j == 0) dg = og = 0.0;
            og *= -2.0;
            conf6[0] = conf6[1] = conf6[2] = dg * inv_ND;
            conf6[3] = conf6[4] = conf6[5] = og * inv_ND;
        }
        double sg6[6] = {0, 0, 0, 0, 0, 0};
        if (sgwb && lmin + j != 0) {
            double S = orc_sgwb_psd(sg_type, f, sgwb);
            for (int e = 0; e < 6; e++) sg6[e] = R6[(size_t)e * Nlayer + j] * S * inv_ND;
        }
        for (int q = 0; q < Ncoarse; q++) {
            double c6[6], i6[6], ld;
            for (int e = 0; e < 6; e++) c6[e] = inst6[e];
            if (mode == 1) {
                c6[0] += conf6[0]; c6[1] += conf6[1]; c6[2] += conf6[2];
                c6[3] -= conf6[3] / 2.; c6[4] -= conf6[4] / 2.; c6[5] -= conf6[5] / 2.;
            } else if (mode == 2) {
                for (int e = 0; e < 6; e++) c6[e] += conf6[e] * mod[(size_t)e * Ncoarse + q];
            }
            if (sgwb)
                for (int e = 0; e < 6; e++) c6[e] += sg6[e];
            orc_invert3(c6, i6, &ld);
            size_t k = (size_t)q + (size_t)j * Ncoarse;
            double s = 0.0;
            s -= 0.5 * Qd * i6[0] * Pxx[k];
            s -= 0.5 * Qd * i6[1] * Pyy[k];
            s -= 0.5 * Qd * i6[2] * Pzz[k];
            s -= Qd * i6[3] * Pxy[k];
            s -= Qd * i6[4] * Pxz[k];
            s -= Qd * i6[5] * Pyz[k];
            s -= 0.5 * Qd * ld;
            logL += s;
        }
    }
    logL -= 0.5 * 3 * (Nlayer * NT) * log2pi;
    return logL;
}

/* The cells' sample (cross-)covariances of wavelet data on Nlayer layers
 * (coarse_grain_wavelet_data, noise/src/glass_noise_model.c:1057-1102):
 * X, Y, Z hold pixel i of layer j at i + j NT; P as above. */
void orc_noise_coarse_stats(int NT, int Nlayer, int Q, const double *X, const double *Y, const double *Z, double *P)
{
    const int Ncoarse = NT / Q;
    const size_t Npix = (size_t)Nlayer * Ncoarse;
    double invQ = 1.0 / (double)Q;
    for (int j = 0; j < Nlayer; j++)
        for (int q = 0; q < Ncoarse; q++) {
            double sxx = 0, syy = 0, szz = 0, sxy = 0, sxz = 0, syz = 0;
            for (int i = q * Q; i < (q + 1) * Q; i++) {
                size_t k = (size_t)i + (size_t)j * NT;
                double wx = X[k], wy = Y[k], wz = Z[k];
                sxx += wx * wx; syy += wy * wy; szz += wz * wz;
                sxy += wx * wy; sxz += wx * wz; syz += wy * wz;
            }
            size_t kc = (size_t)q + (size_t)j * Ncoarse;
            P[kc] = sxx * invQ; P[Npix + kc] = syy * invQ; P[2 * Npix + kc] = szz * invQ;
            P[3 * Npix + kc] = sxy * invQ; P[4 * Npix + kc] = sxz * invQ; P[5 * Npix + kc] = syz * invQ;
        }
}

void orc_noise_wavelet_logl_sgwb_batch(int NF, int NT, double df, int lmin, int Nlayer, int Q, const double *P,
                                       int mode, const double *mod, int nprop, const double *inst,
                                       const double *sgal, int sg_type, const double *sgwb, int nresp,
                                       const double *resp, double *logl, int nthreads)
{
    double *f = malloc(sizeof(double) * Nlayer), *R6 = malloc(sizeof(double) * 6 * (size_t)Nlayer);
    for (int j = 0; j < Nlayer; j++) f[j] = (double)(lmin + j) * df;
    orc_sgwb_response(nresp, resp, Nlayer, f, R6);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int p = 0; p < nprop; p++)
        logl[p] = orc_noise_wavelet_logl_sgwb(NF, NT, df, lmin, Nlayer, Q, P, mode, mod, inst + 12 * (size_t)p,
                                              sgal ? sgal + 5 * (size_t)p : NULL, sg_type, sgwb + 4 * (size_t)p, R6);
    free(f);
    free(R6);
}

void orc_noise_wavelet_logl_batch(int NF, int NT, double df, int lmin, int Nlayer, int Q, const double *P, int mode,
                                  const double *mod, int nprop, const double *inst, const double *sgal, double *logl,
                                  int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int p = 0; p < nprop; p++)
        logl[p] = orc_noise_wavelet_logl(NF, NT, df, lmin, Nlayer, Q, P, mode, mod, inst + 12 * (size_t)p,
                                         sgal ? sgal + 5 * (size_t)p : NULL);
}

/* ------------------------------------------------ the UCB sampler's noise step */

/*
 * noise_model_mcmc's likelihood change (ucb/src/glass_ucb_sampler.c:29-73,
 * Fourier, two channels) for a chain whose residual is r = data - model:
 * each channel's covariance C = 1/invC scaled by sqrt(eta eta)
 * (generate_noise_model, ucb/src/glass_ucb_model.c:336-346), inverted and its
 * log-determinant taken (utils/src/glass_math.c:253-257), then
 * logL = -fourier_nwip(r, r, invC')/2 per channel (gaussian_log_likelihood,
 * utils/src/glass_model.c:726-774) and logLnorm = -sum logdetC
 * (:788-803).  Returns (logL + logLnorm)(eta_y) - (logL + logLnorm)(eta_x).
 * rA, rE: 2 NFFT doubles.
 */
double orc_noise_eta_delta(int NFFT, const double *rA, const double *rE, const double *invCA, const double *invCE,
                           const double *eta_x, const double *eta_y)
{
    double tot[2];
    for (int w = 0; w < 2; w++) {
        const double *eta = w ? eta_y : eta_x;
        double ca = 0.0, ce = 0.0, norm = 0.0;
        for (int n = 0; n < NFFT; n++) {
            double CA = (1.0 / invCA[n]) * sqrt(eta[0] * eta[0]);
            double CE = (1.0 / invCE[n]) * sqrt(eta[1] * eta[1]);
            norm -= log(CA) + log(CE);
            double iA = 1. / CA, iE = 1. / CE;
            ca += (rA[2 * n] * rA[2 * n] + rA[2 * n + 1] * rA[2 * n + 1]) * iA;
            ce += (rE[2 * n] * rE[2 * n] + rE[2 * n + 1] * rE[2 * n + 1]) * iE;
        }
        double chi2 = 2.0 * ca + 2.0 * ce;
        tot[w] = -0.5 * chi2 + norm;
    }
    return tot[1] - tot[0];
}
