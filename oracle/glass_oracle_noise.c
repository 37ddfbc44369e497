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
double orc_noise_logl(double T, double fmin, int N, const double *X, const double *Y, const double *Z,
                      const double *sacc, const double *soms, const double *sgal)
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
