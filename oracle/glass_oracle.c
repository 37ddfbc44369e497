/*
 * glass_oracle.c -- CPU restatement of the GLASS UCB likelihood path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA path is checked
 * against; it is called from tests/, from __graft_entry__.smoke() and from the
 * CPU-baseline leg of bench.py, and from nowhere else.  The product library
 * (glass_gb300/csrc) never links or calls it.
 *
 * Pinning: every function here is compared against the reference's own code
 * (compiled from its sources into oracle/_ref by Makefile.ref) through the
 * golden vectors in tests/golden/, which tests/golden/make_golden.py
 * generates from oracle/_ref.
 *
 * Arithmetic is IEEE double throughout, in the same order of operations as the
 * reference where that order matters for rounding; the FFT is a plain iterative
 * radix-2 transform (the reference uses kissfft, external/kissfft/kiss_fft.c,
 * which gives the same transform to rounding).
 *
 * Array conventions (same as the reference): complex frequency series are
 * interleaved re/im doubles, 0-based.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Physical constants: utils/src/glass_constants.h:31,40,54,69,78,89 and
 * utils/src/glass_lisa.h:31.  The values must be identical to the reference's
 * because the carrier phase multiplies them by ~1e5. */
#define ORC_SQ3 1.73205080757
#define ORC_PI2 6.283185307179586
#define ORC_CLIGHT 299792458.
#define ORC_YEAR 3.15581497632e7
#define ORC_AU 1.49597870700e11
#define ORC_VEARTH 0.00010103671
#define ORC_LARM 2.5e9
#define ORC_SPS 8.321000e-23
#define ORC_SACC 9.000000e-30
#define ORC_SLOC 2.89e-24
#define ORC_INVSQ6 0.408248290463863 /* utils/src/glass_lisa.c:435 */

enum { ORC_FMT_SANGRIA = 0, ORC_FMT_PHASE = 1, ORC_FMT_FREQUENCY = 2 };
enum { ORC_NOISE_SCIRDV1 = 0, ORC_NOISE_SANGRIA = 1, ORC_NOISE_RADLER = 2 };

typedef struct {
    double L, fstar, ecc, R;
} orc_orbit_t;

/* utils/src/glass_lisa.c:125-136 (initialize_analytic_orbit) */
static orc_orbit_t orc_make_orbit(void)
{
    orc_orbit_t o;
    o.L = ORC_LARM;
    o.fstar = ORC_CLIGHT / (2.0 * M_PI * ORC_LARM);
    o.ecc = ORC_LARM / (2.0 * ORC_SQ3 * ORC_AU);
    o.R = ORC_AU * o.ecc;
    return o;
}

double orc_fstar(void) { return orc_make_orbit().fstar; }

/* utils/src/glass_lisa.c:77-124 (analytic_orbits); x,y,z are 1-based [4] */
static void orc_analytic_orbits(const orc_orbit_t *o, double t, double *x, double *y, double *z)
{
    static const double sbs[3] = {0.0, 0.866025403784439, -0.866025403784438};
    static const double cbs[3] = {1.0, -0.5, -0.5};
    double alpha = ORC_PI2 * t / ORC_YEAR;
    double sa = sin(alpha), ca = cos(alpha);
    double sa2 = sa * sa, ca2 = ca * ca, saca = sa * ca;
    double AUca = ORC_AU * ca, AUsa = ORC_AU * sa;
    for (int i = 0; i < 3; i++) {
        double sb = sbs[i], cb = cbs[i];
        x[i + 1] = AUca + o->R * (saca * sb - (1. + sa2) * cb);
        y[i + 1] = AUsa + o->R * (saca * cb - (1. + ca2) * sb);
        z[i + 1] = -ORC_SQ3 * o->R * (ca * cb + sa * sb);
    }
}

void orc_orbit_positions(double t, double *xyz9)
{
    orc_orbit_t o = orc_make_orbit();
    double x[4], y[4], z[4];
    orc_analytic_orbits(&o, t, x, y, z);
    for (int i = 0; i < 3; i++) {
        xyz9[3 * i + 0] = x[i + 1];
        xyz9[3 * i + 1] = y[i + 1];
        xyz9[3 * i + 2] = z[i + 1];
    }
}

/* utils/src/glass_lisa.c:1566-1596 (LISA_polarization_tensor) */
static void orc_polarization_tensor(double costh, double phi, double ep[4][4], double ec[4][4], double k[4])
{
    double u[4], v[4];
    double sinth = sqrt(1.0 - costh * costh);
    double cosph = cos(phi), sinph = sin(phi);
    u[1] = costh * cosph; u[2] = costh * sinph; u[3] = -sinth;
    v[1] = sinph;         v[2] = -cosph;        v[3] = 0.;
    k[1] = -sinth * cosph; k[2] = -sinth * sinph; k[3] = -costh;
    for (int i = 1; i <= 3; i++)
        for (int j = 1; j <= 3; j++) {
            ep[i][j] = v[i] * v[j] - u[i] * u[j];
            ec[i][j] = u[i] * v[j] + v[i] * u[j];
        }
}

/* utils/src/glass_lisa.c:1521-1564 (LISA_detector_tensor) */
static void orc_detector_tensor(double L, double ep[4][4], double ec[4][4], const double *x, const double *y,
                                const double *z, const double *k, double dp[4][4], double dc[4][4], double kr[4][4])
{
    double r12[4], r13[4], r23[4];
    r12[1] = (x[2] - x[1]) / L; r13[1] = (x[3] - x[1]) / L; r23[1] = (x[3] - x[2]) / L;
    r12[2] = (y[2] - y[1]) / L; r13[2] = (y[3] - y[1]) / L; r23[2] = (y[3] - y[2]) / L;
    r12[3] = (z[2] - z[1]) / L; r13[3] = (z[3] - z[1]) / L; r23[3] = (z[3] - z[2]) / L;
    double p12 = 0, p13 = 0, p23 = 0, c12 = 0, c13 = 0, c23 = 0;
    for (int i = 1; i <= 3; i++)
        for (int j = 1; j <= 3; j++) {
            p12 += r12[i] * r12[j] * ep[i][j]; c12 += r12[i] * r12[j] * ec[i][j];
            p23 += r23[i] * r23[j] * ep[i][j]; c23 += r23[i] * r23[j] * ec[i][j];
            p13 += r13[i] * r13[j] * ep[i][j]; c13 += r13[i] * r13[j] * ec[i][j];
        }
    dp[1][2] = dp[2][1] = p12; dc[1][2] = dc[2][1] = c12;
    dp[2][3] = dp[3][2] = p23; dc[2][3] = dc[3][2] = c23;
    dp[1][3] = dp[3][1] = p13; dc[1][3] = dc[3][1] = c13;
    double k12 = 0, k13 = 0, k23 = 0;
    for (int i = 1; i <= 3; i++) {
        k12 += k[i] * r12[i]; k13 += k[i] * r13[i]; k23 += k[i] * r23[i];
    }
    kr[1][2] = k12; kr[1][3] = k13; kr[2][3] = k23;
    kr[2][1] = -k12; kr[3][1] = -k13; kr[3][2] = -k23;
}

/* In-place forward complex DFT, X[k] = sum_n x[n] exp(-2 pi i k n / N), N a
 * power of two (the convention of kiss_fft with inverse=0). */
static void orc_fft(double *z, int N)
{
    for (int i = 1, j = 0; i < N; i++) {
        int bit = N >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double tr = z[2 * i], ti = z[2 * i + 1];
            z[2 * i] = z[2 * j]; z[2 * i + 1] = z[2 * j + 1];
            z[2 * j] = tr; z[2 * j + 1] = ti;
        }
    }
    for (int len = 2; len <= N; len <<= 1) {
        int half = len >> 1;
        for (int k = 0; k < half; k++) {
            double ang = -ORC_PI2 * (double)k / (double)len;
            double wr = cos(ang), wi = sin(ang);
            for (int s = 0; s < N; s += len) {
                int a = s + k, b = s + k + half;
                double xr = z[2 * b] * wr - z[2 * b + 1] * wi;
                double xi = z[2 * b] * wi + z[2 * b + 1] * wr;
                z[2 * b] = z[2 * a] - xr; z[2 * b + 1] = z[2 * a + 1] - xi;
                z[2 * a] += xr; z[2 * a + 1] += xi;
            }
        }
    }
}

void orc_forward_complex_fft(double *z, int N) { orc_fft(z, N); }

static int orc_is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/*
 * ucb/src/glass_ucb_waveform.c:738-1001 (ucb_waveform) with analytic orbits,
 * followed by the TDI synthesis of utils/src/glass_lisa.c:458-710.
 * X,Y,Z,A,E: 2N doubles each, 0-based.  NI as in the reference (only the
 * "phase"/"frequency" formats skip Y,Z,A,E when NI==1).
 * Returns 0, or -1 when N is not a power of two.
 */
int orc_ucb_waveform(int format, double T, double t0, const double *params, int NP, double *X, double *Y,
                     double *Z, double *A, double *E, int N, int NI)
{
    if (!orc_is_pow2(N)) return -1;
    orc_orbit_t orb = orc_make_orbit();
    double f0 = params[0] / T, costh = params[1], phi = params[2], amp = exp(params[3]);
    double cosi = params[4], psi = params[5], phi0 = params[6];
    double dfdt = NP > 7 ? params[7] / (T * T) : 0.0;
    double d2fdt2 = NP > 8 ? params[8] / (T * T * T) : 0.0;
    long q = (long)(f0 * T);
    double cosps = cos(2. * psi), sinps = sin(2. * psi);
    double Aplus = amp * (1. + cosi * cosi) * 0.5, Across = -amp * cosi;
    double df = ORC_PI2 * (((double)q) / T);
    double DPr = Aplus * cosps, DPi = -Across * sinps, DCr = -Aplus * sinps, DCi = -Across * cosps;
    double ep[4][4], ec[4][4], k[4];
    orc_polarization_tensor(costh, phi, ep, ec, k);

    /* d[(i-1)*3+(j-1)] holds the complex series of arm ij */
    double *d[9];
    for (int a = 0; a < 9; a++) d[a] = calloc(2 * (size_t)N, sizeof(double));

    double x[4], y[4], z[4], dp[4][4], dc[4][4], kr[4][4];
    for (int n = 1; n <= N; n++) {
        double t = t0 + T * (double)(n - 1) / (double)N;
        orc_analytic_orbits(&orb, t, x, y, z);
        orc_detector_tensor(orb.L, ep, ec, x, y, z, k, dp, dc, kr);
        for (int i = 1; i <= 3; i++) {
            double kdotx = (x[i] * k[1] + y[i] * k[2] + z[i] * k[3]) / ORC_CLIGHT;
            double xi = t - kdotx;
            double fi = f0;
            if (NP > 7) fi += dfdt * xi;
            if (NP > 8) fi += 0.5 * d2fdt2 * xi * xi;
            double fonfs = fi / orb.fstar;
            double arg2 = ORC_PI2 * f0 * xi - phi0 - df * t;
            if (NP > 7) arg2 += M_PI * dfdt * xi * xi;
            if (NP > 8) arg2 += (M_PI / 3.0) * d2fdt2 * xi * xi * xi;
            double aevol = 1.0;
            if (NP > 7) aevol += 0.66666666666666666666 * dfdt / f0 * xi;
            for (int j = 1; j <= 3; j++) {
                if (i == j) continue;
                double arg1 = 0.5 * fonfs * (1.0 + kr[i][j]);
                double sinc = 0.25 * sin(arg1) / arg1;
                double tran1r = aevol * (dp[i][j] * DPr + dc[i][j] * DCr);
                double tran1i = aevol * (dp[i][j] * DPi + dc[i][j] * DCi);
                double tran2r = cos(arg1 - arg2), tran2i = sin(arg1 - arg2);
                double *s = d[(i - 1) * 3 + (j - 1)];
                s[2 * (n - 1)] = sinc * (tran1r * tran2r + tran1i * tran2i);
                s[2 * (n - 1) + 1] = sinc * (-tran1r * tran2i + tran1i * tran2r);
            }
        }
    }
    /* slow-part FFTs, fftshift and 1/(2N) normalisation (:940-962) */
    double inv2N = 1. / (double)(2 * N);
    double *a[9] = {0};
    const int arms[6] = {1, 2, 3, 5, 6, 7}; /* 12,13,21,23,31,32 */
    for (int m = 0; m < 6; m++) {
        double *s = d[arms[m]];
        orc_fft(s, N);
        a[arms[m]] = malloc(2 * (size_t)N * sizeof(double));
        for (int b = 0; b < N; b++) {
            int src = (b + N / 2) % N;
            a[arms[m]][2 * b] = s[2 * src] * inv2N;
            a[arms[m]][2 * b + 1] = s[2 * src + 1] * inv2N;
        }
    }
    double *d12 = a[1], *d13 = a[2], *d21 = a[3], *d23 = a[5], *d31 = a[6], *d32 = a[7];

    /* TDI synthesis, evaluated per bin with direct trig instead of the
     * reference's recursion (the two agree to ~1e-14 relative) */
    double sqT = sqrt(T);
    int half = N / 2;
    for (int b = 0; b < N; b++) {
        int jr = 2 * b, ji = jr + 1;
        double f = ((double)(q + b - half)) / T;
        double fonfs = f / orb.fstar;
        double c1 = cos(fonfs), s1 = sin(fonfs);
        double c2 = 2. * c1 * c1 - 1.0, s2 = 2. * s1 * c1;
        double ux[2] = {d12[jr] - d13[jr], d12[ji] - d13[ji]}, vx[2] = {d21[jr] - d31[jr], d21[ji] - d31[ji]};
        double uy[2] = {d23[jr] - d21[jr], d23[ji] - d21[ji]}, vy[2] = {d32[jr] - d12[jr], d32[ji] - d12[ji]};
        double uz[2] = {d31[jr] - d32[jr], d31[ji] - d32[ji]}, vz[2] = {d13[jr] - d23[jr], d13[ji] - d23[ji]};
        if (format == ORC_FMT_SANGRIA) {
            /* utils/src/glass_lisa.c:645-710 */
            double pref = f * (4.0 / orb.fstar * sqT) * s1;
            X[jr] = pref * (ux[0] * c2 + ux[1] * s2 + vx[0] * c1 + vx[1] * s1);
            X[ji] = pref * (ux[1] * c2 - ux[0] * s2 + vx[1] * c1 - vx[0] * s1);
            Y[jr] = pref * (uy[0] * c2 + uy[1] * s2 + vy[0] * c1 + vy[1] * s1);
            Y[ji] = pref * (uy[1] * c2 - uy[0] * s2 + vy[1] * c1 - vy[0] * s1);
            Z[jr] = pref * (uz[0] * c2 + uz[1] * s2 + vz[0] * c1 + vz[1] * s1);
            Z[ji] = pref * (uz[1] * c2 - uz[0] * s2 + vz[1] * c1 - vz[0] * s1);
            A[jr] = (Z[jr] - X[jr]) * M_SQRT1_2; A[ji] = (Z[ji] - X[ji]) * M_SQRT1_2;
            E[jr] = (X[jr] - 2 * Y[jr] + Z[jr]) * ORC_INVSQ6; E[ji] = (X[ji] - 2 * Y[ji] + Z[ji]) * ORC_INVSQ6;
        } else {
            /* utils/src/glass_lisa.c:458-549 ("phase") and :551-643 ("frequency") */
            double c3 = 2. * c1 * c2 - c1, s3 = 2. * s1 * c2 + s1;
            double pref = (format == ORC_FMT_PHASE) ? sqT : sqT * 2. * fonfs;
            double *Ch[3] = {X, Y, Z};
            double *u[3] = {ux, uy, uz}, *v[3] = {vx, vy, vz};
            int nch = NI > 1 ? 3 : 1;
            for (int c = 0; c < nch; c++) {
                double *U = u[c], *V = v[c];
                Ch[c][jr] = pref * (U[0] * c3 + U[1] * s3 + V[0] * c2 + V[1] * s2 - U[0] * c1 - U[1] * s1 - V[0]);
                Ch[c][ji] = pref * (U[1] * c3 - U[0] * s3 + V[1] * c2 - V[0] * s2 - U[1] * c1 + U[0] * s1 - V[1]);
            }
            if (NI > 1) {
                A[jr] = (Z[jr] - X[jr]) * M_SQRT1_2; A[ji] = (Z[ji] - X[ji]) * M_SQRT1_2;
                E[jr] = (X[jr] - 2 * Y[jr] + Z[jr]) * ORC_INVSQ6; E[ji] = (X[ji] - 2 * Y[ji] + Z[ji]) * ORC_INVSQ6;
                if (format == ORC_FMT_PHASE) { A[ji] = -A[ji]; E[ji] = -E[ji]; }
            }
        }
    }
    for (int m = 0; m < 9; m++) { free(d[m]); free(a[m]); }
    return 0;
}

/* utils/src/glass_lisa.c:1082-1120 (get_noise_levels) */
static void orc_noise_levels(int model, double f, double *Spm, double *Sop)
{
    if (model == ORC_NOISE_RADLER) {
        *Spm = 2.5e-48 * (1.0 + pow(f / 1e-4, -2)) / f / f;
        *Sop = 1.8e-37 * (0.5) * (0.5) * f * f;
    } else if (model == ORC_NOISE_SCIRDV1) {
        double fonc = ORC_PI2 * f / ORC_CLIGHT;
        double Sa_a = 9.00e-30 * (1.0 + (0.4e-3 / f) * (0.4e-3 / f)) * (1.0 + pow((f / 8.e-3), 4));
        double Sa_d = Sa_a * pow(ORC_PI2 * f, -4.);
        *Spm = Sa_d * (fonc) * (fonc);
        double Soms_d = 2.25e-22 * (1. + pow(2.e-3 / f, 4.));
        *Sop = Soms_d * (fonc) * (fonc);
    } else {
        *Spm = 5.76e-30 / (ORC_PI2 * f * ORC_CLIGHT) / (ORC_PI2 * f * ORC_CLIGHT) * (1.0 + pow(0.4e-3 / f, 2)) *
               (1.0 + pow(f / 8.0e-3, 4));
        *Sop = 1.28e-22 * (ORC_PI2 * f / ORC_CLIGHT) * (ORC_PI2 * f / ORC_CLIGHT) * (1.0 + pow(2.0e-3 / f, 4));
    }
}

/* utils/src/glass_lisa.c:1137-1145 (AEnoise_FF) */
double orc_aenoise_ff(int model, double f)
{
    orc_orbit_t o = orc_make_orbit();
    double Spm, Sop;
    orc_noise_levels(model, f, &Spm, &Sop);
    double x = f / o.fstar;
    double cosx = cos(x), cos2x = cos(2. * x), sx = sin(x);
    return 8. * (sx * sx) * (2. * Spm * (3. + 2. * cosx + cos2x) + Sop * (2. + cosx));
}

static double orc_ipow(double x, int n)
{
    double xn = 1.0;
    for (int i = 0; i < n; i++) xn *= x;
    return xn;
}

/* utils/src/glass_lisa.c:1188-1198 (AEnoise) with rednoise (:1183) */
double orc_aenoise(double f)
{
    orc_orbit_t o = orc_make_orbit();
    double fonfstar = f / o.fstar;
    double trans = orc_ipow(sin(fonfstar), 2);
    double red = 1. + 16.0 * (pow((2.0e-5 / f), 10.0) + orc_ipow(1.0e-4 / f, 2));
    return (16.0 / 3.0) * trans *
           ((2.0 + cos(fonfstar)) * (ORC_SPS + ORC_SLOC) +
            2.0 * (3.0 + 2.0 * cos(fonfstar) + cos(2.0 * fonfstar)) *
                (ORC_SLOC / 2.0 + ORC_SACC / orc_ipow(ORC_PI2 * f, 4) * red)) /
           orc_ipow(2.0 * o.L, 2);
}

/* (int)pow(2,(int)log2(v)+1) as the reference writes it
 * (ucb/src/glass_ucb_waveform.c:712,719): for v <= 0 or NaN the reference's
 * (int) conversion is undefined; on both x86 and Arm the result is then
 * clamped to Nmin by the caller, which is what returning 0 reproduces. */
static int orc_pow2_above(double v)
{
    if (!(v > 0.0)) return 0;
    double l = log2(v);
    int e = (int)l + 1;
    if (e < 0) return 0;
    if (e > 30) return 1 << 30;
    return (int)pow(2, e);
}

/* ucb/src/glass_ucb_waveform.c:698-725 (ucb_bandwidth) */
int orc_ucb_bandwidth(double f, double fdot, double costheta, double A, double T, int NFFT)
{
    orc_orbit_t o = orc_make_orbit();
    int Nmin = 16;
    int Nmax = (int)pow(2, (int)log2((double)(NFFT / 2)));
    double sqT = sqrt(T);
    double sf = sin(f / o.fstar);
    double sn = orc_aenoise(f);
    double sintheta = sin(acos(costheta));
    double bw = 2 * T * ((4. + ORC_PI2 * f * (ORC_AU / ORC_CLIGHT) * sintheta) / ORC_YEAR + fabs(fdot) * T);
    int DS = orc_pow2_above(bw - 1);
    if (DS > Nmax) DS = Nmax;
    if (DS < Nmin) DS = Nmin;
    double SNRm = A * sqT * sf / sqrt(sn); /* analytic_snr, ucb/src/glass_ucb_waveform.c:22-25 */
    int SS = orc_pow2_above(SNRm - 1);
    if (SS > Nmax) SS = Nmax;
    if (SS < Nmin) SS = Nmin;
    return (DS > SS) ? DS : SS;
}

/* ucb/src/glass_ucb_waveform.c:727-736 (ucb_alignment); out = {BW,qmin,qmax,imin,imax} */
void orc_ucb_alignment(double T, int NFFT, int data_qmin, const double *params, int *out)
{
    double f0 = params[0] / T, costh = params[1], amp = exp(params[3]), dfdt = params[7] / (T * T);
    int BW = 2 * orc_ucb_bandwidth(f0, dfdt, costh, amp, T, NFFT);
    int qmin = (int)(f0 * T) - BW / 2;
    out[0] = BW;
    out[1] = qmin;
    out[2] = qmin + BW;
    out[3] = qmin - data_qmin;
    out[4] = qmin - data_qmin + BW;
}

/* utils/src/glass_math.c:362-380 (fourier_nwip) */
double orc_fourier_nwip(const double *a, const double *b, const double *invC, int N)
{
    double arg = 0.0;
    for (int n = 0; n < N; n++) {
        double product = a[2 * n] * b[2 * n] + a[2 * n + 1] * b[2 * n + 1];
        arg += product * invC[n];
    }
    return 2.0 * arg;
}

/*
 * One proposal on one A/E segment, in the residual form used by the
 * batched engine.  r = data minus every other source of the chain.
 *   term = -sum_{bins j in template support, 0<=j<NFFT} sum_{A,E}
 *              (|r_j - h_j|^2 - |r_j|^2) * invC_j
 * equals logL(model with h) - logL(model without h) of
 * utils/src/glass_model.c:726-774 (the reference's gaussian_log_likelihood),
 * so the sampler's delta logL (ucb/src/glass_ucb_sampler.c:155-160) is
 * term_y - term_x.  hh = (h|h) over the clipped support (:362 convention).
 * Returns the waveform size N used, or a negative value on error.
 */
int orc_dlogl_term(int format, double T, double t0, int NFFT, int qmin, const double *rA, const double *rE,
                   const double *invCA, const double *invCE, const double *params, double *term, double *hh)
{
    int al[5];
    orc_ucb_alignment(T, NFFT, qmin, params, al);
    int N = al[0], imin = al[3];
    double *buf = malloc(10 * (size_t)N * sizeof(double));
    double *X = buf, *Y = X + 2 * N, *Z = Y + 2 * N, *A = Z + 2 * N, *E = A + 2 * N;
    if (orc_ucb_waveform(format, T, t0, params, 8, X, Y, Z, A, E, N, 2) != 0) { free(buf); return -1; }
    double s = 0.0, h2 = 0.0;
    for (int i = 0; i < N; i++) {
        int j = i + imin;
        if (j < 0 || j >= NFFT) continue;
        double ar = rA[2 * j] - A[2 * i], ai = rA[2 * j + 1] - A[2 * i + 1];
        double er = rE[2 * j] - E[2 * i], ei = rE[2 * j + 1] - E[2 * i + 1];
        double ra = rA[2 * j] * rA[2 * j] + rA[2 * j + 1] * rA[2 * j + 1];
        double re = rE[2 * j] * rE[2 * j] + rE[2 * j + 1] * rE[2 * j + 1];
        s += (ar * ar + ai * ai - ra) * invCA[j] + (er * er + ei * ei - re) * invCE[j];
        h2 += (A[2 * i] * A[2 * i] + A[2 * i + 1] * A[2 * i + 1]) * invCA[j] +
              (E[2 * i] * E[2 * i] + E[2 * i + 1] * E[2 * i + 1]) * invCE[j];
    }
    *term = -s;
    *hh = 2.0 * h2;
    free(buf);
    return N;
}

/*
 * Batched form of orc_dlogl_term over independent proposals (OpenMP over
 * items, one proposal per thread at a time, as the reference runs one chain
 * per OpenMP thread: apps/src/ucb_mcmc.c:230).  Segment s holds NFFT bins
 * starting at seg_qmin[s]; its residual and inverse noise are at offset
 * s*2*NFFT (rA, rE) and s*NFFT (invCA, invCE).
 */
void orc_dlogl_batch(int format, double T, double t0, int NFFT, const int *seg_qmin, const double *rA,
                     const double *rE, const double *invCA, const double *invCE, int nitems, const int *item_seg,
                     const double *params, const double *term_x, double *dlogl, double *term_y, double *hh,
                     int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int it = 0; it < nitems; it++) {
        int s = item_seg[it];
        double ty = 0, h2 = 0;
        orc_dlogl_term(format, T, t0, NFFT, seg_qmin[s], rA + (size_t)s * 2 * NFFT, rE + (size_t)s * 2 * NFFT,
                       invCA + (size_t)s * NFFT, invCE + (size_t)s * NFFT, params + (size_t)it * 8, &ty, &h2);
        term_y[it] = ty;
        hh[it] = h2;
        dlogl[it] = ty - (term_x ? term_x[it] : 0.0);
    }
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/*
 * ucb/src/glass_ucb_waveform.c:364-522 (ucb_fisher) on one source in an A/E
 * segment: one-sided difference with epsilon = 1e-6 in params-array
 * coordinates, cos-parameters clamped at 1, and the inner products taken over
 * the perturbed template's first BW bins with invC read from segment bin 0
 * (the reference's indexing, reproduced as-is).  NaN elements become 10.
 * fisher: 64 doubles, row-major.
 */
void orc_ucb_fisher(int format, double T, double t0, int NFFT, int qmin, const double *invCA, const double *invCE,
                    const double *params, double *fisher)
{
    const int NP = 8;
    double eps = 1.0e-6, inv = 1. / eps;
    int al[5];
    orc_ucb_alignment(T, NFFT, qmin, params, al);
    int BW0 = al[0];
    size_t len = 2 * (size_t)NFFT;
    double *h0 = calloc(5 * len, sizeof(double));
    orc_ucb_waveform(format, T, t0, params, NP, h0, h0 + len, h0 + 2 * len, h0 + 3 * len, h0 + 4 * len, BW0, 2);
    double *dA = calloc(NP * len, sizeof(double)), *dE = calloc(NP * len, sizeof(double));
    double *hp = calloc(5 * len, sizeof(double));
    int BWp = BW0;
    for (int i = 0; i < NP; i++) {
        double p[8];
        for (int j = 0; j < NP; j++) p[j] = params[j];
        p[i] += eps;
        if ((i == 1 || i == 4) && p[i] > 1.0) p[i] = 1.0;
        int alp[5];
        orc_ucb_alignment(T, NFFT, qmin, p, alp);
        BWp = alp[0];
        memset(hp, 0, 5 * len * sizeof(double));
        orc_ucb_waveform(format, T, t0, p, NP, hp, hp + len, hp + 2 * len, hp + 3 * len, hp + 4 * len, BWp, 2);
        for (int n = 0; n < 2 * BWp; n++) {
            dA[i * len + n] = (hp[3 * len + n] - h0[3 * len + n]) * inv;
            dE[i * len + n] = (hp[4 * len + n] - h0[4 * len + n]) * inv;
        }
    }
    for (int i = 0; i < NP; i++)
        for (int j = i; j < NP; j++) {
            double v = orc_fourier_nwip(dA + i * len, dA + j * len, invCA, BWp) +
                       orc_fourier_nwip(dE + i * len, dE + j * len, invCE, BWp);
            if (v != v) v = 10.0;
            fisher[i * NP + j] = fisher[j * NP + i] = v;
        }
    free(h0); free(dA); free(dE); free(hp);
}

/* ------------------------------------------------------------ F-statistic */

/* Inverse of a 4x4 matrix in place by Gauss-Jordan elimination with partial
 * pivoting (the textbook algorithm; the reference calls LAPACKE dgetrf/dgetri,
 * utils/src/glass_math.c:501-523, which gives the same inverse to rounding for
 * the well-conditioned filter matrices of the F-statistic).  Returns -1 for a
 * singular matrix. */
int orc_invert4(double *m)
{
    double a[4][8];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            a[i][j] = m[4 * i + j];
            a[i][4 + j] = (i == j) ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; c++) {
        int p = c;
        for (int r = c + 1; r < 4; r++)
            if (fabs(a[r][c]) > fabs(a[p][c])) p = r;
        if (a[p][c] == 0.0) return -1;
        if (p != c)
            for (int j = 0; j < 8; j++) { double t = a[c][j]; a[c][j] = a[p][j]; a[p][j] = t; }
        double inv = 1.0 / a[c][c];
        for (int j = 0; j < 8; j++) a[c][j] *= inv;
        for (int r = 0; r < 4; r++) {
            if (r == c) continue;
            double f = a[r][c];
            if (f == 0.0) continue;
            for (int j = 0; j < 8; j++) a[r][j] -= f * a[c][j];
        }
    }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) m[4 * i + j] = a[i][4 + j];
    return 0;
}

static int orc_sgn(double v) { return (v > 0) - (v < 0); }

/*
 * Maximum-likelihood amplitude, inclination, polarisation and phase from the
 * filter coefficients a (ucb/src/glass_ucb_fstatistic.c:552-570, the A/E
 * half of get_F_params).  out: A, iota, psi, phase.
 */
void orc_fstat_params(const double *a, double *out)
{
    double a1p4 = a[0] + a[3], a2m3 = a[1] - a[2], a1m4 = a[0] - a[3], a2p3 = a[1] + a[2];
    double Ap = sqrt(a1p4 * a1p4 + a2m3 * a2m3) + sqrt(a1m4 * a1m4 + a2p3 * a2p3);
    double Ac = sqrt(a1p4 * a1p4 + a2m3 * a2m3) - sqrt(a1m4 * a1m4 + a2p3 * a2p3);
    double psi = atan2(Ap * a[3] - Ac * a[0], -(Ac * a[1] + Ap * a[2]));
    psi *= 0.5;
    double c = (double)orc_sgn(sin(2.0 * psi));
    out[0] = 0.5 * (Ap + sqrt(Ap * Ap - Ac * Ac));
    out[1] = acos(-Ac / (Ap + sqrt(Ap * Ap - Ac * Ac)));
    out[2] = psi;
    out[3] = atan2(c * (Ap * a[3] - Ac * a[0]), -c * (Ac * a[2] + Ap * a[1]));
}

/*
 * ucb/src/glass_ucb_fstatistic.c:646-703 (get_Fstat_logL), A/E channels, on
 * one segment of NFFT bins starting at bin qmin:
 *  - four filters (:231-348): ucb_waveform with amplitude 2, inclination pi/2
 *    and (psi, phase) = (0, 0), (pi/4, pi), (0, 3pi/2), (pi/4, pi/2), all of
 *    BW = ucb_bandwidth(f0, fdot, cos theta, A = 1e-22) samples;
 *  - N^i = 4 sum (d.A^i + d.E^i)/C_A and M^ij = 4 sum (A^i.A^j)/C_A +
 *    4 sum (E^i.E^j)/C_A over the filter bins i whose segment bin
 *    k = q - qmin + i - BW/2 satisfies 0 < k < NFFT (:350-516; the A-channel
 *    noise weights both channels, and bin 0 is left out, as there);
 *  - logL = N^T M^-1 N / 2 (:599-622), a = M^-1 N (:624-644) and the
 *    maximum-likelihood parameters (:525-597).
 * dA, dE: 2 NFFT doubles (re/im); C_A = 1/invCA.
 * out: logL_AE, A, iota, psi, phase.  Returns BW, or -1.
 */
int orc_fstat_logl(int format, double T, double t0, int NFFT, int qmin, const double *dA, const double *dE,
                   const double *invCA, double f0, double fdot, double theta, double phi, double *out)
{
    static const double psi_f[4] = {0.0, M_PI_4, 0.0, M_PI_4};
    static const double phase_f[4] = {0.0, M_PI, 3.0 * M_PI_2, M_PI_2};
    long q = (long)(f0 * T);
    int BW = orc_ucb_bandwidth(f0, fdot, cos(theta), 1.e-22, T, NFFT);
    size_t len = 2 * (size_t)BW;
    double *buf = calloc(4 * 5 * len, sizeof(double));
    double *Af[4], *Ef[4];
    for (int f = 0; f < 4; f++) {
        double p[8];
        p[0] = f0 * T;
        p[1] = cos(theta);
        p[2] = phi;
        p[3] = log(2.0);
        p[4] = cos(M_PI_2);
        p[5] = psi_f[f];
        p[6] = phase_f[f];
        p[7] = fdot * (T * T);
        double *h = buf + (size_t)f * 5 * len;
        if (orc_ucb_waveform(format, T, t0, p, 8, h, h + len, h + 2 * len, h + 3 * len, h + 4 * len, BW, 2)) {
            free(buf);
            return -1;
        }
        Af[f] = h + 3 * len;
        Ef[f] = h + 4 * len;
    }
    long qq = q - (long)qmin;
    double Nv[4] = {0, 0, 0, 0}, M[16] = {0};
    for (int i = 0; i < BW; i++) {
        long k = qq + i - BW / 2;
        if (!(k > 0 && k < NFFT)) continue;
        double C = 1.0 / invCA[k];
        int re = 2 * i, im = re + 1;
        for (int f = 0; f < 4; f++)
            Nv[f] += (dA[2 * k] * Af[f][re] + dA[2 * k + 1] * Af[f][im] + dE[2 * k] * Ef[f][re] +
                      dE[2 * k + 1] * Ef[f][im]) / C;
        for (int f = 0; f < 4; f++)
            for (int g = f; g < 4; g++)
                M[4 * f + g] += 4.0 * (Af[f][re] * Af[g][re] + Af[f][im] * Af[g][im]) / C +
                                4.0 * (Ef[f][re] * Ef[g][re] + Ef[f][im] * Ef[g][im]) / C;
    }
    for (int f = 0; f < 4; f++) Nv[f] *= 4.0;
    for (int f = 0; f < 4; f++)
        for (int g = f + 1; g < 4; g++) M[4 * g + f] = M[4 * f + g];
    free(buf);
    /* No filter bin inside the segment leaves M = 0; LAPACK's dgetrf/dgetri
     * then leave it as it is (its LU factors are zero and dgetri stops at the
     * zero pivot), so logL = 0 and a = 0. */
    int any = 0;
    for (int c = 0; c < 16; c++) any |= (M[c] != 0.0);
    if (any && orc_invert4(M)) return -1;
    const double *m = M;
    out[0] = 0.5 * (m[0] * Nv[0] * Nv[0] + 2 * m[1] * Nv[0] * Nv[1] + 2 * m[2] * Nv[0] * Nv[2] +
                    2 * m[3] * Nv[0] * Nv[3] + m[5] * Nv[1] * Nv[1] + 2 * m[6] * Nv[1] * Nv[2] +
                    2 * m[7] * Nv[1] * Nv[3] + m[10] * Nv[2] * Nv[2] + 2 * m[11] * Nv[2] * Nv[3] +
                    m[15] * Nv[3] * Nv[3]);
    double a[4];
    for (int i = 0; i < 4; i++)
        a[i] = m[4 * i] * Nv[0] + m[4 * i + 1] * Nv[1] + m[4 * i + 2] * Nv[2] + m[4 * i + 3] * Nv[3];
    orc_fstat_params(a, out + 1);
    return BW;
}

/* Batched form: cells[4 c] = f0, fdot, theta, phi on segment cell_seg[c];
 * out[5 c ..] as orc_fstat_logl (OpenMP over cells). */
void orc_fstat_batch(int format, double T, double t0, int NFFT, const int *seg_qmin, const double *dA,
                     const double *dE, const double *invCA, int ncells, const int *cell_seg, const double *cells,
                     double *out, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 8)
#endif
    for (int c = 0; c < ncells; c++) {
        int s = cell_seg[c];
        const double *x = cells + 4 * (size_t)c;
        if (orc_fstat_logl(format, T, t0, NFFT, seg_qmin[s], dA + (size_t)s * 2 * NFFT, dE + (size_t)s * 2 * NFFT,
                           invCA + (size_t)s * NFFT, x[0], x[1], x[2], x[3], out + 5 * (size_t)c) < 0)
            for (int k = 0; k < 5; k++) out[5 * (size_t)c + k] = NAN;
    }
}

/* ucb/src/glass_ucb_waveform.c:307-314 (ucb_fdot) */
double orc_ucb_fdot(double Mc, double f0)
{
    double M = Mc * 4.92569043916e-6; /* TSUN, utils/src/glass_constants.h:60 */
    return 19.2 * pow(pow(M_PI, 8) * pow(M, 5) * pow(f0, 11), 1. / 3.);
}

/* Lowest frequency of a segment starting at bin qmin, as the reference holds
 * it (utils/src/glass_data.c:2065: fmin = floor(fmin T)/T, and qmin =
 * (int)(fmin T) at :1078): qmin/T, raised by an ulp where needed so that
 * (int)(fmin T) gives qmin back. */
double orc_segment_fmin(int qmin, double T)
{
    double fmin = (double)qmin / T;
    while ((int)(fmin * T) < qmin) fmin = nextafter(fmin, INFINITY);
    return fmin;
}

/*
 * ucb/src/glass_ucb_proposal.c:1085-1182 (build_fstatistic_proposal) on one
 * segment, with the grid of setup_fstatistic_proposal (:927-943): n_f cells
 * of one bin in frequency, n_theta in cos(theta) and n_phi in phi, each
 * evaluated at its centre with fdot = 0 and, where that gives logL > 1, along
 * a scan of ten chirp masses up to the first logL < 1; the density is the
 * square of the largest logL, normalised so that its mean is 1.
 * tensor: n_f n_theta n_phi doubles, [i][j][k]; info = {n_f, norm, maxp}.
 */
void orc_fstat_proposal(int format, double T, double t0, int NFFT, int qmin, const double *dA, const double *dE,
                        const double *invCA, int n_theta, int n_phi, double *tensor, double *info, int nthreads)
{
    double fmin = orc_segment_fmin(qmin, T);
    double fmax = fmin + NFFT / T;
    int n_f = (int)((fmax - fmin) * T);
    double d_f = (int)((fmax - fmin) * T) / (double)n_f / T;
    double d_theta = 2. / (double)n_theta;
    double d_phi = ORC_PI2 / (double)n_phi;
    int n_fdot = 10;
    double d_fdot = (1.1 - 0.1) / n_fdot;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for collapse(2) schedule(dynamic, 4)
#endif
    for (int i = 0; i < n_f; i++)
        for (int j = 0; j < n_theta; j++) {
            double f = fmin + i * d_f;
            f += d_f / 2;
            for (int k = 0; k < n_phi; k++) {
                double theta = acos((-1. + (double)j * d_theta + d_theta / 2));
                double phi = (double)k * d_phi + d_phi / 2;
                double o[5];
                orc_fstat_logl(format, T, t0, NFFT, qmin, dA, dE, invCA, f, 0, theta, phi, o);
                double logL_AE = o[0], logLmax = logL_AE;
                if (logL_AE > 1) {
                    for (int n = 0; n < n_fdot; n++) {
                        double fdot = orc_ucb_fdot(0.1 + n * d_fdot, f);
                        orc_fstat_logl(format, T, t0, NFFT, qmin, dA, dE, invCA, f, fdot, theta, phi, o);
                        logL_AE = o[0];
                        if (logL_AE > logLmax) logLmax = logL_AE;
                        if (logL_AE < 1) break;
                    }
                }
                tensor[((size_t)i * n_theta + j) * n_phi + k] = logLmax * logLmax;
            }
        }
    double norm = 0.0;
    size_t n = (size_t)n_f * n_theta * n_phi;
    for (size_t c = 0; c < n; c++) norm += tensor[c];
    norm = (n_f * n_theta * n_phi) / norm;
    double maxp = -1.e60;
    for (size_t c = 0; c < n; c++) {
        tensor[c] *= norm;
        if (tensor[c] > maxp) maxp = tensor[c];
    }
    info[0] = n_f;
    info[1] = norm;
    info[2] = maxp;
}
