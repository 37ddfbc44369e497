/*
 * glass_oracle_wdm.c -- CPU restatement of GLASS's WDM wavelet transforms.
 *
 * TEST INFRASTRUCTURE ONLY (see glass_oracle.c).  Pinned to the reference's
 * own functions (compiled into oracle/_ref) through tests/golden/wdm.npz.
 *
 * Follows utils/src/glass_wavelet.c:
 *   build_wdm_filter_freq        :305-349  (Meyer window, incomplete beta)
 *   wavelet_transform_freq       :410-460  (FFT -> WDM)
 *   wavelet_transform_inverse_freq :351-405 (WDM -> FFT)
 *   wavelet_transform_timefreq   :293-303  (real FFT, then the above)
 *   wavelet_transform_timefreq_by_layers :544-611 (per-source layers)
 * with the FFT conventions of utils/src/glass_math.c:703-853 (kissfft:
 * forward unnormalised exp(-i), inverse divided by N, real FFT of N samples to
 * N/2+1 bins).  The window exponent (nx; the reference hard-codes 6 as
 * WAVELET_FILTER_CONSTANT, utils/src/glass_wavelet.h:21) is a parameter here.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cplx;

/* utils/src/glass_math.c:1214-1242: I_x(a,b) through the hypergeometric
 * series, which terminates for integer b. */
static double orc_hyp(double a, double b, double c, double x)
{
    const double TOL = 1e-8;
    double term = a * b * x / c, value = 1.0 + term;
    int n = 1;
    while (fabs(term) > TOL) {
        a++, b++, c++, n++;
        term *= a * b * x / c / n;
        value += term;
    }
    return value;
}

double orc_incomplete_beta(double a, double b, double x)
{
    double F = orc_hyp(a, 1 - b, a + 1, x);
    double B = exp(lgamma(a) + lgamma(b) - lgamma(a + b));
    return pow(x, a) * F / B / a;
}

/* utils/src/glass_wavelet.c:305-349 */
void orc_wdm_window(int Nf, int Nt, double A, double nx, int forward, double *phif)
{
    double DeltaOmega = M_PI / Nf;
    double domega = 2 * DeltaOmega / (double)Nt;
    double B = DeltaOmega - 2 * A, insDOM = 1.0 / sqrt(DeltaOmega);
    for (int i = 0; i < Nt / 2 + 1; i++) {
        double omega = domega * i, z = 0.0;
        if (fabs(omega) >= A && fabs(omega) < A + B) {
            double x = (fabs(omega) - A) / B;
            double y = orc_incomplete_beta(nx, nx, x);
            z = insDOM * cos(y * M_PI_2);
        }
        if (fabs(omega) < A) z = insDOM;
        phif[i] = z;
    }
    double norm = 0.0;
    for (int i = 0; i < Nt / 2 + 1; i++) norm += (i == 0 ? 1.0 : 2.0) * phif[i] * phif[i];
    norm *= domega * M_1_PI;
    norm = sqrt(norm);
    if (forward) norm *= Nf / 2.0;
    for (int i = 0; i < Nt / 2 + 1; i++) phif[i] /= norm;
}

/* Mixed-radix decimation-in-time DFT, X[k] = sum x[n] exp(sign 2 pi i k n/N)
 * (sign -1 forward), recursive over the smallest prime factor; O(p^2) per
 * butterfly, so fine for the small factors WDM grids have.  The twiddles come
 * from one table of the top-level roots: a sub-transform of length N/s uses
 * every s-th root. */
static void orc_dft_rec(const cplx *x, cplx *X, int N, int stride, const cplx *w, int Ntop, cplx *tmp)
{
    if (N == 1) {
        X[0] = x[0];
        return;
    }
    int p = 2;
    while (p * p <= N && N % p) p++;
    if (N % p) p = N;
    int M = N / p;
    const long long s = Ntop / N;
    for (int r = 0; r < p; r++) orc_dft_rec(x + r * stride, tmp + r * M, M, stride * p, w, Ntop, X);
    for (int k = 0; k < M; k++)
        for (int q = 0; q < p; q++) {
            cplx acc = 0;
            for (int r = 0; r < p; r++) acc += tmp[r * M + k] * w[((long long)r * (k + q * M) % N) * s];
            X[k + q * M] = acc;
        }
}

/* Stockham autosort FFT for N = 2^a 3^b (radix-3 stages, then radix 4, then
 * one radix 2): stage with radix R after sub-length p reads x[i + m N/R]
 * (i < N/R, k = i mod p), multiplies by w^{m k N/(p R)}, and writes the R-point
 * DFT to y[(i - k) R + k + q p]. */
static int orc_smooth23(int N)
{
    while (N % 3 == 0) N /= 3;
    return N > 0 && (N & (N - 1)) == 0;
}

static void orc_stockham(const cplx *x, cplx *X, int N, int sign)
{
    cplx *w = malloc(sizeof(cplx) * N), *a = malloc(sizeof(cplx) * N), *b = malloc(sizeof(cplx) * N);
    for (int j = 0; j < N; j++) {
        double ang = sign * 2.0 * M_PI * (double)j / (double)N;
        w[j] = cos(ang) + I * sin(ang);
    }
    memcpy(a, x, sizeof(cplx) * N);
    int p = 1, rem = N;
    while (rem > 1) {
        int R = rem % 3 == 0 ? 3 : rem % 4 == 0 ? 4 : 2;
        int nb = N / R, step = N / (p * R);
        cplx wr[4];
        for (int q = 0; q < R; q++) wr[q] = w[(long long)q * (N / R) % N];
        for (int i = 0; i < nb; i++) {
            int k = i % p, j = (i - k) * R + k;
            cplx v[4];
            for (int m = 0; m < R; m++) v[m] = a[i + m * nb] * w[(long long)m * k * step % N];
            for (int q = 0; q < R; q++) {
                cplx acc = 0;
                for (int m = 0; m < R; m++) acc += v[m] * wr[(m * q) % R];
                b[j + q * p] = acc;
            }
        }
        cplx *t = a;
        a = b;
        b = t;
        p *= R;
        rem /= R;
    }
    memcpy(X, a, sizeof(cplx) * N);
    free(w);
    free(a);
    free(b);
}

static void orc_dft(const cplx *x, cplx *X, int N, int sign)
{
    if (orc_smooth23(N)) {
        orc_stockham(x, X, N, sign);
        return;
    }
    cplx *tmp = malloc(sizeof(cplx) * N);
    cplx *xx = malloc(sizeof(cplx) * N);
    cplx *w = malloc(sizeof(cplx) * N);
    for (int j = 0; j < N; j++) {
        double ang = sign * 2.0 * M_PI * (double)j / (double)N;
        w[j] = cos(ang) + I * sin(ang);
    }
    memcpy(xx, x, sizeof(cplx) * N);
    orc_dft_rec(xx, X, N, 1, w, N, tmp);
    free(tmp);
    free(xx);
    free(w);
}

void orc_complex_fft(const double *in, double *out, int N, int inverse)
{
    orc_dft((const cplx *)in, (cplx *)out, N, inverse ? 1 : -1);
    if (inverse)
        for (int i = 0; i < 2 * N; i++) out[i] /= N;
}

/* real FFT of N samples -> N/2+1 bins (utils/src/glass_math.c:808-817) */
void orc_rfft(const double *t, double *f, int N)
{
    cplx *x = malloc(sizeof(cplx) * N), *X = malloc(sizeof(cplx) * N);
    for (int i = 0; i < N; i++) x[i] = t[i];
    orc_dft(x, X, N, -1);
    for (int k = 0; k <= N / 2; k++) {
        f[2 * k] = creal(X[k]);
        f[2 * k + 1] = cimag(X[k]);
    }
    free(x);
    free(X);
}

/* inverse real FFT, N/2+1 bins -> N samples, divided by N (:819-828); the
 * imaginary parts of the DC and Nyquist bins are ignored, as kiss_fftri does */
void orc_irfft(const double *f, double *t, int N)
{
    cplx *X = malloc(sizeof(cplx) * N), *x = malloc(sizeof(cplx) * N);
    for (int k = 0; k <= N / 2; k++) X[k] = f[2 * k] + I * f[2 * k + 1];
    X[0] = creal(X[0]);
    if (N % 2 == 0) X[N / 2] = creal(X[N / 2]);
    for (int k = N / 2 + 1; k < N; k++) X[k] = conj(X[N - k]);
    orc_dft(X, x, N, 1);
    for (int i = 0; i < N; i++) t[i] = creal(x[i]) / N;
    free(X);
    free(x);
}

/* utils/src/glass_wavelet.c:410-460: N/2+1 FFT bins -> NF*NT coefficients,
 * layout wdm[n + NT m], DC and Nyquist layers packed in row 0 */
void orc_wdm_from_freq(int Nf, int Nt, const double *phif, const double *freqdata, double *wdm)
{
    cplx *DX = malloc(sizeof(cplx) * Nt), *DXt = malloc(sizeof(cplx) * Nt);
    for (int m = 0; m <= Nf; m++) {
        int center = m * Nt / 2;
        for (int i = 0; i < Nt; i++) DX[i] = 0;
        for (int j = -Nt / 2 + 1; j < Nt / 2; j++) {
            int idx = center + j;
            if (m == 0 && idx < 0) continue;
            if (m == Nf && idx > center) continue;
            double weight = phif[abs(j)];
            if (j == 0 && (m == 0 || m == Nf)) weight /= 2.0;
            DX[Nt / 2 + j] = weight * (freqdata[2 * idx] + I * freqdata[2 * idx + 1]);
        }
        orc_complex_fft((double *)DX, (double *)DXt, Nt, 1);
        if (m == 0) {
            for (int n = 0; n < Nt; n += 2) wdm[n] = creal(DXt[n]) * M_SQRT2;
        } else if (m == Nf) {
            for (int n = 0; n < Nt; n += 2) wdm[n + 1] = creal(DXt[n]) * M_SQRT2;
        } else {
            int sgn = m % 2 == 0 ? 1 : -1;
            for (int n = 0; n < Nt; n++) wdm[n + Nt * m] = ((n + m) % 2 == 0) ? creal(DXt[n]) : sgn * cimag(DXt[n]);
        }
    }
    free(DX);
    free(DXt);
}

/* utils/src/glass_wavelet.c:351-405: NF*NT coefficients -> N/2+1 FFT bins */
void orc_wdm_to_freq(int Nf, int Nt, const double *phif, const double *wdm, double *freqdata)
{
    int ND = Nf * Nt;
    memset(freqdata, 0, sizeof(double) * (ND + 2));
    cplx *pre = malloc(sizeof(cplx) * Nt), *res = malloc(sizeof(cplx) * Nt);
    for (int m = 0; m < Nf + 1; m++) {
        int center = m * Nt / 2;
        for (int n = 0; n < Nt; n++) pre[n] = 0;
        if (m == 0) {
            for (int n = 0; n < Nt; n++) pre[n] = wdm[(2 * n) % Nt] * M_SQRT1_2;
        } else if (m == Nf) {
            for (int n = 0; n < Nt; n++) pre[n] = wdm[(2 * n) % Nt + 1] * M_SQRT1_2;
        } else {
            for (int n = 0; n < Nt; n++) pre[n] = ((n + m) % 2 == 0) ? wdm[n + Nt * m] + 0 * I : -I * wdm[n + Nt * m];
        }
        orc_complex_fft((double *)pre, (double *)res, Nt, 0);
        int imin = center - Nt / 2, imax = center + Nt / 2;
        if (imin < 0) imin = 0;
        if (imax > ND / 2 + 1) imax = ND / 2 + 1;
        for (int i = imin; i < imax; i++) {
            int iind = abs(i - center);
            if (iind > Nt / 2) continue;
            cplx v = (m == 0 || m == Nf) ? res[(2 * i) % Nt] : res[i % Nt];
            v *= phif[iind] * Nf / 2;
            freqdata[2 * i] += creal(v);
            freqdata[2 * i + 1] += cimag(v);
        }
    }
    free(pre);
    free(res);
}

/* utils/src/glass_wavelet.c:293-303 (forward, time -> WDM) */
void orc_wdm_forward(int Nf, int Nt, const double *phif, const double *time, double *wdm)
{
    int ND = Nf * Nt;
    double *f = malloc(sizeof(double) * (ND + 2));
    orc_rfft(time, f, ND);
    orc_wdm_from_freq(Nf, Nt, phif, f, wdm);
    free(f);
}

/* WDM -> time: the inverse transform to frequency, then the inverse real FFT */
void orc_wdm_inverse(int Nf, int Nt, const double *phif, const double *wdm, double *time)
{
    int ND = Nf * Nt;
    double *f = malloc(sizeof(double) * (ND + 2));
    orc_wdm_to_freq(Nf, Nt, phif, wdm, f);
    orc_irfft(f, time, ND);
    free(f);
}

/* utils/src/glass_wavelet.c:544-611: heterodyned series of Nt*(Nlayers+1)
 * samples -> coefficients of layers jmin .. jmin+Nlayers-1, written in place
 * with layout k = n*Nlayers + (m - jmin). */
void orc_wdm_by_layers(int Nf, int Nt, int jmin, int Nlayers, const double *phif, double *timedata)
{
    int N = Nt * (Nlayers + 1);
    double *freq = malloc(sizeof(double) * (N + 2));
    double normalization = sqrt((double)Nf) / (Nlayers + 1.0);
    orc_rfft(timedata, freq, N);
    cplx *DX = malloc(sizeof(cplx) * Nt), *DXt = malloc(sizeof(cplx) * Nt);
    memset(timedata, 0, sizeof(double) * N);
    for (int m = jmin; m < jmin + Nlayers; m++) {
        int center = (m - jmin + 1) * Nt / 2;
        for (int i = 0; i < Nt; i++) DX[i] = 0;
        for (int j = -Nt / 2 + 1; j < Nt / 2; j++) {
            int idx = center + j;
            if (idx < 0 || idx > N / 2) continue;
            double weight = phif[abs(j)];
            if (j == 0 && (m == 0 || m == Nf)) weight /= 2.0;
            DX[Nt / 2 + j] = weight * (freq[2 * idx] + I * freq[2 * idx + 1]);
        }
        orc_complex_fft((double *)DX, (double *)DXt, Nt, 1);
        int off = m - jmin;
        if (m == 0 || m == Nf) {
            for (int n = 0; n < Nt; n += 2) timedata[n * Nlayers + off] = creal(DXt[n]) * M_SQRT2 * normalization;
        } else {
            int sgn = m % 2 == 0 ? 1 : -1;
            for (int n = 0; n < Nt; n++)
                timedata[n * Nlayers + off] =
                    (((n + m) % 2 == 0) ? creal(DXt[n]) : sgn * cimag(DXt[n])) * normalization;
        }
    }
    free(freq);
    free(DX);
    free(DXt);
}
