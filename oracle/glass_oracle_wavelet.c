/*
 * glass_oracle_wavelet.c -- CPU restatement of GLASS's wavelet-domain UCB
 * waveform and its sparse-pixel likelihoods.
 *
 * TEST INFRASTRUCTURE ONLY (see glass_oracle.c).  Pinned to the reference's
 * own functions (compiled into oracle/_ref) through tests/golden/
 * wavelet_waveform.npz and wavelet_likelihood.npz.
 *
 * Follows:
 *   ucb/src/glass_ucb_waveform.c
 *     ucb_phase, ucb_amplitude, ucb_barycenter_waveform   :330-362
 *     ucb_wavelet_layers                                   :1003-1042
 *     build_interpolated_waveform                          :1044-1057
 *     ucb_waveform_wavelet                                 :1061-1240
 *   utils/src/glass_lisa.c
 *     initialize_interpolated_analytic_orbits              :271-380
 *     LISA_spacecraft_to_barycenter_time                   :712-754
 *     hplus_and_hcross, LISA_TDI_spline                    :757-887
 *     LISA_spline_response                                 :920-1074
 *   utils/src/glass_math.c
 *     cubic splines (coefficients, evaluation)             :24-224
 *     wavelet_nwip                                         :382-391
 *     even_sampled_search, binary_search                   :393-402, :443-473
 *     unwrap_phase                                         :1034-1052
 *     extract_amplitude_and_phase                          :1244-1308
 *   utils/src/glass_model.c
 *     delta_log_likelihood                                 :624-691
 *     gaussian_log_likelhood_wavelet                       :805-855
 * Floating-point operations are in the reference's order (compiled with
 * -ffp-contract=off), because the carrier phase (~1e6 rad) turns last-bit
 * differences in times into 1e-10 relative differences in the waveform.
 *
 * Out-of-range spline lookups (below the first node or at/after the last),
 * where the reference's binary search reads outside its array, are clamped
 * to the first/last interval here; the waveform never makes such lookups on
 * the grids it is used with.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define W_SQ3 1.73205080757
#define W_PI2 6.283185307179586
#define W_CLIGHT 299792458.
#define W_YEAR 3.15581497632e7
#define W_AU 1.49597870700e11
#define W_VEARTH 0.00010103671
#define W_LARM 2.5e9
#define W_ORBIT_SAMPLES_PER_YEAR 200 /* utils/src/glass_lisa.h:37 */

/* WDM pieces from glass_oracle_wdm.c */
void orc_wdm_window(int Nf, int Nt, double A, double nx, int forward, double *phif);
void orc_wdm_by_layers(int Nf, int Nt, int jmin, int Nlayers, const double *phif, double *timedata);

/* ------------------------------------------------------------ splines */
typedef struct {
    int n;
    int even; /* 1: even_sampled_search, 0: binary_search */
    double *x, *c0, *c1, *c2, *c3;
} wspline;

/* natural cubic spline (utils/src/glass_math.c:101-175) */
static void wsp_init(wspline *s, int n, const double *x, const double *y, int even)
{
    s->n = n;
    s->even = even;
    s->x = malloc(sizeof(double) * n);
    s->c0 = malloc(sizeof(double) * n);
    s->c1 = malloc(sizeof(double) * n);
    s->c2 = malloc(sizeof(double) * n);
    s->c3 = malloc(sizeof(double) * n);
    double *h = calloc(n, sizeof(double)), *al = calloc(n, sizeof(double));
    double *l = calloc(n, sizeof(double)), *z = calloc(n, sizeof(double)), *mu = calloc(n, sizeof(double));
    for (int i = 0; i < n; i++) s->x[i] = x[i];
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
    s->c0[n - 1] = y[n - 1];
    s->c1[n - 1] = s->c2[n - 1] = s->c3[n - 1] = 0.0;
    for (int i = n - 2; i >= 0; i--) {
        s->c0[i] = y[i];
        s->c2[i] = z[i] - mu[i] * s->c2[i + 1];
        s->c1[i] = (s->c0[i + 1] - s->c0[i]) / h[i] - h[i] * (s->c2[i + 1] + 2.0 * s->c2[i]) / 3.0;
        s->c3[i] = (s->c2[i + 1] - s->c2[i]) / (3.0 * h[i]);
    }
    free(h);
    free(al);
    free(l);
    free(z);
    free(mu);
}

static void wsp_free(wspline *s)
{
    free(s->x);
    free(s->c0);
    free(s->c1);
    free(s->c2);
    free(s->c3);
}

/* interval of v: even_sampled_search (floor of the scaled offset, clamped to
 * [0, n-1]) or binary_search (largest node <= v) */
static int wsp_index(const wspline *s, double v)
{
    if (s->even) {
        double dx = s->x[1] - s->x[0];
        int j = (int)floor((v - s->x[0]) / dx);
        if (j < 0) j = 0;
        if (j > s->n - 1) j = s->n - 1;
        return j;
    }
    if (v <= s->x[0]) return 0;
    if (v >= s->x[s->n - 1]) return v == s->x[s->n - 1] ? s->n - 1 : s->n - 2;
    int lo = 0, hi = s->n - 1; /* x[lo] <= v < x[hi] */
    while (hi - lo > 1) {
        int mid = (lo + hi) / 2;
        if (s->x[mid] <= v)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

static double wsp_eval(const wspline *s, double v)
{
    int j = wsp_index(s, v);
    double d = v - s->x[j];
    return s->c0[j] + s->c1[j] * d + s->c2[j] * d * d + s->c3[j] * d * d * d;
}

/* ------------------------------------------------------ interpolated orbit */
typedef struct {
    int n;
    double *t;
    wspline pos[3][3]; /* [spacecraft][x,y,z] */
} worbit;

/* analytic_orbits (utils/src/glass_lisa.c:77-124), positions of the 3 S/C */
static void w_analytic(double t, double p[3][3])
{
    static const double sbs[3] = {0.0, 0.866025403784439, -0.866025403784438};
    static const double cbs[3] = {1.0, -0.5, -0.5};
    const double R = W_AU * (W_LARM / (2.0 * W_SQ3 * W_AU));
    double alpha = W_PI2 * t / W_YEAR;
    double sa = sin(alpha), ca = cos(alpha);
    double sa2 = sa * sa, ca2 = ca * ca, saca = sa * ca;
    double AUca = W_AU * ca, AUsa = W_AU * sa;
    for (int i = 0; i < 3; i++) {
        double sb = sbs[i], cb = cbs[i];
        p[i][0] = AUca + R * (saca * sb - (1. + sa2) * cb);
        p[i][1] = AUsa + R * (saca * cb - (1. + ca2) * sb);
        p[i][2] = -W_SQ3 * R * (ca * cb + sa * sb);
    }
}

/* number of orbit nodes for an observation of Tobs seconds */
int orc_orbit_nodes(double Tobs)
{
    int n = (int)(W_ORBIT_SAMPLES_PER_YEAR * Tobs / W_YEAR);
    return n < 20 ? 20 : n;
}

static void worbit_init(worbit *o, double Tobs, double t0)
{
    int n = orc_orbit_nodes(Tobs);
    double buffer = Tobs / (double)(n - 1);
    double cadence = (Tobs + 2.0 * buffer) / (double)(n - 1);
    o->n = n;
    o->t = malloc(sizeof(double) * n);
    double *v = malloc(sizeof(double) * 9 * n);
    for (int k = 0; k < n; k++) {
        double t = t0 + k * cadence - buffer, p[3][3];
        w_analytic(t, p);
        o->t[k] = t;
        for (int i = 0; i < 3; i++)
            for (int d = 0; d < 3; d++) v[(3 * i + d) * n + k] = p[i][d];
    }
    for (int i = 0; i < 3; i++)
        for (int d = 0; d < 3; d++) wsp_init(&o->pos[i][d], n, o->t, v + (3 * i + d) * n, 0);
    free(v);
}

static void worbit_free(worbit *o)
{
    for (int i = 0; i < 3; i++)
        for (int d = 0; d < 3; d++) wsp_free(&o->pos[i][d]);
    free(o->t);
}

/* orbit node times and positions (metres), pos[(3 s + d) n + k] */
void orc_orbit_grid(double Tobs, double t0, double *t, double *pos)
{
    worbit o;
    worbit_init(&o, Tobs, t0);
    for (int k = 0; k < o.n; k++) {
        t[k] = o.t[k];
        for (int i = 0; i < 3; i++)
            for (int d = 0; d < 3; d++) pos[(3 * i + d) * o.n + k] = o.pos[i][d].c0[k];
    }
    worbit_free(&o);
}

/* spacecraft-1 light-time shift, time_shifted = time - k.r_1 / c
 * (LISA_spacecraft_to_barycenter_time with flag -1) */
static void w_sc_to_ssb(const worbit *o, double costh, double phi, const double *time, double *out, int n)
{
    double sinth = sqrt(1.0 - costh * costh), cosph = cos(phi), sinph = sin(phi);
    double k[3] = {-sinth * cosph, -sinth * sinph, -costh};
    for (int i = 0; i < n; i++) {
        double r[3];
        for (int d = 0; d < 3; d++) r[d] = wsp_eval(&o->pos[0][d], time[i]) / W_CLIGHT;
        double kr = 0.0;
        for (int d = 0; d < 3; d++) kr += k[d] * r[d];
        out[i] = time[i] - kr;
    }
}

/* ------------------------------------------------------ spline response */
typedef struct {
    double Ap, Ac, c2p, s2p;
    const wspline *amp, *phase;
} wpol;

static void w_hpc(const wpol *P, double t, double *hp, double *hc, double *hpf, double *hcf)
{
    double amp = wsp_eval(P->amp, t), ph = wsp_eval(P->phase, t);
    double cp = cos(ph), sp = sin(ph);
    *hp = amp * (P->Ap * P->c2p * cp + P->Ac * P->s2p * sp);
    *hc = amp * (P->Ac * P->c2p * sp - P->Ap * P->s2p * cp);
    *hpf = amp * (-P->Ap * P->c2p * sp + P->Ac * P->s2p * cp);
    *hcf = amp * (P->Ac * P->c2p * cp + P->Ap * P->s2p * sp);
}

/* One TDI Michelson channel with vertex a and arms b, c (LISA_TDI_spline).
 * The eight delayed single-link terms; each term adds the pattern
 * +(s1 coefficient) - (s2 coefficient) with coefficient tables chosen per term. */
static void w_tdi(const wpol *P, double tn, int a, int b, int c, const double *App, const double *Apm,
                  const double *Acp, const double *Acm, const double *kr, const double *L, double *M, double *Mf)
{
    double m = 0.0, mf = 0.0, hp, hc, hpf, hcf, t;
    /* 1 */
    t = tn - kr[a] - 2.0 * L[c] - 2.0 * L[b];
    w_hpc(P, t, &hp, &hc, &hpf, &hcf);
    m += hp * Apm[b] + hc * Acm[b];
    m -= hp * App[c] + hc * Acp[c];
    mf += hpf * Apm[b] + hcf * Acm[b];
    mf -= hpf * App[c] + hcf * Acp[c];
    /* 2 */
    t = tn - kr[b] - L[c] - 2.0 * L[b];
    w_hpc(P, t, &hp, &hc, &hpf, &hcf);
    m -= hp * Apm[c] + hc * Acm[c];
    m += hp * App[c] + hc * Acp[c];
    mf -= hpf * Apm[c] + hcf * Acm[c];
    mf += hpf * App[c] + hcf * Acp[c];
    /* 3 */
    t = tn - kr[c] - L[b] - 2.0 * L[c];
    w_hpc(P, t, &hp, &hc, &hpf, &hcf);
    m += hp * App[b] + hc * Acp[b];
    m -= hp * Apm[b] + hc * Acm[b];
    mf += hpf * App[b] + hcf * Acp[b];
    mf -= hpf * Apm[b] + hcf * Acm[b];
    /* 4 */
    t = tn - kr[a] - 2.0 * L[b];
    w_hpc(P, t, &hp, &hc, &hpf, &hcf);
    m -= hp * Apm[b] + hc * Acm[b];
    m += hp * Apm[c] + hc * Acm[c];
    mf -= hpf * Apm[b] + hcf * Acm[b];
    mf += hpf * Apm[c] + hcf * Acm[c];
    /* 5 */
    t = tn - kr[a] - 2.0 * L[c];
    w_hpc(P, t, &hp, &hc, &hpf, &hcf);
    m += hp * App[c] + hc * Acp[c];
    m -= hp * App[b] + hc * Acp[b];
    mf += hpf * App[c] + hcf * Acp[c];
    mf -= hpf * App[b] + hcf * Acp[b];
    /* 6 */
    t = tn - kr[c] - L[b];
    w_hpc(P, t, &hp, &hc, &hpf, &hcf);
    m -= hp * App[b] + hc * Acp[b];
    m += hp * Apm[b] + hc * Acm[b];
    mf -= hpf * App[b] + hcf * Acp[b];
    mf += hpf * Apm[b] + hcf * Acm[b];
    /* 7 */
    t = tn - kr[b] - L[c];
    w_hpc(P, t, &hp, &hc, &hpf, &hcf);
    m += hp * Apm[c] + hc * Acm[c];
    m -= hp * App[c] + hc * Acp[c];
    mf += hpf * Apm[c] + hcf * Acm[c];
    mf -= hpf * App[c] + hcf * Acp[c];
    /* 8 */
    t = tn - kr[a];
    w_hpc(P, t, &hp, &hc, &hpf, &hcf);
    m -= hp * Apm[c] + hc * Acm[c];
    m += hp * App[b] + hc * Acp[b];
    mf -= hpf * Apm[c] + hcf * Acm[c];
    mf += hpf * App[b] + hcf * Acp[b];
    *M = m;
    *Mf = mf;
}

/* amplitude with sign flips at zero crossings, and phase relative to the
 * reference phase phiR (extract_amplitude_and_phase) */
static void w_amp_phase(int n, const double *M, const double *Mf, const double *phiR, double *As, double *Dphi)
{
    double *flip = malloc(sizeof(double) * n), *pj = malloc(sizeof(double) * n);
    for (int i = 0; i < n; i++) As[i] = sqrt(M[i] * M[i] + Mf[i] * Mf[i]);
    flip[0] = 1.0;
    pj[0] = 0.0;
    int i = 1;
    do {
        flip[i] = flip[i - 1];
        pj[i] = pj[i - 1];
        if (As[i] < As[i - 1] && As[i] < As[i + 1]) {
            double d1 = As[i + 1] + As[i - 1] - 2.0 * As[i];
            double d2 = -As[i + 1] + As[i - 1] - 2.0 * As[i];
            double d3 = -As[i + 1] + As[i - 1] + 2.0 * As[i];
            if (fabs(d2 / d1) < 0.1) {
                flip[i + 1] = -1.0 * flip[i];
                pj[i + 1] = pj[i] + M_PI;
                i++;
            }
            if (fabs(d3 / d1) < 0.1) {
                flip[i] = -1.0 * flip[i - 1];
                pj[i] = pj[i - 1] + M_PI;
            }
        }
        i++;
    } while (i < n - 1);
    flip[n - 1] = flip[n - 2];
    pj[n - 1] = pj[n - 2];
    for (i = 0; i < n; i++) {
        As[i] = flip[i] * As[i];
        double v = remainder(phiR[i], W_PI2);
        Dphi[i] = -atan2(Mf[i], M[i]) + pj[i] - v;
    }
    free(flip);
    free(pj);
}

static void w_unwrap(int n, double *ph)
{
    double v = ph[0];
    for (int i = 0; i < n; i++) {
        double u = ph[i];
        double q = rint(fabs(u - v) / W_PI2);
        if (q > 0.0) {
            if (v > u)
                u += q * W_PI2;
            else
                u -= q * W_PI2;
        }
        v = u;
        ph[i] = u;
    }
}

/* LISA_spline_response for a UCB: amplitude and phase (relative to phiR) of
 * the X, Y, Z responses at the n times t; amp[c*n + i], dphi[c*n + i] */
static void w_response(const worbit *o, const double *t, int n, double costh, double phi, double cosi, double psi,
                       const wspline *amp, const wspline *phase, const double *phiR, double *ramp, double *rphase)
{
    double u[3], v[3], k[3], ep[3][3], ec[3][3];
    double sinth = sqrt(1.0 - costh * costh), cosph = cos(phi), sinph = sin(phi);
    u[0] = costh * cosph; u[1] = costh * sinph; u[2] = -sinth;
    v[0] = sinph;         v[1] = -cosph;        v[2] = 0.;
    k[0] = -sinth * cosph; k[1] = -sinth * sinph; k[2] = -costh;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            ep[i][j] = v[i] * v[j] - u[i] * u[j];
            ec[i][j] = u[i] * v[j] + v[i] * u[j];
        }
    wpol P;
    P.c2p = cos(2. * psi);
    P.s2p = sin(2. * psi);
    P.Ap = 0.5 * (1. + cosi * cosi);
    P.Ac = -cosi;
    P.amp = amp;
    P.phase = phase;
    double *M = malloc(sizeof(double) * 3 * n), *Mf = malloc(sizeof(double) * 3 * n);
    for (int m = 0; m < n; m++) {
        double x[3][3], nv[3][3], L[3], kr[3], kn[3], dp[3], dc[3], App[3], Apm[3], Acp[3], Acm[3];
        for (int i = 0; i < 3; i++)
            for (int d = 0; d < 3; d++) x[i][d] = wsp_eval(&o->pos[i][d], t[m]) / W_CLIGHT;
        for (int d = 0; d < 3; d++) {
            nv[0][d] = x[1][d] - x[2][d];
            nv[1][d] = x[2][d] - x[0][d];
            nv[2][d] = x[0][d] - x[1][d];
        }
        for (int i = 0; i < 3; i++) {
            L[i] = 0.0;
            for (int d = 0; d < 3; d++) L[i] += nv[i][d] * nv[i][d];
            L[i] = sqrt(L[i]);
        }
        for (int i = 0; i < 3; i++)
            for (int d = 0; d < 3; d++) nv[i][d] /= L[i];
        for (int i = 0; i < 3; i++) {
            kr[i] = 0.0;
            for (int d = 0; d < 3; d++) kr[i] += k[d] * x[i][d];
        }
        for (int i = 0; i < 3; i++) {
            kn[i] = 0.0;
            for (int d = 0; d < 3; d++) kn[i] += k[d] * nv[i][d];
        }
        for (int i = 0; i < 3; i++) {
            dp[i] = dc[i] = 0.0;
            for (int j = 0; j < 3; j++)
                for (int l = 0; l < 3; l++) {
                    dp[i] += (nv[i][j] * nv[i][l]) * ep[j][l];
                    dc[i] += (nv[i][j] * nv[i][l]) * ec[j][l];
                }
        }
        for (int i = 0; i < 3; i++) {
            App[i] = dp[i] / (1.0 + kn[i]);
            Apm[i] = dp[i] / (1.0 - kn[i]);
            Acp[i] = dc[i] / (1.0 + kn[i]);
            Acm[i] = dc[i] / (1.0 - kn[i]);
        }
        w_tdi(&P, t[m], 0, 1, 2, App, Apm, Acp, Acm, kr, L, &M[m], &Mf[m]);
        w_tdi(&P, t[m], 1, 2, 0, App, Apm, Acp, Acm, kr, L, &M[n + m], &Mf[n + m]);
        w_tdi(&P, t[m], 2, 0, 1, App, Apm, Acp, Acm, kr, L, &M[2 * n + m], &Mf[2 * n + m]);
    }
    for (int c = 0; c < 3; c++) {
        w_amp_phase(n, M + c * n, Mf + c * n, phiR, ramp + c * n, rphase + c * n);
        w_unwrap(n, rphase + c * n);
    }
    free(M);
    free(Mf);
}

/* ------------------------------------------------------ the waveform */
/* ucb_wavelet_layers: first layer and number of layers holding the signal */
void orc_wavelet_layers(double Tobs, const double *params, double df, double A, int *jstart, int *jwidth)
{
    double fstart = params[0] / Tobs;
    double fstop = (params[0] / Tobs + params[7] / Tobs / Tobs);
    double fmin, fmax;
    if (fstart < fstop) {
        fmin = fstart * (1.0 - W_VEARTH);
        fmax = fstop * (1.0 + W_VEARTH);
    } else {
        fmin = fstop * (1.0 - W_VEARTH);
        fmax = fstart * (1.0 + W_VEARTH);
    }
    int j = (int)rint(fmin / df);
    double dfmin = fmin - j * df, dfmax = fmax - j * df;
    int jmin = j, jmax = j;
    if (dfmin < 0.0 && fabs(dfmin) > A / W_PI2) jmin = j - 1;
    if (dfmax > 0.0 && fabs(dfmax) > A / W_PI2) jmax = j + 1;
    *jstart = jmin;
    *jwidth = jmax - jmin + 1;
}

/*
 * ucb_waveform_wavelet on a grid of NF layers x NT pixels of duration wdt and
 * bandwidth wdf, Meyer window (A, nx), data pixels [kmin, kmax): writes the
 * pixel list (k - kmin), its length, and X, Y, Z at the listed pixels (the
 * arrays are indexed by k - kmin and are not cleared).  As in the reference,
 * the n-th listed pixel receives the n-th coefficient of the per-layer
 * transform.  Returns the first layer; *nlayers receives the layer count.
 */
int orc_ucb_waveform_wavelet(double Tobs, double t0, const double *params, int NF, int NT, double wdt, double wdf,
                             double A, double nx, int kmin, int kmax, int *list, int *nlist, double *X, double *Y,
                             double *Z, int *nlayers)
{
    worbit o;
    worbit_init(&o, Tobs, t0);
    const int ns = o.n;
    const double dt = Tobs / (double)(ns - 1);
    double *tssb = malloc(sizeof(double) * ns), *amp = malloc(sizeof(double) * ns);
    double *ph = malloc(sizeof(double) * ns);
    for (int i = 0; i < ns; i++) tssb[i] = t0 + i * dt;
    {
        /* ucb_barycenter_waveform on the orbit nodes */
        double f0 = params[0] / Tobs, phi0 = params[6], fdot = params[7] / Tobs / Tobs, fddot = 0.0;
        double A0 = exp(params[3]);
        for (int i = 0; i < ns; i++) {
            double t = o.t[i];
            ph[i] = -phi0 + W_PI2 * (f0 * t + 0.5 * fdot * t * t + 1.0 / 6.0 * fddot * t * t * t);
            amp[i] = A0 * (1.0 + 2.0 / 3.0 * fdot / f0 * t);
        }
    }
    int jmin, nl;
    orc_wavelet_layers(Tobs, params, wdf, A, &jmin, &nl);
    *nlayers = nl;
    wspline samp, sph;
    wsp_init(&samp, ns, o.t, amp, 1);
    wsp_init(&sph, ns, o.t, ph, 1);
    const double costh = params[1], phi = params[2], cosi = params[4], psi = params[5];
    double *tsc = malloc(sizeof(double) * ns), *phsc = malloc(sizeof(double) * ns);
    w_sc_to_ssb(&o, costh, phi, tssb, tsc, ns);
    for (int i = 0; i < ns; i++) phsc[i] = wsp_eval(&sph, tsc[i]);

    const int nds = NT * (nl + 1);
    const double dtds = wdt / (double)(nl + 1);
    const double fhet = (jmin - 1) * wdf;
    double *tds = malloc(sizeof(double) * nds), *phds = malloc(sizeof(double) * nds);
    double *phhet = malloc(sizeof(double) * nds), *tsc2 = malloc(sizeof(double) * nds);
    for (int i = 0; i < nds; i++) {
        tds[i] = t0 + i * dtds;
        phhet[i] = W_PI2 * fhet * tds[i];
    }
    w_sc_to_ssb(&o, costh, phi, tds, tsc2, nds);
    for (int i = 0; i < nds; i++) phds[i] = wsp_eval(&sph, tsc2[i]);

    double *ramp = malloc(sizeof(double) * 3 * ns), *rph = malloc(sizeof(double) * 3 * ns);
    w_response(&o, tssb, ns, costh, phi, cosi, psi, &samp, &sph, phsc, ramp, rph);

    double *win = malloc(sizeof(double) * (NT / 2 + 1));
    orc_wdm_window(nl + 1, NT, A, nx, 1, win);
    double *wave = malloc(sizeof(double) * 3 * nds);
    for (int c = 0; c < 3; c++) {
        wspline sa, sp;
        wsp_init(&sa, ns, tssb, ramp + c * ns, 0);
        wsp_init(&sp, ns, tssb, rph + c * ns, 0);
        double *w = wave + c * nds;
        for (int i = 0; i < nds; i++) {
            double a = wsp_eval(&sa, tds[i]);
            double p = wsp_eval(&sp, tds[i]);
            p += phds[i];
            p -= phhet[i];
            w[i] = a * cos(p);
        }
        wsp_free(&sa);
        wsp_free(&sp);
        orc_wdm_by_layers(NF, NT, jmin, nl, win, w);
    }
    int n = 0;
    for (int i = 0; i < NT; i++)
        for (int j = jmin; j < jmin + nl; j++) {
            int k = i + j * NT;
            if (k >= kmin && k < kmax) list[n++] = k - kmin;
        }
    *nlist = n;
    for (int m = 0; m < n; m++) {
        X[list[m]] = wave[m];
        Y[list[m]] = wave[nds + m];
        Z[list[m]] = wave[2 * nds + m];
    }
    free(tssb);
    free(amp);
    free(ph);
    free(tsc);
    free(phsc);
    free(tds);
    free(phds);
    free(phhet);
    free(tsc2);
    free(ramp);
    free(rph);
    free(win);
    free(wave);
    wsp_free(&samp);
    wsp_free(&sph);
    worbit_free(&o);
    return jmin;
}

/* ------------------------------------------------------ likelihoods */
double orc_wavelet_nwip(const double *a, const double *b, const double *invC, const int *list, int n)
{
    double s = 0.0;
    for (int i = 0; i < n; i++) {
        int k = list[i];
        s += a[k] * b[k] * invC[k];
    }
    return s;
}

/*
 * One model's share of delta_log_likelihood: dh and hh over the model's pixel
 * list with the nine XYZ cross terms.  d and h are 3 channels of N pixels
 * (channel-major), invC is 9 arrays of N pixels, invC[(3 i + j) N + k].
 */
void orc_wavelet_dh_hh(int N, const double *d, const double *h, const double *invC, const int *list, int n,
                       double *dh, double *hh)
{
    static const int pr[9][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}, {1, 0}, {2, 0}, {2, 1}};
    double a = 0, b = 0;
    for (int q = 0; q < 9; q++) {
        int i = pr[q][0], j = pr[q][1];
        a += orc_wavelet_nwip(d + i * N, h + j * N, invC + (3 * i + j) * N, list, n);
    }
    for (int q = 0; q < 9; q++) {
        int i = pr[q][0], j = pr[q][1];
        b += orc_wavelet_nwip(h + i * N, h + j * N, invC + (3 * i + j) * N, list, n);
    }
    *dh = a;
    *hh = b;
}

/* delta_log_likelihood for models x and y against data d */
double orc_wavelet_delta_logl(int N, const double *d, const double *hx, const int *lx, int nx, const double *hy,
                              const int *ly, int ny, const double *invC)
{
    double dhx, hhx, dhy, hhy;
    orc_wavelet_dh_hh(N, d, hx, invC, lx, nx, &dhx, &hhx);
    orc_wavelet_dh_hh(N, d, hy, invC, ly, ny, &dhy, &hhy);
    double lx_ = -0.5 * (hhx - 2.0 * dhx);
    double ly_ = -0.5 * (hhy - 2.0 * dhy);
    return ly_ - lx_;
}

/*
 * gaussian_log_likelhood_wavelet: residual = d - h on the model's pixels (set
 * to zero where the pixel's time index is outside [imin, imax]), then
 * -(XX + 2 XY)/2 over all N pixels; pixel k has time index (k + kmin) % NT.
 */
double orc_wavelet_logl_full(int N, int NT, int kmin, int imin, int imax, const double *d, const double *h,
                             const int *list, int n, const double *invC)
{
    double *r = malloc(sizeof(double) * 3 * N);
    memcpy(r, d, sizeof(double) * 3 * N);
    for (int q = 0; q < n; q++) {
        int k = list[q];
        int i = (k + kmin) % NT;
        if (k >= 0 && k < N) {
            for (int c = 0; c < 3; c++) r[c * N + k] -= h[c * N + k];
            if (i < imin || i > imax)
                for (int c = 0; c < 3; c++) r[c * N + k] = 0.0;
        }
    }
    int *all = malloc(sizeof(int) * N);
    for (int k = 0; k < N; k++) all[k] = k;
    double XX = 0.0, XY = 0.0;
    XX += orc_wavelet_nwip(r, r, invC + 0 * N, all, N);
    XX += orc_wavelet_nwip(r + N, r + N, invC + 4 * N, all, N);
    XX += orc_wavelet_nwip(r + 2 * N, r + 2 * N, invC + 8 * N, all, N);
    XY += orc_wavelet_nwip(r, r + N, invC + 1 * N, all, N);
    XY += orc_wavelet_nwip(r, r + 2 * N, invC + 2 * N, all, N);
    XY += orc_wavelet_nwip(r + N, r + 2 * N, invC + 5 * N, all, N);
    free(r);
    free(all);
    return -0.5 * (XX + 2.0 * XY);
}

/* snr_wavelet */
double orc_wavelet_snr(int N, const double *h, const int *list, int n, const double *invC)
{
    double s = 0.0;
    s += orc_wavelet_nwip(h, h, invC + 0 * N, list, n);
    s += orc_wavelet_nwip(h + N, h + N, invC + 4 * N, list, n);
    s += orc_wavelet_nwip(h + 2 * N, h + 2 * N, invC + 8 * N, list, n);
    s += orc_wavelet_nwip(h, h + N, invC + 1 * N, list, n) * 2;
    s += orc_wavelet_nwip(h, h + 2 * N, invC + 2 * N, list, n) * 2;
    s += orc_wavelet_nwip(h + N, h + 2 * N, invC + 5 * N, list, n) * 2;
    return sqrt(s);
}
