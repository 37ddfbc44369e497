/*
 * glass_oracle_sampler.c -- CPU restatement of the GLASS sampler's
 * Metropolis-Hastings tail and parallel-tempering exchange, and the host C
 * library's rand_r, the reference's random-number generator.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the CUDA sampler kernels, called
 * from tests/.  The product library never links it.
 */
#include <math.h>
#include <stdlib.h>

/* rand_r of the C library (utils/src/glass_utils.c:19-22 divides it by
 * RAND_MAX): n successive values from *seed, which is advanced. */
void orc_rand_r_seq(unsigned int *seed, int n, int *out)
{
    for (int i = 0; i < n; i++) out[i] = rand_r(seed);
}

int orc_rand_max(void) { return RAND_MAX; }

static double orc_u01(unsigned int *seed) { return (double)rand_r(seed) / (double)RAND_MAX; }

/*
 * ptmcmc (utils/src/glass_sampler.c:19-63) for nens independent ladders of NC
 * chains: ladder e's chain c is entry e NC + c of logL, logLnorm, index (the
 * permutation, chain ids 0..NC-1 within the ladder), seed and acceptance;
 * temperature[NC] is shared.  From the hottest pair down: one draw that is
 * always < 1, then exchange with probability exp(dlogL (T2 - T1)/(T2 T1)).
 */
void orc_ptmcmc(int nens, int NC, const double *temperature, const double *logL, const double *logLnorm, int *index,
                unsigned int *seed, double *acceptance)
{
    for (int e = 0; e < nens; e++) {
        int *idx = index + (size_t)e * NC;
        unsigned int *r = seed + (size_t)e * NC;
        double *acc = acceptance + (size_t)e * NC;
        const double *L = logL + (size_t)e * NC, *Ln = logLnorm ? logLnorm + (size_t)e * NC : NULL;
        for (int b = NC - 1; b > 0; b--) {
            int a = b - 1;
            acc[a] = 0;
            int olda = idx[a], oldb = idx[b];
            double heat1 = temperature[a], heat2 = temperature[b];
            double logL1 = L[olda] + (Ln ? Ln[olda] : 0.0);
            double logL2 = L[oldb] + (Ln ? Ln[oldb] : 0.0);
            if (orc_u01(&r[a]) < 1.0) {
                double dlogL = logL2 - logL1;
                double H = (heat2 - heat1) / (heat2 * heat1);
                double alpha = exp(dlogL * H);
                double beta = orc_u01(&r[a]);
                if (alpha >= beta) {
                    idx[a] = oldb;
                    idx[b] = olda;
                    acc[a] = 1;
                }
            }
        }
    }
}

/*
 * The accept/reject tail of ucb_mcmc (ucb/src/glass_ucb_sampler.c:141-172) for
 * n chains: where the prior of the proposal is finite, the SNR rule (snr < 5
 * sets logPy = -inf, :149-152), logH = dlogl/T + (logPy - logPx) +
 * (logQxy - logQyx), one draw loga = log U(0,1) from the chain's stream, and
 * acceptance if logH is finite and above loga; no draw otherwise.  On
 * acceptance params_x takes params_y (8 per chain) and logL_x grows by dlogl.
 * snr may be NULL (no SNR rule).
 */
void orc_mh_accept(int n, const double *T, double *logL_x, const double *dlogl, const double *logPx,
                   const double *logPy, const double *logQxy, const double *logQyx, const double *snr,
                   unsigned int *seed, double *params_x, const double *params_y, int *accepted)
{
    for (int i = 0; i < n; i++) {
        accepted[i] = 0;
        double lpy = logPy[i];
        if (!(lpy > -INFINITY)) continue;
        if (snr && snr[i] < 5.0) lpy = -INFINITY;
        double logH = 0.0;
        logH += dlogl[i] / T[i];
        logH += lpy - logPx[i];
        logH += logQxy[i] - logQyx[i];
        double loga = log(orc_u01(&seed[i]));
        if (isfinite(logH) && logH > loga) {
            accepted[i] = 1;
            logL_x[i] += dlogl[i];
            for (int k = 0; k < 8; k++) params_x[8 * (size_t)i + k] = params_y[8 * (size_t)i + k];
        }
    }
}

/* rand_r_N_0_1 (utils/src/glass_utils.c:24-35): Marsaglia's polar method. */
static double orc_n01(unsigned int *seed)
{
    double u, v, s;
    do {
        u = 2 * orc_u01(seed) - 1;
        v = 2 * orc_u01(seed) - 1;
        s = u * u + v * v;
    } while (s >= 1 || s == 0);
    return u * sqrt(-2 * log(s) / s);
}

/*
 * draw_from_fisher (ucb/src/glass_ucb_proposal.c:348-391) for n chains: chain
 * i's parameters x = params_x[8 i ..], eigenvectors evec[64 i + 8 j + k] =
 * fisher_evectr[j][k], eigenvalues evalue[8 i ..].  Eight N(0,1) amplitudes
 * over sqrt(eigenvalue), one uniform picks the eigenvector c, jump_j = amp_c
 * evec[j][c] (0.01 x_j where that is NaN), y = x + jump with cos(theta) and
 * cos(iota) reflected (x - jump) where they reach +-1; logQ = 0, or -inf where
 * a parameter of y is NaN.  c is clamped to 7 when the uniform is exactly 1.
 */
void orc_fisher_draw(int n, const double *params_x, const double *evec, const double *evalue, unsigned int *seed,
                     double *params_y, double *logQ)
{
    for (int i = 0; i < n; i++) {
        const double *x = params_x + 8 * (size_t)i, *ev = evec + 64 * (size_t)i, *el = evalue + 8 * (size_t)i;
        double *y = params_y + 8 * (size_t)i;
        double amps[8], jump[8];
        for (int k = 0; k < 8; k++) {
            amps[k] = orc_n01(&seed[i]) / sqrt(el[k]);
            jump[k] = 0.0;
        }
        int c = (int)(orc_u01(&seed[i]) * 8.0);
        if (c > 7) c = 7;
        for (int j = 0; j < 8; j++) jump[j] += amps[c] * ev[8 * j + c];
        for (int j = 0; j < 8; j++)
            if (jump[j] != jump[j]) jump[j] = 0.01 * x[j];
        for (int j = 0; j < 8; j++) y[j] = x[j] + jump[j];
        if (y[1] >= 1.) y[1] = x[1] - jump[1];
        if (y[1] <= -1.) y[1] = x[1] - jump[1];
        if (y[4] >= 1.) y[4] = x[4] - jump[4];
        if (y[4] <= -1.) y[4] = x[4] - jump[4];
        logQ[i] = 0.0;
        for (int j = 0; j < 8; j++)
            if (y[j] != y[j]) logQ[i] = -INFINITY;
    }
}

/* ------------------------------------------------------------- priors */
/* The UCB prior pieces on p[8] with bounds pr[16] (pr[2k], pr[2k+1]) and log
 * prior volumes lv[8]; p is wrapped in place where the reference wraps it. */
#define ORC_2PI 6.283185307179586

/* check_range (ucb/src/glass_ucb_prior.c:400-438): 1 when outside. */
static int orc_check_range(double *p, const double *pr)
{
    for (int k = 0; k < 8; k++)
        if (p[k] != p[k]) return 1;
    if (p[0] < pr[0] || p[0] > pr[1]) return 1;
    if (p[1] < pr[2] || p[1] > pr[3]) return 1;
    if (p[2] < pr[4] || p[2] >= pr[5]) {
        p[2] = atan2(sin(p[2]), cos(p[2]));
        if (p[2] < 0.0) p[2] += ORC_2PI;
    }
    if (p[3] < pr[6] || p[3] > pr[7]) return 1;
    if (p[4] < pr[8] || p[4] > pr[9]) return 1;
    while (p[5] < pr[10]) p[5] += M_PI;
    while (p[5] > pr[11]) p[5] -= M_PI;
    while (p[6] < pr[12]) p[6] += ORC_2PI;
    while (p[6] > pr[13]) p[6] -= ORC_2PI;
    if (p[7] < pr[14] || p[7] > pr[15]) return 1;
    return 0;
}

/* evalaute_sky_location_prior without the galaxy histogram (:590-639). */
static double orc_sky_prior(double *p, const double *pr, const double *lv)
{
    double logP = 0.0;
    if (p[1] < pr[2] || p[1] > pr[3]) return -INFINITY;
    logP -= lv[1];
    if (pr[4] > 0.0 || pr[5] < ORC_2PI) {
        if (p[2] < pr[4] || p[2] > pr[5]) return -INFINITY;
    } else if (p[2] < pr[4] || p[2] >= pr[5]) {
        p[2] = atan2(sin(p[2]), cos(p[2]));
        if (p[2] < 0.0) p[2] += ORC_2PI;
    }
    logP -= lv[2];
    return logP;
}

/* evaluate_uniform_priors (:560-588) */
static double orc_uniform_priors(double *p, const double *pr, const double *lv)
{
    if (orc_check_range(p, pr)) return -INFINITY;
    double logP = 0.0;
    logP -= log(pr[1] - pr[0]);
    for (int k = 3; k < 8; k++) logP -= lv[k];
    return logP;
}

/* evaluate_ucb_prior (:536-556), blind search, uniform sky */
double orc_ucb_prior(double *p, const double *pr, const double *lv)
{
    if (orc_check_range(p, pr)) return -INFINITY;
    double logP = 0.0;
    logP += orc_sky_prior(p, pr, lv);
    logP += orc_uniform_priors(p, pr, lv);
    return logP;
}

/* draw_from_uniform_prior (utils/src/glass_sampler.c:96-107) */
static double orc_prior_draw(double *p, const double *pr, const double *lv, unsigned int *seed)
{
    double logQ = 0.0;
    for (int k = 0; k < 8; k++) {
        p[k] = pr[2 * k] + orc_u01(seed) * (pr[2 * k + 1] - pr[2 * k]);
        logQ -= lv[k];
    }
    return logQ;
}

/* ---------------------------------------------------- birth/death step */
/* The F-statistic proposal grid: density tensor[(i nt + j) np + k]. */
typedef struct {
    const double *tensor;
    int nf, nt, np;
    double df, dt, dp, maxp;
    int qmin;
    double T;
} orc_fgrid;

/* evaluate_fstatistic_proposal (ucb/src/glass_ucb_proposal.c:1640-1673) */
static double orc_fstat_density(double *p, const orc_fgrid *g, const double *pr, const double *lv)
{
    double logP = 0.0;
    logP += orc_sky_prior(p, pr, lv);
    logP += orc_uniform_priors(p, pr, lv);
    int i = (int)floor((p[0] - g->qmin) / (g->df * g->T));
    int j = (int)floor((p[1] + 1) / g->dt);
    int k = (int)floor(p[2] / g->dp);
    if (i < 0 || i >= g->nf || j < 0 || j >= g->nt || k < 0 || k >= g->np) return -INFINITY;
    return logP + log(g->tensor[((size_t)i * g->nt + j) * g->np + k]);
}

/* draw_from_fstatistic (:1526-1568): a prior draw, then rejection sampling
 * of the frequency and sky cell. */
static double orc_fstat_draw(double *p, const orc_fgrid *g, const double *pr, const double *lv, unsigned int *seed)
{
    orc_prior_draw(p, pr, lv, seed);
    double q, ct, ph, pc, alpha;
    do {
        double i = orc_u01(seed) * g->nf, j = orc_u01(seed) * g->nt, k = orc_u01(seed) * g->np;
        q = (double)g->qmin + i * g->df * g->T;
        ct = -1. + j * g->dt;
        ph = k * g->dp;
        int ii = (int)i < g->nf ? (int)i : g->nf - 1, jj = (int)j < g->nt ? (int)j : g->nt - 1;
        int kk = (int)k < g->np ? (int)k : g->np - 1;
        pc = g->tensor[((size_t)ii * g->nt + jj) * g->np + kk];
        alpha = orc_u01(seed) * g->maxp;
    } while (pc < alpha);
    p[0] = q;
    p[1] = ct;
    p[2] = ph;
    return orc_fstat_density(p, g, pr, lv);
}

/*
 * ucb_rjmcmc (ucb/src/glass_ucb_sampler.c:454-566) with rj_birth_death
 * (:175-249) for chain i, in two halves around the likelihood, as the device
 * kernels split it.  Propose: the proposal kind by rejection on rjw[9] (0:
 * prior, 1: F-statistic draw), the always-birth/death draw, birth or death,
 * the new source or the removed one and the proposal densities.
 */
void orc_rj_propose(int n, int maxsrc, const int *Nlive, const int *Neff, const double *src, const double *prior,
                    const double *logPV, const double *rjw, const double *tensor, int nf, int nt, int np, double df,
                    double dt, double dp, double maxp, int qmin, double T, unsigned int *seed, int *move, int *slot,
                    int *kind, double *params_y, double *logQxy, double *logQyx, double *logPy)
{
    orc_fgrid g = {tensor, nf, nt, np, df, dt, dp, maxp, qmin, T};
    for (int i = 0; i < n; i++) {
        unsigned int *s = &seed[i];
        int k;
        do k = (int)floor(9 * orc_u01(s));
        while (rjw[k] <= orc_u01(s));
        orc_u01(s);
        int Nx = Nlive[i];
        const double *x = src + (size_t)i * maxsrc * 8;
        double *y = params_y + 8 * (size_t)i;
        double lqxy = 0.0, lqyx = 0.0, lpy = 0.0;
        if (orc_u01(s) < 0.5) {
            move[i] = 1;
            slot[i] = Nx;
            if (Nx + 1 < Neff[i]) {
                lqyx = k == 0 ? orc_prior_draw(y, prior, logPV, s) : orc_fstat_draw(y, &g, prior, logPV, s);
            } else {
                lpy = -INFINITY;
            }
        } else {
            move[i] = -1;
            int kill = (int)(orc_u01(s) * (double)Nx);
            slot[i] = kill;
            if (Nx - 1 > -1) {
                for (int c = 0; c < 8; c++) y[c] = x[8 * kill + c];
                if (k == 0) {
                    for (int c = 0; c < 8; c++) lqxy -= logPV[c];
                } else {
                    double yk[8];
                    for (int c = 0; c < 8; c++) yk[c] = y[c];
                    lqxy = orc_fstat_density(yk, &g, prior, logPV);
                }
            } else {
                lpy = -INFINITY;
            }
        }
        kind[i] = k;
        logQxy[i] = lqxy;
        logQyx[i] = lqyx;
        logPy[i] = lpy;
    }
}

/* Accept: the birth's SNR cut (snr = sqrt(hh) < 5), the priors of both
 * source lists, logH, one draw, and on acceptance the new list. */
void orc_rj_accept(int n, int maxsrc, int *Nlive, double *src, const int *move, const int *slot, double *params_y,
                   const double *logQxy, const double *logQyx, const double *logPy, const double *T,
                   const double *dlogl, const double *hh, int prior_only, const double *prior, const double *logPV,
                   unsigned int *seed, double *logL_x, int *accepted)
{
    for (int i = 0; i < n; i++) {
        int Nx = Nlive[i], mv = move[i], sl = slot[i], Ny = Nx + mv;
        double *x = src + (size_t)i * maxsrc * 8;
        double *y = params_y + 8 * (size_t)i;
        double lpy = logPy[i];
        if (mv > 0 && lpy > -INFINITY && !prior_only && hh && sqrt(hh[i]) < 5.0) lpy = -INFINITY;
        double logPx = 0.0;
        if (lpy > -INFINITY) {
            double ycopy[64][8];
            for (int m = 0; m < Ny && m < 64; m++) {
                const double *from = (mv > 0) ? (m < Nx ? x + 8 * m : y) : x + 8 * (m < sl ? m : m + 1);
                for (int c = 0; c < 8; c++) ycopy[m][c] = from[c];
            }
            for (int m = 0; m < Nx; m++) logPx += orc_ucb_prior(x + 8 * m, prior, logPV);
            for (int m = 0; m < Ny && m < 64; m++) {
                lpy += orc_ucb_prior(ycopy[m], prior, logPV);
                if (mv > 0 && m == Nx)
                    for (int c = 0; c < 8; c++) y[c] = ycopy[m][c];
            }
        }
        double logH = 0.0;
        if (lpy > -INFINITY && !prior_only) logH += dlogl[i] / T[i];
        logH += lpy - logPx;
        logH += logQxy[i] - logQyx[i];
        double loga = log(orc_u01(&seed[i]));
        accepted[i] = 0;
        if (isfinite(logH) && logH > loga) {
            accepted[i] = 1;
            if (mv > 0) {
                for (int c = 0; c < 8; c++) x[8 * Nx + c] = y[c];
            } else {
                for (int m = sl; m < Ny; m++)
                    for (int c = 0; c < 8; c++) x[8 * m + c] = x[8 * (m + 1) + c];
            }
            Nlive[i] = Ny;
            logL_x[i] += dlogl[i];
        }
    }
}
