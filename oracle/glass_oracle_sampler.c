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
