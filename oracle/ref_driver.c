/*
 * Flat C entry points around the reference's own functions, compiled together
 * with the reference sources into oracle/_ref/libglassref.so (Makefile.ref).
 * Test infrastructure only: it lets Python drive the reference code with plain
 * pointers so that golden vectors can be generated and the CPU restatement in
 * glass_oracle.c can be pinned against it.
 *
 * Every function sets up the reference structs the same way the reference's
 * apps do for a single frequency segment (apps/src/ucb_mcmc.c:40-120,
 * utils/src/glass_data.c:179-280), with analytic orbits
 * (utils/src/glass_lisa.c:125-136).
 */
#include "glass_utils.h"
#include "glass_ucb.h"
#include "glass_noise.h"

static void setup_orbit(struct Orbit *orbit)
{
    memset(orbit, 0, sizeof(*orbit));
    initialize_analytic_orbit(orbit);
}

int ref_driver_present(void) { return 1; }

double ref_fstar(void)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    return orbit.fstar;
}

/* ucb/src/glass_ucb_waveform.c:738 with analytic orbits */
void ref_ucb_waveform(const char *format, double T, double t0, double *params, int NP,
                      double *X, double *Y, double *Z, double *A, double *E, int BW, int NI)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    ucb_waveform(&orbit, (char *)format, T, t0, params, NP, X, Y, Z, A, E, BW, NI);
}

/* ucb/src/glass_ucb_waveform.c:698 */
int ref_ucb_bandwidth(double f, double fdot, double costheta, double amp, double T, int NFFT)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    return ucb_bandwidth(orbit.L, orbit.fstar, f, fdot, costheta, amp, T, NFFT);
}

/* ucb/src/glass_ucb_waveform.c:727; out = {BW, qmin, qmax, imin, imax} */
void ref_ucb_alignment(double T, int NFFT, int data_qmin, double *params, int *out)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    struct Data data;
    memset(&data, 0, sizeof(data));
    data.T = T;
    data.NFFT = NFFT;
    data.qmin = data_qmin;
    struct Source source;
    memset(&source, 0, sizeof(source));
    source.params = params;
    ucb_alignment(&orbit, &data, &source);
    out[0] = source.BW;
    out[1] = source.qmin;
    out[2] = source.qmax;
    out[3] = source.imin;
    out[4] = source.imax;
}

/* utils/src/glass_lisa.c:1082 + :1137 */
double ref_aenoise_ff(const char *model, double f)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    double Spm, Sop;
    get_noise_levels((char *)model, f, &Spm, &Sop);
    return AEnoise_FF(orbit.L, orbit.fstar, f, Spm, Sop);
}

/* utils/src/glass_lisa.c:1188 */
double ref_aenoise(double f)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    return AEnoise(orbit.L, orbit.fstar, f);
}

/* utils/src/glass_math.c:362 */
double ref_fourier_nwip(const double *a, const double *b, const double *invC, int N)
{
    return fourier_nwip(a, b, invC, N);
}

/*
 * One A/E frequency segment (Nchannel = 2, Fourier basis) and a model of
 * Nsrc sources: generate_ucb_model (ucb/src/glass_ucb_model.c:55) followed by
 * gaussian_log_likelihood (utils/src/glass_model.c:726).
 *   dA, dE : 2*NFFT doubles each (re/im interleaved data)
 *   invCA, invCE : NFFT doubles each
 *   params : Nsrc * 8 doubles
 * If snr_out is not NULL it receives snr() of every source
 * (utils/src/glass_math.c:403), the value the sampler rejects on.
 */
double ref_log_likelihood(const char *format, double T, double t0, int NFFT, int qmin,
                          const double *dA, const double *dE,
                          const double *invCA, const double *invCE,
                          int Nsrc, const double *params, double *snr_out)
{
    struct Orbit orbit;
    setup_orbit(&orbit);

    struct Data *data = calloc(1, sizeof(struct Data));
    data->NFFT = NFFT;
    data->N = 2 * NFFT;
    data->Nchannel = 2;
    data->Nlayer = 1;
    data->T = T;
    data->sqT = sqrt(T);
    data->t0 = t0;
    data->qmin = qmin;
    data->qmax = qmin + NFFT;
    data->fmin = qmin / T;
    data->fmax = (qmin + NFFT) / T;
    strcpy(data->format, format);
    strcpy(data->basis, "fourier");
    data->tdi = malloc(sizeof(struct TDI));
    alloc_tdi(data->tdi, data->N, data->Nchannel);
    memcpy(data->tdi->A, dA, sizeof(double) * data->N);
    memcpy(data->tdi->E, dE, sizeof(double) * data->N);

    int Nmax = Nsrc > 0 ? Nsrc : 1;
    struct Model *model = calloc(1, sizeof(struct Model));
    alloc_model(data, model, UCB_MODEL_NP, Nmax);
    model->Nlive = Nsrc;
    model->t0 = t0;
    for (int n = 0; n < NFFT; n++) {
        model->noise->invC[0][0][n] = invCA[n];
        model->noise->invC[1][1][n] = invCE[n];
        model->noise->C[0][0][n] = 1.0 / invCA[n];
        model->noise->C[1][1][n] = 1.0 / invCE[n];
    }
    for (int s = 0; s < Nsrc; s++)
        for (int p = 0; p < UCB_MODEL_NP; p++) model->source[s]->params[p] = params[s * UCB_MODEL_NP + p];

    generate_ucb_model(&orbit, data, model, -1);
    if (snr_out)
        for (int s = 0; s < Nsrc; s++) snr_out[s] = snr(model->source[s], model->noise);
    double logL = gaussian_log_likelihood(data, model);

    free_model(model);
    free_tdi(data->tdi);
    free(data);
    return logL;
}

/*
 * ucb/src/glass_ucb_waveform.c:364 on one source in an A/E segment.
 * fisher: 64 doubles (row-major), evalue: 8, evectr: 64 (evectr[i*8+j] =
 * component i of eigenvector j, as matrix_eigenstuff stores it).
 */
void ref_ucb_fisher(const char *format, double T, double t0, int NFFT, int qmin,
                    const double *invCA, const double *invCE, const double *params,
                    double *fisher, double *evalue, double *evectr)
{
    struct Orbit orbit;
    setup_orbit(&orbit);

    struct Data *data = calloc(1, sizeof(struct Data));
    data->NFFT = NFFT;
    data->N = 2 * NFFT;
    data->Nchannel = 2;
    data->Nlayer = 1;
    data->T = T;
    data->t0 = t0;
    data->qmin = qmin;
    strcpy(data->format, format);
    strcpy(data->basis, "fourier");

    struct Noise *noise = malloc(sizeof(struct Noise));
    alloc_noise(noise, NFFT, 1, 2);
    for (int n = 0; n < NFFT; n++) {
        noise->invC[0][0][n] = invCA[n];
        noise->invC[1][1][n] = invCE[n];
        noise->C[0][0][n] = 1.0 / invCA[n];
        noise->C[1][1][n] = 1.0 / invCE[n];
    }

    struct Source *source = malloc(sizeof(struct Source));
    alloc_source(source, data->N, UCB_MODEL_NP, data->Nchannel);
    for (int p = 0; p < UCB_MODEL_NP; p++) source->params[p] = params[p];
    map_array_to_ucb_params(source, source->params, T);
    ucb_alignment(&orbit, data, source);
    ucb_waveform(&orbit, data->format, T, t0, source->params, UCB_MODEL_NP, source->tdi->X,
                 source->tdi->Y, source->tdi->Z, source->tdi->A, source->tdi->E, source->BW,
                 source->tdi->Nchannel);
    ucb_fisher(&orbit, data, source, noise);
    for (int i = 0; i < UCB_MODEL_NP; i++) {
        evalue[i] = source->fisher_evalue[i];
        for (int j = 0; j < UCB_MODEL_NP; j++) {
            fisher[i * UCB_MODEL_NP + j] = source->fisher_matrix[i][j];
            evectr[i * UCB_MODEL_NP + j] = source->fisher_evectr[i][j];
        }
    }
    free_source(source);
    free_noise(noise);
    free(data);
}

/* A WDM grid of NF layers x NT pixels with a hand-filled struct Wavelets: the
 * reference's initialize_wavelet (utils/src/glass_wavelet.c:210) fixes
 * NF = 1536; the transforms themselves only read NF, NT and the window. */
static void ref_wdm_grid(struct Wavelets *w, int NF, int NT)
{
    memset(w, 0, sizeof(*w));
    w->NF = NF;
    w->NT = NT;
    w->A = 0.0;
    w->window_freq_forward = malloc(sizeof(double) * (NT / 2 + 1));
    build_wdm_filter_freq(w->window_freq_forward, NF, NT, 0.0, true);
}

/* utils/src/glass_wavelet.c:327 */
void ref_wdm_window(int NF, int NT, double A, int forward, double *out)
{
    build_wdm_filter_freq(out, NF, NT, A, forward != 0);
}

/* utils/src/glass_wavelet.c:293: wavelet_transform_timefreq (time overwritten) */
void ref_wdm_forward(int NF, int NT, double *time, double *wdm)
{
    struct Wavelets w;
    ref_wdm_grid(&w, NF, NT);
    wavelet_transform_timefreq(&w, time);
    memcpy(wdm, time, sizeof(double) * NF * NT);
    free(w.window_freq_forward);
}

/* utils/src/glass_wavelet.c:351 + utils/src/glass_math.c:819 */
void ref_wdm_inverse(int NF, int NT, double *wdm, double *time)
{
    struct Wavelets w;
    ref_wdm_grid(&w, NF, NT);
    double *freq = malloc(sizeof(double) * (NF * NT + 2));
    wavelet_transform_inverse_freq(&w, wdm, freq);
    glass_inverse_real_fft_outplace(freq, time, NF * NT);
    free(freq);
    free(w.window_freq_forward);
}

/* utils/src/glass_wavelet.c:544 with the grid's forward window */
void ref_wdm_by_layers(int NF, int NT, int jmin, int Nlayers, double *timedata)
{
    struct Wavelets w;
    ref_wdm_grid(&w, NF, NT);
    wavelet_transform_timefreq_by_layers(&w, jmin, Nlayers, w.window_freq_forward, timedata);
    free(w.window_freq_forward);
}

/* ucb/src/glass_ucb_waveform.c:1061 with interpolated analytic orbits
 * (utils/src/glass_lisa.c:271) and a hand-filled WDM grid (A = 0): X, Y, Z
 * are indexed by k - kmin and must be zeroed by the caller; returns Nwavelet. */
int ref_ucb_waveform_wavelet(double Tobs, double t0, double *params, int NF, int NT, double dt, double df,
                             int kmin, int kmax, int *list, double *X, double *Y, double *Z)
{
    struct Orbit *orbit = calloc(1, sizeof(struct Orbit));
    initialize_interpolated_analytic_orbits(orbit, Tobs, t0);
    struct Wavelets w;
    memset(&w, 0, sizeof(w));
    w.NF = NF;
    w.NT = NT;
    w.dt = dt;
    w.df = df;
    w.A = 0.0;
    w.kmin = kmin;
    w.kmax = kmax;
    int n = 0;
    ucb_waveform_wavelet(orbit, &w, Tobs, t0, params, list, &n, X, Y, Z);
    free_orbit(orbit);
    return n;
}

/*
 * ucb_fisher_wavelet (ucb/src/glass_ucb_waveform.c:524) on one source of a
 * hand-filled wavelet grid (A = 0) with interpolated analytic orbits:
 * invC[(3 i + j) N + k] the per-pixel inverse noise covariance of the N =
 * kmax - kmin pixels, F[64] row-major.  Returns 0, or 1 when the reference
 * regularised the matrix (an eigenvalue <= 0).
 */
int ref_ucb_fisher_wavelet(double Tobs, double t0, double *params, int NF, int NT, double dt, double df,
                           int kmin, int kmax, int imin, int imax, const double *invC, double *F)
{
    struct Orbit *orbit = calloc(1, sizeof(struct Orbit));
    initialize_interpolated_analytic_orbits(orbit, Tobs, t0);
    struct Wavelets w;
    memset(&w, 0, sizeof(w));
    w.NF = NF;
    w.NT = NT;
    w.dt = dt;
    w.df = df;
    w.A = 0.0;
    w.kmin = kmin;
    w.kmax = kmax;
    w.imin = imin;
    w.imax = imax;
    const int N = kmax - kmin;
    struct Data *data = calloc(1, sizeof(struct Data));
    data->N = N;
    data->Nchannel = 3;
    data->T = Tobs;
    data->t0 = t0;
    data->wdm = &w;
    struct Noise *noise = malloc(sizeof(struct Noise));
    alloc_noise(noise, N, 1, 3);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < N; k++) {
                noise->invC[i][j][k] = invC[(3 * i + j) * N + k];
                noise->C[i][j][k] = i == j ? 1.0 / invC[(3 * i + j) * N + k] : 0.0;
            }
    struct Source *source = malloc(sizeof(struct Source));
    alloc_source(source, N, UCB_MODEL_NP, 3);
    for (int p = 0; p < UCB_MODEL_NP; p++) source->params[p] = params[p];
    map_array_to_ucb_params(source, source->params, Tobs);
    ucb_fisher_wavelet(orbit, data, source, noise);
    int reg = 0;
    for (int i = 0; i < UCB_MODEL_NP; i++) {
        if (!(source->fisher_evalue[i] > 0)) reg = 1;
        for (int j = 0; j < UCB_MODEL_NP; j++) F[i * UCB_MODEL_NP + j] = source->fisher_matrix[i][j];
    }
    free_source(source);
    free_noise(noise);
    free(data);
    free_orbit(orbit);
    return reg;
}

/* orbit node times and positions of initialize_interpolated_analytic_orbits:
 * t[Norb], pos[(3 s + d) Norb + n]; returns Norb */
int ref_orbit_grid(double Tobs, double t0, double *t, double *pos)
{
    struct Orbit *orbit = calloc(1, sizeof(struct Orbit));
    initialize_interpolated_analytic_orbits(orbit, Tobs, t0);
    int n = orbit->Norb;
    if (t) {
        for (int k = 0; k < n; k++) {
            t[k] = orbit->t[k];
            for (int s = 0; s < 3; s++) {
                pos[(3 * s + 0) * n + k] = orbit->x[s][k];
                pos[(3 * s + 1) * n + k] = orbit->y[s][k];
                pos[(3 * s + 2) * n + k] = orbit->z[s][k];
            }
        }
    }
    free_orbit(orbit);
    return n;
}

static struct Noise *ref_wavelet_noise(int N, double *invC)
{
    struct Noise *noise = calloc(1, sizeof(struct Noise));
    noise->N = N;
    noise->invC = malloc(sizeof(double **) * 3);
    for (int i = 0; i < 3; i++) {
        noise->invC[i] = malloc(sizeof(double *) * 3);
        for (int j = 0; j < 3; j++) noise->invC[i][j] = invC + (3 * i + j) * N;
    }
    return noise;
}

static void ref_wavelet_noise_free(struct Noise *noise)
{
    for (int i = 0; i < 3; i++) free(noise->invC[i]);
    free(noise->invC);
    free(noise);
}

static struct TDI *ref_tdi_view(int N, double *xyz)
{
    struct TDI *t = calloc(1, sizeof(struct TDI));
    t->N = N;
    t->Nchannel = 3;
    t->X = xyz;
    t->Y = xyz + N;
    t->Z = xyz + 2 * N;
    return t;
}

/* utils/src/glass_model.c:624 for one-source models x and y: d, hx, hy are 3
 * channels of N pixels, invC 9 arrays of N pixels ([i][j][k]) */
double ref_wavelet_delta_logl(int N, double *d, double *invC, double *hx, int *lx, int nx, double *hy, int *ly,
                              int ny)
{
    struct Data data;
    memset(&data, 0, sizeof(data));
    data.N = N;
    data.tdi = ref_tdi_view(N, d);
    struct Noise *noise = ref_wavelet_noise(N, invC);
    struct Model mx, my;
    memset(&mx, 0, sizeof(mx));
    memset(&my, 0, sizeof(my));
    mx.tdi = ref_tdi_view(N, hx);
    my.tdi = ref_tdi_view(N, hy);
    mx.noise = my.noise = noise;
    mx.list = lx;
    mx.Nlist = nx;
    my.list = ly;
    my.Nlist = ny;
    double r = delta_log_likelihood(&data, &mx, &my);
    free(data.tdi);
    free(mx.tdi);
    free(my.tdi);
    ref_wavelet_noise_free(noise);
    return r;
}

/* utils/src/glass_model.c:805 on a wavelet segment of N pixels starting at
 * kmin, grid of NT pixels per layer, edge buffer [imin, imax] */
double ref_wavelet_logl_full(int N, int NT, int kmin, int imin, int imax, double *d, double *h, int *list, int n,
                             double *invC)
{
    struct Wavelets w;
    memset(&w, 0, sizeof(w));
    w.NT = NT;
    w.kmin = kmin;
    w.imin = imin;
    w.imax = imax;
    struct Data data;
    memset(&data, 0, sizeof(data));
    data.N = N;
    data.tdi = ref_tdi_view(N, d);
    data.wdm = &w;
    double *res = malloc(sizeof(double) * 3 * N);
    struct Model m;
    memset(&m, 0, sizeof(m));
    m.tdi = ref_tdi_view(N, h);
    m.residual = ref_tdi_view(N, res);
    m.noise = ref_wavelet_noise(N, invC);
    m.list = list;
    m.Nlist = n;
    double r = gaussian_log_likelhood_wavelet(&data, &m);
    free(data.tdi);
    free(m.tdi);
    free(m.residual);
    free(res);
    ref_wavelet_noise_free(m.noise);
    return r;
}

/* utils/src/glass_math.c:428 */
double ref_wavelet_snr(int N, double *h, int *list, int n, double *invC)
{
    struct Source s;
    memset(&s, 0, sizeof(s));
    s.tdi = ref_tdi_view(N, h);
    s.list = list;
    s.Nlist = n;
    struct Noise *noise = ref_wavelet_noise(N, invC);
    double r = snr_wavelet(&s, noise);
    free(s.tdi);
    ref_wavelet_noise_free(noise);
    return r;
}

/* A one-segment struct Data for the F-statistic (ucb/src/glass_ucb_fstatistic.c
 * reads T, t0, NFFT, fmin, format, dft->X/A/E and noise->C[0][0]); the X
 * channel of the data is zero.  fmin is qmin/T, raised by an ulp where needed
 * so that (int)(fmin T) == qmin as in utils/src/glass_data.c:1078. */
static struct Data *fstat_data(const char *format, double T, double t0, int NFFT, int qmin, const double *dA,
                               const double *dE, const double *invCA)
{
    struct Data *data = calloc(1, sizeof(struct Data));
    data->NFFT = NFFT;
    data->N = 2 * NFFT;
    data->Nchannel = 2;
    data->Nlayer = 1;
    data->T = T;
    data->sqT = sqrt(T);
    data->t0 = t0;
    data->fmin = (double)qmin / T;
    while ((int)(data->fmin * T) < qmin) data->fmin = nextafter(data->fmin, INFINITY);
    data->fmax = data->fmin + NFFT / T;
    data->qmin = (int)(data->fmin * T);
    data->qmax = data->qmin + NFFT;
    strcpy(data->format, format);
    strcpy(data->basis, "fourier");
    data->dft = malloc(sizeof(struct TDI));
    alloc_tdi(data->dft, data->N, 3);
    memcpy(data->dft->A, dA, sizeof(double) * data->N);
    memcpy(data->dft->E, dE, sizeof(double) * data->N);
    data->noise = malloc(sizeof(struct Noise));
    alloc_noise(data->noise, NFFT, 1, 2);
    for (int n = 0; n < NFFT; n++) {
        data->noise->invC[0][0][n] = invCA[n];
        data->noise->C[0][0][n] = 1.0 / invCA[n];
        data->noise->invC[1][1][n] = invCA[n];
        data->noise->C[1][1][n] = 1.0 / invCA[n];
    }
    return data;
}

static void fstat_data_free(struct Data *data)
{
    free_tdi(data->dft);
    free_noise(data->noise);
    free(data);
}

/* ucb/src/glass_ucb_fstatistic.c:646 (get_Fstat_logL) for n cells
 * (f0, fdot, theta, phi); out[6 c ..] = logL_X, logL_AE, Fparams[0..3]. */
void ref_fstat_logl(const char *format, double T, double t0, int NFFT, int qmin, const double *dA, const double *dE,
                    const double *invCA, int n, const double *cells, double *out)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    struct Data *data = fstat_data(format, T, t0, NFFT, qmin, dA, dE, invCA);
    for (int c = 0; c < n; c++) {
        const double *x = cells + 4 * c;
        double *o = out + 6 * c;
        get_Fstat_logL(&orbit, data, x[0], x[1], x[2], x[3], &o[0], &o[1], o + 2);
    }
    fstat_data_free(data);
}

/* ucb/src/glass_ucb_proposal.c:1085 (build_fstatistic_proposal) with the grid
 * of setup_fstatistic_proposal (:927-971) at n_theta x n_phi sky cells.
 * tensor: n_f n_theta n_phi doubles; info = {n_f, norm, maxp}. */
void ref_fstat_proposal(const char *format, double T, double t0, int NFFT, int qmin, const double *dA,
                        const double *dE, const double *invCA, int n_theta, int n_phi, double *tensor, double *info)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    struct Data *data = fstat_data(format, T, t0, NFFT, qmin, dA, dE, invCA);
    struct Flags flags;
    memset(&flags, 0, sizeof(flags));
    flags.quiet = 1;
    flags.threads = 1;
    int n_f = (int)((data->fmax - data->fmin) * data->T);
    struct Proposal proposal;
    memset(&proposal, 0, sizeof(proposal));
    proposal.matrix = malloc(3 * sizeof(double *));
    for (int i = 0; i < 3; i++) proposal.matrix[i] = calloc(2, sizeof(double));
    proposal.matrix[0][0] = (double)n_f;
    proposal.matrix[0][1] = (int)((data->fmax - data->fmin) * data->T) / (double)n_f / data->T;
    proposal.matrix[1][0] = (double)n_theta;
    proposal.matrix[1][1] = 2. / (double)n_theta;
    proposal.matrix[2][0] = (double)n_phi;
    proposal.matrix[2][1] = PI2 / (double)n_phi;
    proposal.tensor = malloc(n_f * sizeof(double **));
    for (int i = 0; i < n_f; i++) {
        proposal.tensor[i] = malloc(n_theta * sizeof(double *));
        for (int j = 0; j < n_theta; j++) proposal.tensor[i][j] = calloc(n_phi, sizeof(double));
    }
    build_fstatistic_proposal(&orbit, data, &flags, &proposal);
    for (int i = 0; i < n_f; i++) {
        for (int j = 0; j < n_theta; j++) {
            for (int k = 0; k < n_phi; k++) tensor[((size_t)i * n_theta + j) * n_phi + k] = proposal.tensor[i][j][k];
            free(proposal.tensor[i][j]);
        }
        free(proposal.tensor[i]);
    }
    free(proposal.tensor);
    info[0] = n_f;
    info[1] = proposal.norm;
    info[2] = proposal.maxp;
    for (int i = 0; i < 3; i++) free(proposal.matrix[i]);
    free(proposal.matrix);
    fstat_data_free(data);
}

/* The noise module's XYZ likelihood for n noise models on the grid
 * f = fmin + k/T, k < NFFT (noise/src/glass_noise_model.c:1378-1403 for the
 * grid): generate_instrument_noise_model (:389), optionally
 * generate_galactic_foreground_model (:612) added by
 * generate_full_covariance_matrix (:894), invert_noise_covariance_matrix
 * (utils/src/glass_math.c:240) and my_noise_log_likelihood
 * (noise/src/glass_noise_model.c:1243), as noise_instrument_model_mcmc
 * combines them (noise/src/glass_noise_sampler.c:555-572).
 * inst[12 p ..] = sacc[6], soms[6]; sgal[5 p ..] or NULL. */
void ref_noise_logl(double T, double fmin, int NFFT, const double *X, const double *Y, const double *Z, int n,
                    const double *inst, const double *sgal, double *logl)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    struct Data *data = calloc(1, sizeof(struct Data));
    data->NFFT = NFFT;
    data->N = 2 * NFFT;
    data->Nchannel = 3;
    data->Nlayer = 1;
    data->T = T;
    data->fmin = fmin;
    strcpy(data->basis, "fourier");
    data->tdi = malloc(sizeof(struct TDI));
    alloc_tdi(data->tdi, data->N, 3);
    memcpy(data->tdi->X, X, sizeof(double) * data->N);
    memcpy(data->tdi->Y, Y, sizeof(double) * data->N);
    memcpy(data->tdi->Z, Z, sizeof(double) * data->N);
    struct InstrumentModel inst_model;
    memset(&inst_model, 0, sizeof(inst_model));
    alloc_instrument_model(&inst_model, NFFT, 1, 3);
    for (int k = 0; k < NFFT; k++) inst_model.psd->f[k] = data->fmin + (double)k / data->T;
    struct ForegroundModel gal;
    memset(&gal, 0, sizeof(gal));
    alloc_foreground_model(&gal, NFFT, 1, 3);
    for (int k = 0; k < NFFT; k++) gal.psd->f[k] = data->fmin + (double)k / data->T;
    struct Noise *psd = malloc(sizeof(struct Noise));
    alloc_noise(psd, NFFT, 1, 3);
    for (int p = 0; p < n; p++) {
        for (int l = 0; l < 6; l++) {
            inst_model.sacc[l] = inst[12 * p + l];
            inst_model.soms[l] = inst[12 * p + 6 + l];
        }
        generate_instrument_noise_model(&orbit, &inst_model);
        copy_Cij(inst_model.psd->C, psd->C, psd->Nchannel, psd->N);
        if (sgal) {
            for (int q = 0; q < 5; q++) gal.sgal[q] = sgal[5 * p + q];
            generate_galactic_foreground_model(&gal);
            generate_full_covariance_matrix(psd, gal.psd, 3);
        }
        invert_noise_covariance_matrix(psd);
        logl[p] = my_noise_log_likelihood(data, psd);
    }
    free_noise(psd);
    free_noise(inst_model.psd);
    free(inst_model.sacc);
    free(inst_model.soms);
    free_noise(gal.psd);
    free(gal.sgal);
    free_tdi(data->tdi);
    free(data);
}

/* ref_noise_logl for one channel (d0 = X) or two (d0, d1 = A, E): the
 * reference's instrument (+ foreground) covariance with Nchannel 1 or 2,
 * invert_noise_covariance_matrix and noise_log_likelihood. */
void ref_noise_logl_channels(int nch, double T, double fmin, int NFFT, const double *d0, const double *d1, int n,
                             const double *inst, const double *sgal, double *logl)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    struct Data *data = calloc(1, sizeof(struct Data));
    data->NFFT = NFFT;
    data->N = 2 * NFFT;
    data->Nchannel = nch;
    data->Nlayer = 1;
    data->T = T;
    data->fmin = fmin;
    strcpy(data->basis, "fourier");
    data->tdi = malloc(sizeof(struct TDI));
    alloc_tdi(data->tdi, data->N, nch);
    if (nch == 1) {
        memcpy(data->tdi->X, d0, sizeof(double) * data->N);
    } else {
        memcpy(data->tdi->A, d0, sizeof(double) * data->N);
        memcpy(data->tdi->E, d1, sizeof(double) * data->N);
    }
    struct InstrumentModel inst_model;
    memset(&inst_model, 0, sizeof(inst_model));
    alloc_instrument_model(&inst_model, NFFT, 1, nch);
    for (int k = 0; k < NFFT; k++) inst_model.psd->f[k] = data->fmin + (double)k / data->T;
    struct ForegroundModel gal;
    memset(&gal, 0, sizeof(gal));
    alloc_foreground_model(&gal, NFFT, 1, nch);
    for (int k = 0; k < NFFT; k++) gal.psd->f[k] = data->fmin + (double)k / data->T;
    struct Noise *psd = malloc(sizeof(struct Noise));
    alloc_noise(psd, NFFT, 1, nch);
    for (int p = 0; p < n; p++) {
        for (int l = 0; l < 6; l++) {
            inst_model.sacc[l] = inst[12 * p + l];
            inst_model.soms[l] = inst[12 * p + 6 + l];
        }
        generate_instrument_noise_model(&orbit, &inst_model);
        copy_Cij(inst_model.psd->C, psd->C, psd->Nchannel, psd->N);
        if (sgal) {
            for (int q = 0; q < 5; q++) gal.sgal[q] = sgal[5 * p + q];
            generate_galactic_foreground_model(&gal);
            generate_full_covariance_matrix(psd, gal.psd, nch);
        }
        invert_noise_covariance_matrix(psd);
        logl[p] = noise_log_likelihood(data, psd);
    }
    free_noise(psd);
    free_noise(inst_model.psd);
    free(inst_model.sacc);
    free(inst_model.soms);
    free_noise(gal.psd);
    free(gal.sgal);
    free_tdi(data->tdi);
    free(data);
}

/* The noise module's coarse-grained wavelet likelihood for n noise models on
 * layers lmin .. lmin + Nlayer - 1 of an NF x NT grid (pixel dt, layer df):
 * coarse_grain_wavelet_data (noise/src/glass_noise_model.c:1057) of the
 * wavelet data X, Y, Z (pixel i of layer j at i + j NT), then per model
 * generate_instrument_noise_model_wavelet (:561), for mode 1/2
 * generate_galactic_foreground_model_wavelet (:656), the stationary (:983,
 * modes 0/1) or modulated (:923, mode 2) coarse covariance,
 * invert_noise_covariance_matrix and my_noise_log_likelihood_wavelet_coarse
 * (:1211).  The modulation cache (6 x NT/Q: XX, YY, ZZ, XY, XZ, YZ) is given,
 * as galaxy_modulation_cache_for_Q (utils/src/glass_galaxy.c:773) would have
 * filled it. */
void ref_noise_wavelet_logl(int NF, int NT, double dt, double df, int lmin, int Nlayer, int Q, const double *X,
                            const double *Y, const double *Z, int mode, const double *mod, int n, const double *inst,
                            const double *sgal, double *logl, double *P_out)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    struct Wavelets wdm;
    memset(&wdm, 0, sizeof(wdm));
    wdm.NF = NF;
    wdm.NT = NT;
    wdm.dt = dt;
    wdm.df = df;
    wdm.kmin = lmin * NT;
    wdm.kmax = (lmin + Nlayer) * NT;
    struct Data *data = calloc(1, sizeof(struct Data));
    data->wdm = &wdm;
    data->Nchannel = 3;
    data->Nlayer = Nlayer;
    data->lmin = lmin;
    data->lmax = lmin + Nlayer;
    data->N = Nlayer * NT;
    data->NFFT = data->N / 2;
    data->T = NT * dt;
    strcpy(data->basis, "wavelet");
    data->tdi = malloc(sizeof(struct TDI));
    alloc_tdi(data->tdi, data->N, 3);
    memcpy(data->tdi->X, X, sizeof(double) * data->N);
    memcpy(data->tdi->Y, Y, sizeof(double) * data->N);
    memcpy(data->tdi->Z, Z, sizeof(double) * data->N);
    struct CoarseStats stats;
    alloc_coarse_stats(&stats, Nlayer, Q, NT);
    coarse_grain_wavelet_data(data, &stats);
    const int Ncoarse = NT / Q;
    const size_t Npix = (size_t)Nlayer * Ncoarse;
    if (P_out) {
        memcpy(P_out, stats.Pxx, sizeof(double) * Npix);
        memcpy(P_out + Npix, stats.Pyy, sizeof(double) * Npix);
        memcpy(P_out + 2 * Npix, stats.Pzz, sizeof(double) * Npix);
        memcpy(P_out + 3 * Npix, stats.Pxy, sizeof(double) * Npix);
        memcpy(P_out + 4 * Npix, stats.Pxz, sizeof(double) * Npix);
        memcpy(P_out + 5 * Npix, stats.Pyz, sizeof(double) * Npix);
    }
    struct InstrumentModel im;
    memset(&im, 0, sizeof(im));
    alloc_instrument_model(&im, Nlayer, Nlayer, 3);
    for (int k = 0; k < Nlayer; k++) im.psd->f[k] = (lmin + k) * df;
    struct ForegroundModel conf;
    memset(&conf, 0, sizeof(conf));
    alloc_foreground_model(&conf, Nlayer, Nlayer, 3);
    for (int k = 0; k < Nlayer; k++) conf.psd->f[k] = (lmin + k) * df;
    conf.Tobs = data->T;
    struct GalaxyModulation gm;
    memset(&gm, 0, sizeof(gm));
    gm.Q_cached = Q;
    gm.Nt_cached = Ncoarse;
    gm.Nt_alloc = Ncoarse;
    if (mod) {
        gm.cache_XX = (double *)mod;
        gm.cache_YY = (double *)mod + Ncoarse;
        gm.cache_ZZ = (double *)mod + 2 * Ncoarse;
        gm.cache_XY = (double *)mod + 3 * Ncoarse;
        gm.cache_XZ = (double *)mod + 4 * Ncoarse;
        gm.cache_YZ = (double *)mod + 5 * Ncoarse;
    }
    conf.modulation = &gm;
    struct Noise *coarse = malloc(sizeof(struct Noise));
    alloc_noise(coarse, (int)Npix, Nlayer, 3);
    for (int p = 0; p < n; p++) {
        for (int l = 0; l < 6; l++) {
            im.sacc[l] = inst[12 * p + l];
            im.soms[l] = inst[12 * p + 6 + l];
        }
        generate_instrument_noise_model_wavelet(&wdm, &orbit, &im);
        if (mode) {
            for (int q = 0; q < 5; q++) conf.sgal[q] = sgal[5 * p + q];
            generate_galactic_foreground_model_wavelet(&wdm, &conf);
        }
        if (mode == 2)
            generate_full_dynamic_covariance_matrix_coarse(&wdm, Q, &im, &conf, NULL, coarse);
        else
            generate_full_stationary_covariance_matrix_coarse(&wdm, Q, &im, mode ? &conf : NULL, NULL, coarse);
        invert_noise_covariance_matrix(coarse);
        logl[p] = my_noise_log_likelihood_wavelet_coarse(data, coarse, &stats);
    }
    free_noise(coarse);
    free_coarse_stats(&stats);
    free_tdi(data->tdi);
    free(data);
}

/* ------------------------------------------------------------ SGWB */
/* The reference reads the instrument's SGWB response from a table file
 * (alloc_pop_sgwb_response, noise/src/glass_noise_model.c:134-189: the row
 * count, then rows f, XX, YY, ZZ, XY, XZ, YZ).  The rows resp[7 i ..] are
 * written to a temporary file in that format and read back by it, so the
 * splines are the reference's own. */
extern struct SGWBResponse *global_SGWBResponse;

static struct SGWBResponse *ref_sgwb_response(int nresp, const double *resp)
{
    char name[] = "/tmp/glass_sgwb_respXXXXXX";
    int fd = mkstemp(name);
    if (fd < 0) return NULL;
    FILE *fp = fdopen(fd, "w");
    fprintf(fp, "%d\n", nresp);
    for (int i = 0; i < nresp; i++) {
        const double *r = resp + 7 * (size_t)i;
        fprintf(fp, "%.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", r[0], r[1], r[2], r[3], r[4], r[5], r[6]);
    }
    fclose(fp);
    struct SGWBResponse *R = calloc(1, sizeof(struct SGWBResponse));
    alloc_pop_sgwb_response(R, name);
    unlink(name);
    /* generate_sgwb_model_wavelet's grid model shares the response */
    global_SGWBResponse = R;
    return R;
}

static void ref_sgwb_init(struct SGWBModel *m, int type, struct SGWBResponse *R, int N)
{
    memset(m, 0, sizeof(*m));
    m->SGWB_type = (SGWB_t)type;
    m->Nparams = SGWB_TEMPLATE_NPARAMS[type];
    m->params = calloc(4, sizeof(double));
    m->psd = malloc(sizeof(struct Noise));
    alloc_noise(m->psd, N, 1, 3);
    m->R = R;
    m->grid_cache = NULL;
}

/* generate_sgwb_model (noise/src/glass_noise_model.c:778-842) on the
 * frequencies f[N]: C6[6 n ..] = xx, yy, zz, xy, xz, yz. */
void ref_sgwb_model(int type, const double *params, int nresp, const double *resp, int N, const double *f, double *C6)
{
    struct SGWBResponse *R = ref_sgwb_response(nresp, resp);
    struct SGWBModel m;
    ref_sgwb_init(&m, type, R, N);
    for (int q = 0; q < m.Nparams; q++) m.params[q] = params[q];
    for (int n = 0; n < N; n++) m.psd->f[n] = f[n];
    generate_sgwb_model(&m);
    for (int n = 0; n < N; n++) {
        double *o = C6 + 6 * (size_t)n;
        o[0] = m.psd->C[0][0][n]; o[1] = m.psd->C[1][1][n]; o[2] = m.psd->C[2][2][n];
        o[3] = m.psd->C[0][1][n]; o[4] = m.psd->C[0][2][n]; o[5] = m.psd->C[1][2][n];
    }
    free_noise(m.psd);
    free(m.params);
}

/* ref_noise_logl with the SGWB of template `type` (parameters sgwb[4 p ..],
 * the template's first 2, 3 or 4) added last, in the order
 * noise_instrument_model_mcmc combines the three
 * (noise/src/glass_noise_sampler.c:559-570). */
void ref_noise_logl_sgwb(double T, double fmin, int NFFT, const double *X, const double *Y, const double *Z, int n,
                         const double *inst, const double *sgal, int type, const double *sgwb, int nresp,
                         const double *resp, double *logl)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    struct SGWBResponse *R = ref_sgwb_response(nresp, resp);
    struct Data *data = calloc(1, sizeof(struct Data));
    data->NFFT = NFFT;
    data->N = 2 * NFFT;
    data->Nchannel = 3;
    data->Nlayer = 1;
    data->T = T;
    data->fmin = fmin;
    strcpy(data->basis, "fourier");
    data->tdi = malloc(sizeof(struct TDI));
    alloc_tdi(data->tdi, data->N, 3);
    memcpy(data->tdi->X, X, sizeof(double) * data->N);
    memcpy(data->tdi->Y, Y, sizeof(double) * data->N);
    memcpy(data->tdi->Z, Z, sizeof(double) * data->N);
    struct InstrumentModel inst_model;
    memset(&inst_model, 0, sizeof(inst_model));
    alloc_instrument_model(&inst_model, NFFT, 1, 3);
    struct ForegroundModel gal;
    memset(&gal, 0, sizeof(gal));
    alloc_foreground_model(&gal, NFFT, 1, 3);
    struct SGWBModel sg;
    ref_sgwb_init(&sg, type, R, NFFT);
    for (int k = 0; k < NFFT; k++)
        inst_model.psd->f[k] = gal.psd->f[k] = sg.psd->f[k] = data->fmin + (double)k / data->T;
    struct Noise *psd = malloc(sizeof(struct Noise));
    alloc_noise(psd, NFFT, 1, 3);
    for (int p = 0; p < n; p++) {
        for (int l = 0; l < 6; l++) {
            inst_model.sacc[l] = inst[12 * p + l];
            inst_model.soms[l] = inst[12 * p + 6 + l];
        }
        generate_instrument_noise_model(&orbit, &inst_model);
        copy_Cij(inst_model.psd->C, psd->C, psd->Nchannel, psd->N);
        if (sgal) {
            for (int q = 0; q < 5; q++) gal.sgal[q] = sgal[5 * p + q];
            generate_galactic_foreground_model(&gal);
            generate_full_covariance_matrix(psd, gal.psd, 3);
        }
        for (int q = 0; q < sg.Nparams; q++) sg.params[q] = sgwb[4 * p + q];
        generate_sgwb_model(&sg);
        generate_full_covariance_matrix(psd, sg.psd, 3);
        invert_noise_covariance_matrix(psd);
        logl[p] = my_noise_log_likelihood(data, psd);
    }
    free_noise(psd);
    free_noise(inst_model.psd);
    free(inst_model.sacc);
    free(inst_model.soms);
    free_noise(gal.psd);
    free(gal.sgal);
    free_noise(sg.psd);
    free(sg.params);
    free_tdi(data->tdi);
    free(data);
}

/* ref_noise_wavelet_logl with the SGWB of template `type` (sgwb[4 p ..]):
 * generate_sgwb_model_wavelet (noise/src/glass_noise_model.c:843-892) on the
 * layer centres, passed to the coarse covariance builders (:923, :983),
 * which add it last. */
void ref_noise_wavelet_logl_sgwb(int NF, int NT, double dt, double df, int lmin, int Nlayer, int Q, const double *X,
                                 const double *Y, const double *Z, int mode, const double *mod, int n,
                                 const double *inst, const double *sgal, int type, const double *sgwb, int nresp,
                                 const double *resp, double *logl)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    struct SGWBResponse *R = ref_sgwb_response(nresp, resp);
    struct Wavelets wdm;
    memset(&wdm, 0, sizeof(wdm));
    wdm.NF = NF;
    wdm.NT = NT;
    wdm.dt = dt;
    wdm.df = df;
    wdm.kmin = lmin * NT;
    wdm.kmax = (lmin + Nlayer) * NT;
    struct Data *data = calloc(1, sizeof(struct Data));
    data->wdm = &wdm;
    data->Nchannel = 3;
    data->Nlayer = Nlayer;
    data->lmin = lmin;
    data->lmax = lmin + Nlayer;
    data->N = Nlayer * NT;
    data->NFFT = data->N / 2;
    data->T = NT * dt;
    strcpy(data->basis, "wavelet");
    data->tdi = malloc(sizeof(struct TDI));
    alloc_tdi(data->tdi, data->N, 3);
    memcpy(data->tdi->X, X, sizeof(double) * data->N);
    memcpy(data->tdi->Y, Y, sizeof(double) * data->N);
    memcpy(data->tdi->Z, Z, sizeof(double) * data->N);
    struct CoarseStats stats;
    alloc_coarse_stats(&stats, Nlayer, Q, NT);
    coarse_grain_wavelet_data(data, &stats);
    const int Ncoarse = NT / Q;
    const size_t Npix = (size_t)Nlayer * Ncoarse;
    struct InstrumentModel im;
    memset(&im, 0, sizeof(im));
    alloc_instrument_model(&im, Nlayer, Nlayer, 3);
    struct ForegroundModel conf;
    memset(&conf, 0, sizeof(conf));
    alloc_foreground_model(&conf, Nlayer, Nlayer, 3);
    struct SGWBModel sg;
    ref_sgwb_init(&sg, type, R, Nlayer);
    for (int k = 0; k < Nlayer; k++) im.psd->f[k] = conf.psd->f[k] = sg.psd->f[k] = (lmin + k) * df;
    conf.Tobs = sg.Tobs = data->T;
    struct GalaxyModulation gm;
    memset(&gm, 0, sizeof(gm));
    gm.Q_cached = Q;
    gm.Nt_cached = Ncoarse;
    gm.Nt_alloc = Ncoarse;
    if (mod) {
        gm.cache_XX = (double *)mod;
        gm.cache_YY = (double *)mod + Ncoarse;
        gm.cache_ZZ = (double *)mod + 2 * Ncoarse;
        gm.cache_XY = (double *)mod + 3 * Ncoarse;
        gm.cache_XZ = (double *)mod + 4 * Ncoarse;
        gm.cache_YZ = (double *)mod + 5 * Ncoarse;
    }
    conf.modulation = &gm;
    struct Noise *coarse = malloc(sizeof(struct Noise));
    alloc_noise(coarse, (int)Npix, Nlayer, 3);
    for (int p = 0; p < n; p++) {
        for (int l = 0; l < 6; l++) {
            im.sacc[l] = inst[12 * p + l];
            im.soms[l] = inst[12 * p + 6 + l];
        }
        generate_instrument_noise_model_wavelet(&wdm, &orbit, &im);
        if (mode) {
            for (int q = 0; q < 5; q++) conf.sgal[q] = sgal[5 * p + q];
            generate_galactic_foreground_model_wavelet(&wdm, &conf);
        }
        for (int q = 0; q < sg.Nparams; q++) sg.params[q] = sgwb[4 * p + q];
        generate_sgwb_model_wavelet(&wdm, &sg);
        if (mode == 2)
            generate_full_dynamic_covariance_matrix_coarse(&wdm, Q, &im, &conf, &sg, coarse);
        else
            generate_full_stationary_covariance_matrix_coarse(&wdm, Q, &im, mode ? &conf : NULL, &sg, coarse);
        invert_noise_covariance_matrix(coarse);
        logl[p] = my_noise_log_likelihood_wavelet_coarse(data, coarse, &stats);
    }
    free_noise(coarse);
    free_coarse_stats(&stats);
    free_tdi(data->tdi);
    free(data);
}

/* The noise module's spline noise model (the one- and two-channel model of
 * noise_spline_model_mcmc / _rjmcmc, noise/src/glass_noise_sampler.c:133,
 * :232) for n models: control points knot_f[p kmax + k],
 * knot_C[(p nch + c) kmax + k] (k < nknots[p]) of each channel c, the
 * transfer floor transfer[NFFT] on the bins f = fmin + k/T;
 * generate_spline_noise_model (noise/src/glass_noise_model.c:366) and
 * noise_log_likelihood (:1104) on the data d0 (X, or A) and d1 (E), 2 NFFT
 * doubles each. */
void ref_spline_noise_logl(int nch, int NFFT, double T, double fmin, const double *d0, const double *d1,
                           const double *transfer, int n, int kmax, const int *nknots, const double *knot_f,
                           const double *knot_C, double *logl)
{
    struct Data *data = calloc(1, sizeof(struct Data));
    data->NFFT = NFFT;
    data->N = 2 * NFFT;
    data->Nchannel = nch;
    data->Nlayer = 1;
    data->T = T;
    data->fmin = fmin;
    strcpy(data->basis, "fourier");
    data->tdi = malloc(sizeof(struct TDI));
    alloc_tdi(data->tdi, data->N, nch);
    if (nch == 1) {
        memcpy(data->tdi->X, d0, sizeof(double) * data->N);
    } else {
        memcpy(data->tdi->A, d0, sizeof(double) * data->N);
        memcpy(data->tdi->E, d1, sizeof(double) * data->N);
    }
    for (int p = 0; p < n; p++) {
        struct SplineModel model;
        memset(&model, 0, sizeof(model));
        alloc_spline_model(&model, NFFT, 1, nch, nknots[p]);
        for (int k = 0; k < NFFT; k++) {
            model.psd->f[k] = fmin + (double)k / T;
            model.psd->transfer[k] = transfer[k];
        }
        for (int k = 0; k < nknots[p]; k++) {
            model.spline->f[k] = knot_f[(size_t)p * kmax + k];
            for (int c = 0; c < nch; c++) model.spline->C[c][c][k] = knot_C[((size_t)p * nch + c) * kmax + k];
        }
        generate_spline_noise_model(&model);
        logl[p] = noise_log_likelihood(data, model.psd);
        free_noise(model.psd);
        free_noise(model.spline);
    }
    free_tdi(data->tdi);
    free(data);
}

/* noise_model_mcmc's likelihood change (ucb/src/glass_ucb_sampler.c:29-73)
 * for n chains with one source each (params[8 c ..]) on one A/E segment:
 * generate_ucb_model, then for eta_x and eta_y (eta[4 c ..] = xA, xE, yA, yE)
 * generate_noise_model, gaussian_log_likelihood and
 * gaussian_log_likelihood_model_norm; out[c] = (logL + norm)(y) - (logL + norm)(x). */
void ref_noise_eta(const char *format, double T, double t0, int NFFT, int qmin, const double *dA, const double *dE,
                   const double *invCA, const double *invCE, int n, const double *params, const double *eta,
                   double *out)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    struct Data *data = calloc(1, sizeof(struct Data));
    data->NFFT = NFFT;
    data->N = 2 * NFFT;
    data->Nchannel = 2;
    data->Nlayer = 1;
    data->T = T;
    data->sqT = sqrt(T);
    data->t0 = t0;
    data->qmin = qmin;
    data->qmax = qmin + NFFT;
    data->fmin = qmin / T;
    data->fmax = (qmin + NFFT) / T;
    strcpy(data->format, format);
    strcpy(data->basis, "fourier");
    data->tdi = malloc(sizeof(struct TDI));
    alloc_tdi(data->tdi, data->N, data->Nchannel);
    memcpy(data->tdi->A, dA, sizeof(double) * data->N);
    memcpy(data->tdi->E, dE, sizeof(double) * data->N);
    data->noise = malloc(sizeof(struct Noise));
    alloc_noise(data->noise, NFFT, 1, 2);
    for (int k = 0; k < NFFT; k++) {
        data->noise->C[0][0][k] = 1.0 / invCA[k];
        data->noise->C[1][1][k] = 1.0 / invCE[k];
        data->noise->C[0][1][k] = data->noise->C[1][0][k] = 0.0;
        data->noise->invC[0][0][k] = invCA[k];
        data->noise->invC[1][1][k] = invCE[k];
    }
    struct Model *model = calloc(1, sizeof(struct Model));
    alloc_model(data, model, UCB_MODEL_NP, 1);
    model->Nlive = 1;
    model->t0 = t0;
    for (int c = 0; c < n; c++) {
        for (int p = 0; p < UCB_MODEL_NP; p++) model->source[0]->params[p] = params[c * UCB_MODEL_NP + p];
        for (int k = 0; k < NFFT; k++) {
            model->noise->invC[0][0][k] = invCA[k];
            model->noise->invC[1][1][k] = invCE[k];
            model->noise->C[0][0][k] = 1.0 / invCA[k];
            model->noise->C[1][1][k] = 1.0 / invCE[k];
        }
        generate_ucb_model(&orbit, data, model, -1);
        double tot[2];
        for (int w = 0; w < 2; w++) {
            model->noise->eta[0] = eta[4 * c + 2 * w];
            model->noise->eta[1] = eta[4 * c + 2 * w + 1];
            generate_noise_model(data, model);
            double logL = gaussian_log_likelihood(data, model);
            double norm = gaussian_log_likelihood_model_norm(data, model);
            tot[w] = logL + norm;
        }
        out[c] = tot[1] - tot[0];
    }
    free_model(model);
    free_noise(data->noise);
    free_tdi(data->tdi);
    free(data);
}

/* ptmcmc (utils/src/glass_sampler.c:19) on one ladder of NC chains whose
 * models hold logL and logLnorm; index, seed and acceptance are updated. */
void ref_ptmcmc(int NC, const double *temperature, const double *logL, const double *logLnorm, int *index,
                unsigned int *seed, double *acceptance)
{
    struct Chain chain;
    memset(&chain, 0, sizeof(chain));
    chain.NC = NC;
    chain.index = index;
    chain.temperature = (double *)temperature;
    chain.acceptance = acceptance;
    chain.r = seed;
    struct Model **model = malloc(sizeof(struct Model *) * NC);
    struct Model *m = calloc(NC, sizeof(struct Model));
    for (int c = 0; c < NC; c++) {
        m[c].logL = logL[c];
        m[c].logLnorm = logLnorm ? logLnorm[c] : 0.0;
        model[c] = &m[c];
    }
    struct Flags flags;
    memset(&flags, 0, sizeof(flags));
    ptmcmc(model, &chain, &flags);
    free(m);
    free(model);
}

/* The reference's draw_from_fisher (ucb/src/glass_ucb_proposal.c:348-391) on
 * one source: x[8], evec[64] (row j = fisher_evectr[j]), evalue[8]; returns
 * its value (0 or -inf) and writes the drawn parameters to y[8]. */
double ref_fisher_draw(const double *x, const double *evec, const double *evalue, unsigned int *seed, double *y)
{
    struct Source s;
    memset(&s, 0, sizeof(s));
    double params[8], val[8], rows[8][8];
    double *rowp[8];
    memcpy(params, x, sizeof(params));
    memcpy(val, evalue, sizeof(val));
    for (int j = 0; j < 8; j++) {
        memcpy(rows[j], evec + 8 * j, sizeof(rows[j]));
        rowp[j] = rows[j];
    }
    s.NP = 8;
    s.params = params;
    s.fisher_evalue = val;
    s.fisher_evectr = rowp;
    return draw_from_fisher(NULL, NULL, &s, NULL, y, seed);
}


/* draw_from_uniform_prior (utils/src/glass_sampler.c:96) with UCB_MODEL_NP
 * parameters: prior16[2 k + {0, 1}] the bounds, logPV8 the log volumes;
 * returns logQ, advances *seed. */
double ref_draw_uniform_prior(const double *prior16, const double *logPV8, unsigned int *seed, double *params)
{
    struct Model m;
    memset(&m, 0, sizeof(m));
    double *rows[UCB_MODEL_NP];
    for (int k = 0; k < UCB_MODEL_NP; k++) rows[k] = (double *)prior16 + 2 * k;
    m.NP = UCB_MODEL_NP;
    m.prior = rows;
    m.logPriorVolume = (double *)logPV8;
    return draw_from_uniform_prior(NULL, &m, NULL, NULL, params, seed);
}

/* evaluate_ucb_prior (ucb/src/glass_ucb_prior.c:536) without the catalogue
 * prior; galaxy != 0 uses skyhist[i nphi + j].  params may be wrapped in place. */
double ref_ucb_prior(double *params, const double *prior16, const double *logPV8, int galaxy, double *skyhist,
                     double dcostheta, double dphi, int nphi)
{
    struct Flags flags;
    memset(&flags, 0, sizeof(flags));
    flags.galaxyPrior = galaxy;
    struct Model m;
    memset(&m, 0, sizeof(m));
    double *rows[UCB_MODEL_NP];
    for (int k = 0; k < UCB_MODEL_NP; k++) rows[k] = (double *)prior16 + 2 * k;
    m.NP = UCB_MODEL_NP;
    m.prior = rows;
    m.logPriorVolume = (double *)logPV8;
    struct Prior pr;
    memset(&pr, 0, sizeof(pr));
    pr.skyhist = skyhist;
    pr.dcostheta = dcostheta;
    pr.dphi = dphi;
    pr.nphi = nphi;
    return evaluate_ucb_prior(&flags, NULL, &m, &pr, params);
}

/* ------------------------------------------------------------------------
 * ucb_rjmcmc (ucb/src/glass_ucb_sampler.c:454) for NC chains on one A/E
 * segment, nsteps successive calls per chain, with the prior (proposal 0)
 * and F-statistic (proposal 1) draws of the reference's cocktail
 * (rjweight[9]) and an F-statistic grid given as input.  The model's
 * likelihood and signal generator are the reference's own
 * (gaussian_log_likelihood, generate_ucb_model), wrapped to record, per call,
 * the proposed state's logL (NaN when not evaluated) and, for a birth whose
 * template was generated, the new source's parameters and SNR.
 * In/out: Nlive[NC], src[(c maxsrc + s) 8 ..], seed[NC].  Out per step k and
 * chain c (index k NC + c): rec_gen, rec_params[8], rec_snr, rec_logLy,
 * and after the call logL, Nlive and seed; logL0[NC] the starting logL.
 */
static int g_rec_gen, g_rec_eval;
static double g_rec_snr, g_rec_logL, g_rec_params[UCB_MODEL_NP];

static double rec_log_likelihood(struct Data *data, struct Model *model)
{
    double l = gaussian_log_likelihood(data, model);
    g_rec_eval = 1;
    g_rec_logL = l;
    return l;
}

static void rec_generate(struct Orbit *orbit, struct Data *data, struct Model *model, int source_id)
{
    generate_ucb_model(orbit, data, model, source_id);
    if (source_id >= 0) {
        g_rec_gen = 1;
        g_rec_snr = snr(model->source[source_id], model->noise);
        for (int p = 0; p < UCB_MODEL_NP; p++) g_rec_params[p] = model->source[source_id]->params[p];
    }
}

void ref_rj_steps(const char *format, double T, double t0, int NFFT, int qmin, const double *dA, const double *dE,
                  const double *invCA, const double *invCE, int NC, int maxsrc, const int *Neff, int *Nlive,
                  double *src, const double *prior16, const double *logPV8, const double *rjw, const double *tensor,
                  int nf, int nt, int np, double df, double dt, double dp, double maxp, const double *temperature,
                  unsigned int *seed, int nsteps, double *logL0, int *rec_gen, double *rec_params, double *rec_snr,
                  double *rec_logLy, double *logL_after, int *Nlive_after, unsigned int *seed_after)
{
    struct Orbit orbit;
    setup_orbit(&orbit);
    struct Data *data = calloc(1, sizeof(struct Data));
    data->NFFT = NFFT;
    data->N = 2 * NFFT;
    data->Nchannel = 2;
    data->Nlayer = 1;
    data->T = T;
    data->sqT = sqrt(T);
    data->t0 = t0;
    data->qmin = qmin;
    data->qmax = qmin + NFFT;
    data->fmin = qmin / T;
    data->fmax = (qmin + NFFT) / T;
    strcpy(data->format, format);
    strcpy(data->basis, "fourier");
    data->tdi = malloc(sizeof(struct TDI));
    alloc_tdi(data->tdi, data->N, data->Nchannel);
    memcpy(data->tdi->A, dA, sizeof(double) * data->N);
    memcpy(data->tdi->E, dE, sizeof(double) * data->N);
    data->noise = malloc(sizeof(struct Noise));
    alloc_noise(data->noise, NFFT, 1, 2);
    for (int n = 0; n < NFFT; n++) {
        data->noise->invC[0][0][n] = invCA[n];
        data->noise->invC[1][1][n] = invCE[n];
        data->noise->C[0][0][n] = 1.0 / invCA[n];
        data->noise->C[1][1][n] = 1.0 / invCE[n];
    }

    struct Flags *flags = calloc(1, sizeof(struct Flags));
    struct Prior *prior = calloc(1, sizeof(struct Prior));
    struct Chain *chain = calloc(1, sizeof(struct Chain));
    chain->NC = NC;
    chain->r = malloc(sizeof(unsigned int) * NC);
    chain->temperature = malloc(sizeof(double) * NC);
    for (int c = 0; c < NC; c++) {
        chain->r[c] = seed[c];
        chain->temperature[c] = temperature[c];
    }

    double ***ten = malloc(sizeof(double **) * nf);
    for (int i = 0; i < nf; i++) {
        ten[i] = malloc(sizeof(double *) * nt);
        for (int j = 0; j < nt; j++) ten[i][j] = (double *)tensor + ((size_t)i * nt + j) * np;
    }
    double *mrow[3];
    double mval[3][2] = {{nf, df}, {nt, dt}, {np, dp}};
    for (int r = 0; r < 3; r++) mrow[r] = mval[r];
    struct Proposal **prop = malloc(sizeof(struct Proposal *) * UCB_PROPOSAL_NPROP);
    for (int k = 0; k < UCB_PROPOSAL_NPROP; k++) {
        prop[k] = calloc(1, sizeof(struct Proposal));
        prop[k]->trial = calloc(NC, sizeof(int));
        prop[k]->accept = calloc(NC, sizeof(int));
        prop[k]->rjweight = rjw[k];
        prop[k]->function = &draw_from_uniform_prior;
        prop[k]->density = &uniform_prior_density;
    }
    prop[1]->function = &draw_from_fstatistic;
    prop[1]->density = &evaluate_fstatistic_proposal;
    prop[1]->matrix = mrow;
    prop[1]->tensor = ten;
    prop[1]->maxp = maxp;

    struct Model **model = malloc(sizeof(struct Model *) * NC), **trial = malloc(sizeof(struct Model *) * NC);
    for (int c = 0; c < NC; c++) {
        struct Model *pair[2];
        for (int w = 0; w < 2; w++) {
            struct Model *m = calloc(1, sizeof(struct Model));
            alloc_model(data, m, UCB_MODEL_NP, maxsrc);
            m->Neff = Neff[c];
            m->t0 = t0;
            m->log_likelihood = &rec_log_likelihood;
            m->generate_signal_model = &rec_generate;
            for (int k = 0; k < UCB_MODEL_NP; k++) {
                m->prior[k][0] = prior16[2 * k];
                m->prior[k][1] = prior16[2 * k + 1];
                m->logPriorVolume[k] = logPV8[k];
            }
            for (int n = 0; n < NFFT; n++) {
                m->noise->invC[0][0][n] = invCA[n];
                m->noise->invC[1][1][n] = invCE[n];
                m->noise->C[0][0][n] = 1.0 / invCA[n];
                m->noise->C[1][1][n] = 1.0 / invCE[n];
            }
            pair[w] = m;
        }
        model[c] = pair[0];
        trial[c] = pair[1];
        model[c]->Nlive = Nlive[c];
        for (int s = 0; s < Nlive[c]; s++)
            for (int p = 0; p < UCB_MODEL_NP; p++)
                model[c]->source[s]->params[p] = src[((size_t)c * maxsrc + s) * 8 + p];
        generate_ucb_model(&orbit, data, model[c], -1);
        model[c]->logL = gaussian_log_likelihood(data, model[c]);
        logL0[c] = model[c]->logL;
    }

    for (int k = 0; k < nsteps; k++) {
        for (int c = 0; c < NC; c++) {
            size_t o = (size_t)k * NC + c;
            g_rec_gen = g_rec_eval = 0;
            g_rec_snr = NAN;
            g_rec_logL = NAN;
            ucb_rjmcmc(&orbit, data, model[c], trial[c], chain, flags, prior, prop, c);
            rec_gen[o] = g_rec_gen;
            rec_snr[o] = g_rec_gen ? g_rec_snr : NAN;
            for (int p = 0; p < 8; p++) rec_params[8 * o + p] = g_rec_gen ? g_rec_params[p] : NAN;
            rec_logLy[o] = g_rec_eval ? g_rec_logL : NAN;
            logL_after[o] = model[c]->logL;
            Nlive_after[o] = model[c]->Nlive;
            seed_after[o] = chain->r[c];
        }
    }
    for (int c = 0; c < NC; c++) {
        Nlive[c] = model[c]->Nlive;
        seed[c] = chain->r[c];
        for (int s = 0; s < maxsrc; s++)
            for (int p = 0; p < 8; p++)
                src[((size_t)c * maxsrc + s) * 8 + p] = s < model[c]->Nlive ? model[c]->source[s]->params[p] : 0.0;
        free_model(model[c]);
        free_model(trial[c]);
    }
    free(model);
    free(trial);
    for (int k = 0; k < UCB_PROPOSAL_NPROP; k++) {
        free(prop[k]->trial);
        free(prop[k]->accept);
        free(prop[k]);
    }
    free(prop);
    for (int i = 0; i < nf; i++) free(ten[i]);
    free(ten);
    free(chain->r);
    free(chain->temperature);
    free(chain);
    free(prior);
    free(flags);
    free_noise(data->noise);
    free_tdi(data->tdi);
    free(data);
}
