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
