/*
 * glass_gb300.h -- C ABI of the GB300 UCB likelihood engine.
 *
 * Two groups of entry points:
 *
 *  1. Drop-in replacements that keep the reference's own signatures, so the
 *     GLASS apps (ucb_mcmc, ucb_wavelet_mcmc, global_fit) link against this
 *     library instead of the reference's object files.  They take host
 *     pointers, run on the calling thread's own CUDA stream and return when
 *     the results are back in host memory.
 *
 *  2. Batched entry points (glass_gpu_*) that evaluate many proposals per
 *     call on device-resident data: plain pointers and sizes, an int status,
 *     no CPU fallback.
 *
 * Every function is thread-safe.  Contexts are not shared between threads
 * unless the caller serialises their use.
 */
#ifndef GLASS_GB300_H
#define GLASS_GB300_H

#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define GLASS_OK 0
#define GLASS_ERR_ARG -1      /* null pointer, bad count, bad enum value */
#define GLASS_ERR_SIZE -2     /* waveform size outside 32..4096 or not a power of two */
#define GLASS_ERR_CUDA -3     /* a CUDA call failed; see glass_gpu_last_error() */
#define GLASS_ERR_FORMAT -4   /* unknown TDI format string */
#define GLASS_ERR_STATE -5    /* no segment bank uploaded yet */

/* per-item status bits written by the batched kernels */
#define GLASS_ITEM_OK 0
#define GLASS_ITEM_NONFINITE 1     /* a parameter was NaN/Inf, or a result was */
#define GLASS_ITEM_BAD_SEGMENT 2   /* segment index out of range */
#define GLASS_ITEM_OUTSIDE 4       /* template support does not overlap the segment */

/* precision of a batched evaluation */
#define GLASS_PREC_FP64 0   /* plain FP64 throughout */
#define GLASS_PREC_MIXED 1  /* FP32 waveform and inner products, FP64/double-float phase */

/* TDI conventions, as the reference's `format` strings */
#define GLASS_FMT_SANGRIA 0   /* "sangria"   utils/src/glass_lisa.c:645 */
#define GLASS_FMT_PHASE 1     /* "phase"     utils/src/glass_lisa.c:458 */
#define GLASS_FMT_FREQUENCY 2 /* "frequency" utils/src/glass_lisa.c:551 */

/* ------------------------------------------------ drop-in (reference ABI) */
struct Orbit; /* utils/src/glass_lisa.h:60-109; read: L, fstar, orbit_function (ucb_waveform), Norb, t, x, y, z
                 (ucb_waveform_wavelet) */
struct Wavelets; /* utils/src/glass_wavelet.h:25-75; read: NF, NT, dt, df, A, kmin, kmax */

/*
 * Replaces ucb_waveform (ucb/src/glass_ucb_waveform.h:210,
 * ucb/src/glass_ucb_waveform.c:738-1001).  Same arguments and outputs:
 * X,Y,Z,A,E receive 2*BW doubles each (re/im interleaved); for the "phase" and
 * "frequency" formats with NI == 1 only X is written.  Spacecraft positions
 * come from orbit->orbit_function, evaluated on the host at the BW sample
 * times, so analytic and tabulated orbits both work.  BW must be a power of
 * two in [32, 4096].  As in the reference, an unsupported format string
 * prints a message and exits the process; so does a device error.
 */
void ucb_waveform(struct Orbit *orbit, char *format, double T, double t0, double *params, int NParams, double *X,
                  double *Y, double *Z, double *A, double *E, int BW, int NI);

/* Status-returning form of ucb_waveform for callers that handle errors. */
int glass_ucb_waveform(const double *orbit_xyz, const char *format, double T, double t0, const double *params,
                       int NParams, double *X, double *Y, double *Z, double *A, double *E, int BW, int NI);

/*
 * Replaces ucb_bandwidth (ucb/src/glass_ucb_waveform.h:185,
 * ucb/src/glass_ucb_waveform.c:698-725): the number of slow-part samples N/2
 * the reference picks for a source (a power of two in [16, Nmax]).
 */
int ucb_bandwidth(double L, double fstar, double f, double fdot, double costheta, double A, double T, int N);

/* ----------------------------- drop-ins for the model and likelihood headers */
struct Data;   /* utils/src/glass_data.h:50-97; read: N, NFFT, Nchannel, T, t0, qmin, tdi, format */
struct Source; /* utils/src/glass_model.h:81-121; read/written: params, tdi, f0 .. phiref, dfdt, BW, qmin,
                  qmax, imin, imax, fisher_matrix, fisher_evectr, fisher_evalue */
struct Model;  /* utils/src/glass_model.h:25-60; read: Nlive, source, noise, tdi, residual, t0 */
struct Noise;  /* utils/src/glass_data.h:337-360; read: invC */
/*
 * Same names, signatures and results as the reference (the structures'
 * layouts are the interface), so that ucb_mcmc links against this library:
 *   analytic_orbits, initialize_analytic_orbit  utils/src/glass_lisa.c:77, :125
 *   map_array_to_ucb_params  ucb/src/glass_ucb_model.c:25 (glass_ucb_model.h)
 *   ucb_alignment            ucb/src/glass_ucb_waveform.c:727 (glass_ucb_waveform.h:170)
 *   add_ucb_model, remove_ucb_model  ucb/src/glass_ucb_model.c:192, :149
 *   generate_ucb_model       ucb/src/glass_ucb_model.c:55 (glass_ucb_model.h:36)
 *   update_ucb_model         ucb/src/glass_ucb_model.c:271 (glass_ucb_model.h:45)
 *   fourier_nwip, snr        utils/src/glass_math.c:362, :403
 *   gaussian_log_likelihood  utils/src/glass_model.c:726
 *   matrix_eigenstuff        utils/src/glass_math.c:475
 *   ucb_fisher               ucb/src/glass_ucb_waveform.c:364 (glass_ucb_waveform.h:150)
 *   wavelet_nwip, snr_wavelet  utils/src/glass_math.c:382, :428 (glass_math.h:261)
 *   delta_log_likelihood     utils/src/glass_model.c:624 (glass_model.h:211), wavelet basis
 *   ucb_fisher_wavelet       ucb/src/glass_ucb_waveform.c:524 (glass_ucb_waveform.h:156)
 * Waveforms come from the GPU ucb_waveform above.  ucb_fisher takes its
 * Fisher matrix for A/E data from the adjoint kernels (glass_gpu_grad_fisher
 * _batch with the reference's noise indexing, fisher_mode 1; the segment's
 * noise is uploaded to the thread's context when it changes), and for X or
 * XYZ data from forward differences of the GPU waveform as the reference
 * does.  ucb_fisher_wavelet takes its Fisher matrix from the batched
 * wavelet Fisher kernels (glass_gpu_wavelet_fisher_batch: the reference's
 * central differences of the FP64 wavelet waveform) on the grid of
 * data->wdm, the segment of data (T, t0; data->N must be kmax - kmin) and the
 * nodes of the caller's orbit, weighted with noise->invC; then the
 * eigen-decomposition and, where an eigenvalue is not positive, the
 * reference's regularisation (0.1 added to the diagonal, decomposition
 * redone; still not positive: report and exit(1)).  The sums over a
 * segment's bins or a pixel list run on the caller's host arrays in
 * the reference's order of operations (bit-identical): a GPU launch per call
 * would cost more than the arithmetic.  matrix_eigenstuff: symmetric input
 * (the reference passes Fisher matrices to LAPACK's general solver);
 * eigenvector j is column j, unit length, pairs sorted by decreasing
 * eigenvalue with each vector's largest component positive (LAPACK's order
 * and signs are not reproduced).  Errors print the reason and exit(1).
 */
void analytic_orbits(struct Orbit *orbit, double t, double *x, double *y, double *z);
void initialize_analytic_orbit(struct Orbit *orbit);
void map_array_to_ucb_params(struct Source *source, double *params, double T);
void ucb_alignment(struct Orbit *orbit, struct Data *data, struct Source *source);
void add_ucb_model(struct Data *data, struct Model *model, struct Source *source);
void remove_ucb_model(struct Data *data, struct Model *model, struct Source *source);
void generate_ucb_model(struct Orbit *orbit, struct Data *data, struct Model *model, int source_id);
void update_ucb_model(struct Orbit *orbit, struct Data *data, struct Model *model_x, struct Model *model_y,
                      int source_id);
double fourier_nwip(const double *a, const double *b, const double *invC, int N);
double snr(struct Source *source, struct Noise *noise);
double gaussian_log_likelihood(struct Data *data, struct Model *model);
void matrix_eigenstuff(double **matrix, double **evectors, double *evalues, int N);
void ucb_fisher(struct Orbit *orbit, struct Data *data, struct Source *source, struct Noise *noise);
double wavelet_nwip(const double *a, const double *b, const double *invC, const int *list, int N);
double snr_wavelet(struct Source *source, struct Noise *noise);
double delta_log_likelihood(struct Data *data, struct Model *model_x, struct Model *model_y);
void ucb_fisher_wavelet(struct Orbit *orbit, struct Data *data, struct Source *source, struct Noise *noise);

/* ---------------------------------------------------------- batched API */
typedef struct glass_gpu_ctx glass_gpu_ctx;

/* Create a context on a CUDA device with its own non-blocking stream. */
int glass_gpu_create(int device, glass_gpu_ctx **ctx);
int glass_gpu_destroy(glass_gpu_ctx *ctx);
/* Run this context's work on a caller-owned cudaStream_t (NULL restores the
 * context's own stream). */
int glass_gpu_set_stream(glass_gpu_ctx *ctx, void *stream);
/* Last error message of this thread (never NULL). */
const char *glass_gpu_last_error(void);

/*
 * The checked build (libglass_gb300_checks.so: python -m glass_gb300.build
 * --checks; the stand-in for compute-sanitizer) checks the kernels' indexed
 * accesses (bank bins, series scratch, proposal indices, size lists, the
 * re-evaluation list, outputs) against the buffers' extents; a failed check
 * records its site and skips the access.  glass_gpu_checked_build() is 1 in
 * that library and 0 in the product one; glass_gpu_check_status synchronises
 * the context's stream and returns in *word the sites that failed since the
 * last call (bits: 1 bank read, 2 series read, 4 series write, 8 proposal
 * index, 16 size list, 32 re-evaluation list, 64 output; 0 in the product
 * library).
 */
int glass_gpu_checked_build(void);
int glass_gpu_check_status(glass_gpu_ctx *ctx, unsigned int *word);

/*
 * Upload a bank of `nseg` A/E frequency segments of NFFT bins each -- the
 * inputs the reference's gaussian_log_likelihood reads
 * (utils/src/glass_model.c:726-774, Nchannel == 2): for segment s,
 *   rA, rE   : residual (data minus every source not being proposed),
 *              2*NFFT doubles at offset s*2*NFFT, re/im interleaved
 *   invCA/E  : inverse noise PSD, NFFT doubles at offset s*NFFT
 *   qmin[s]  : first DFT bin of the segment (Data::qmin)
 * T and t0 are the observation length and the model start time (Model::t0).
 * Replaces any previous bank.  Host pointers; synchronous.
 */
int glass_gpu_bank_upload(glass_gpu_ctx *ctx, int format, double T, double t0, int NFFT, int nseg, const int *qmin,
                          const double *rA, const double *rE, const double *invCA, const double *invCE);

/* Template size of the batched evaluations: 0 (the default) takes N from the
 * reference's bandwidth rule (ucb_alignment, ucb/src/glass_ucb_waveform.c:727),
 * otherwise every proposal uses this N (a power of two in [32, min(4096,
 * NFFT)]), as a caller of ucb_waveform chooses BW. */
int glass_gpu_set_template_size(glass_gpu_ctx *ctx, int n);

/* Replace the residual of one segment (after an accepted move changed the
 * other sources of its chain).  Host pointers, 2*NFFT doubles each. */
int glass_gpu_bank_set_residual(glass_gpu_ctx *ctx, int seg, const double *rA, const double *rE);

/*
 * Batched proposal evaluation: for item i on segment item_seg[i] with
 * parameters params[8*i .. 8*i+7] (the reference's params array,
 * ucb/src/glass_ucb_model.c:40-53), compute
 *   term_y[i] = logL(residual - h_i) - logL(residual)
 * exactly as generate_ucb_model + gaussian_log_likelihood would
 * (ucb/src/glass_ucb_model.c:55-103, utils/src/glass_model.c:726-774), with
 * the template size from ucb_bandwidth and its placement from ucb_alignment
 * (ucb/src/glass_ucb_waveform.c:698-736), and
 *   dlogl[i]  = term_y[i] - term_x[i]       (term_x may be NULL: taken as 0)
 *   hh[i]     = (h_i|h_i) over the segment   (snr^2, utils/src/glass_math.c:403)
 *   status[i] = GLASS_ITEM_* bits            (may be NULL)
 * so dlogl is the sampler's delta logL (ucb/src/glass_ucb_sampler.c:155-160)
 * when term_x holds the current state's term_y.  All pointers are DEVICE
 * pointers; the call is asynchronous on the context's stream.
 */
int glass_gpu_dlogl_batch(glass_gpu_ctx *ctx, int precision, int nitems, const int *item_seg, const double *params,
                          const double *term_x, double *dlogl, double *term_y, double *hh, int *status);

/* Same as glass_gpu_dlogl_batch with HOST pointers: copies in, evaluates,
 * copies out and synchronises.  Two ways to move the data (see
 * glass_gpu_set_host_access): by default, where the device reads pageable
 * host memory in place through the host's page tables (a coherent CPU-GPU
 * link), a gather kernel reads the caller's arrays and a scatter kernel
 * writes the results into them; otherwise the inputs go through one pinned
 * staging buffer of the context (one copy each way).  Either sequence for a
 * batch shape (nitems, precision, term_x given or not) is recorded as a CUDA
 * graph on the first call and replayed on later calls of that shape; a new
 * bank, a new template size or larger buffers drop the recorded graphs.  Not
 * to be called while the context's stream is being captured.
 * In the in-place mode the GPU itself reads item_seg, params and term_x and
 * writes dlogl, term_y, hh and status: every array must be valid, mapped
 * memory of this process for nitems elements until the call returns.  A bad
 * pointer is then a GPU memory fault, not a host crash, and it leaves the
 * context (and every later call on it) in an error state; callers who want a
 * host-side fault for bad pointers select the staging copies with
 * glass_gpu_set_host_access(ctx, 0). */
int glass_gpu_dlogl_batch_host(glass_gpu_ctx *ctx, int precision, int nitems, const int *item_seg,
                               const double *params, const double *term_x, double *dlogl, double *term_y, double *hh,
                               int *status);

/* How glass_gpu_dlogl_batch_host moves host data: mode 1 reads and writes the
 * caller's arrays from the device in place (GLASS_ERR_STATE where the device
 * cannot: cudaDevAttrPageableMemoryAccess and
 * cudaDevAttrPageableMemoryAccessUsesHostPageTables both required), 0 copies
 * through pinned staging, -1 (the default) picks 1 where supported.  The
 * results are identical either way. */
int glass_gpu_set_host_access(glass_gpu_ctx *ctx, int mode);
/* supported: the device can access pageable host memory in place; direct: the
 * in-place path is in use (either may be NULL). */
int glass_gpu_get_host_access(glass_gpu_ctx *ctx, int *supported, int *direct);

/*
 * Gradient of delta logL and Fisher matrix of a batch of proposals, by tangent
 * propagation through the mixed-precision waveform; replaces the reference's
 * finite-difference ucb_fisher (ucb/src/glass_ucb_waveform.c:364-522,
 * declared at ucb/src/glass_ucb_waveform.h:150), which costs eight extra
 * waveforms per source.  Coordinates are the params array's
 * (f0 T, cos theta, phi, ln A, cos iota, psi, phi0, fdot T^2).
 *   term_y[i]      : as glass_gpu_dlogl_batch
 *   grad[8 i + k]  : d term_y / d params[k] = (r - h | dh/dp_k)
 *   fisher[64 i + 8 k + l] : (dh/dp_k | dh/dp_l)   (may be NULL)
 * The template size follows glass_gpu_set_template_size (32 to 4096; sizes
 * 2048 and 4096 are evaluated by clusters of 8 CTAs).  fisher_mode 0
 * weights every template bin with the noise at that bin; 1 reproduces
 * ucb_fisher's indexing, which weights template bin i with the noise of
 * segment bin i (ucb/src/glass_ucb_waveform.c:480-485).  Device pointers;
 * asynchronous.
 */
int glass_gpu_grad_fisher_batch(glass_gpu_ctx *ctx, int nitems, const int *item_seg, const double *params,
                                int fisher_mode, double *term_y, double *grad, double *fisher, int *status);

/* Same with HOST pointers: copies in, evaluates, copies out, synchronises. */
int glass_gpu_grad_fisher_batch_host(glass_gpu_ctx *ctx, int nitems, const int *item_seg, const double *params,
                                     int fisher_mode, double *term_y, double *grad, double *fisher, int *status);

/*
 * F-statistic of sky/frequency cells on the bank's segments; replaces
 * get_Fstat_logL (ucb/src/glass_ucb_fstatistic.c:646-703, declared at
 * ucb/src/glass_ucb_fstatistic.h:79), A/E channels.  Cell c is
 *   cells[4 c ..] = f0 (Hz), fdot (Hz/s), theta (colatitude, rad), phi (rad)
 * on segment cell_seg[c]; its four filters have the reference's size
 * ucb_bandwidth(f0, fdot, cos theta, A = 1e-22) and parameters (:241-344).
 *   logl[c]         = logL_AE = N^T M^-1 N / 2 (:599-622)
 *   fparams[4 c ..] = A, iota, psi, phase, the maximum-likelihood values
 *                     (:525-597, :697-700); may be NULL
 *   status[c]       = GLASS_ITEM_* bits (may be NULL): GLASS_ITEM_OUTSIDE when
 *                     no filter bin lies inside the segment (logL = 0, as the
 *                     reference gives when LAPACK meets the zero matrix),
 *                     GLASS_ITEM_NONFINITE for non-finite input, f0 <= 0,
 *                     filters above 4096 samples (segments over 8192 bins) or
 *                     a singular M.
 * As in the reference, N^i and M^ij run over the segment bins 0 < k < NFFT and
 * weight both channels with the A channel's noise.  logL_X (the X channel) is
 * not computed: the bank holds A and E.  FP64 throughout.  Device pointers;
 * asynchronous on the context's stream.
 */
int glass_gpu_fstat_batch(glass_gpu_ctx *ctx, int ncells, const int *cell_seg, const double *cells, double *logl,
                          double *fparams, int *status);

/* Same with HOST pointers: copies in, evaluates, copies out, synchronises. */
int glass_gpu_fstat_batch_host(glass_gpu_ctx *ctx, int ncells, const int *cell_seg, const double *cells, double *logl,
                               double *fparams, int *status);

/*
 * The F-statistic proposal density of segment seg; replaces
 * build_fstatistic_proposal (ucb/src/glass_ucb_proposal.c:1085-1182, declared
 * at ucb/src/glass_ucb_proposal.h:244) on the grid of
 * setup_fstatistic_proposal (:927-943): n_f cells of one bin in frequency
 * (n_f = (int)((fmax - fmin) T), NFFT or NFFT - 1), n_theta in cos(theta),
 * n_phi in phi (the reference uses 20 x 20).  Each cell is evaluated at its
 * centre with fdot = 0 and, where that gives logL > 1, along the chirp-mass
 * scan Mc = 0.1, 0.2, ... up to its first logL < 1; the density is the square
 * of the largest logL, normalised to mean 1.
 *   tensor: HOST, at least NFFT n_theta n_phi doubles; receives [i][j][k]
 *   info:   HOST, 4 doubles: n_f, norm, maxp (proposal->norm, ->maxp) and the
 *           number of cells that ran the scan
 * Synchronous.
 */
int glass_gpu_fstat_proposal_host(glass_gpu_ctx *ctx, int seg, int n_theta, int n_phi, double *tensor, double *info);

/*
 * Noise-model likelihood of XYZ frequency-domain data (the noise module's
 * sampler, noise/src/glass_noise_sampler.c:395-752).  glass_gpu_noise_setup
 * takes the data (X, Y, Z: 2 NFFT doubles each, re/im) on the bins
 * f = qmin/T + n/T, n < NFFT.  glass_gpu_noise_logl_batch then gives, for each
 * noise model p,
 *   logl[p] = my_noise_log_likelihood (noise/src/glass_noise_model.c:1243)
 * of the covariance generate_instrument_noise_model (:389, three channels)
 * builds from inst[12 p ..] = sacc[6], soms[6] (the reference's link order
 * 12, 21, 23, 32, 13, 31), plus, when sgal is not NULL, the galactic foreground
 * generate_galactic_foreground_model (:612) builds from sgal[5 p ..] =
 * ln A, ln f1, alpha, ln fk, ln f2, inverted as invert_noise_covariance_matrix
 * does (utils/src/glass_math.c:240).  FP64.  Device pointers; asynchronous.
 * The _host form takes host pointers and synchronises.
 */
int glass_gpu_noise_setup(glass_gpu_ctx *ctx, double T, int qmin, int NFFT, const double *X, const double *Y,
                          const double *Z);
int glass_gpu_noise_logl_batch(glass_gpu_ctx *ctx, int nprop, const double *inst, const double *sgal, double *logl);
int glass_gpu_noise_logl_batch_host(glass_gpu_ctx *ctx, int nprop, const double *inst, const double *sgal,
                                    double *logl);

/*
 * A stochastic gravitational-wave background (SGWB) added to the noise
 * covariance of both likelihoods above (the noise module's SGWBModel:
 * generate_sgwb_model, noise/src/glass_noise_model.c:778, in the Fourier
 * domain; generate_sgwb_model_wavelet, :843, at the layer centres over ND in
 * the wavelet domain).  glass_gpu_noise_sgwb_setup sets the spectral template
 * (SGWB_t, noise/src/glass_noise_model.h:99):
 *   0 power law         p = log10 A, alpha
 *   1 lognormal         p = log10 A, log10 fstar [Hz], log10 Delta
 *   2 phase transition  p = rb, b, log10 Ap, log10 fp [Hz]
 * (-1 removes it) and the instrument's response to an isotropic background as
 * the rows resp[7 i ..] = f, XX, YY, ZZ, XY, XZ, YZ, i < nresp (10 .. 3000;
 * the content of the reference's response file, read by
 * alloc_pop_sgwb_response, :134; f log-evenly spaced, f and the auto-responses
 * positive).  The response enters as the reference builds it: cubic splines
 * over log f of log XX, log YY, log ZZ and asinh(XY / 1e-7), ... evaluated at
 * every bin (or layer centre) of the grids set up, now and by later
 * glass_gpu_noise_setup / glass_gpu_noise_wavelet_setup calls.  Host
 * pointers; synchronous.
 *
 * The _sgwb batch forms take sgwb[4 p ..] (the template's first 2, 3 or 4
 * parameters; the rest ignored), or NULL for no background, and add
 * C_ij += R_ij(f) S(f) after the instrument and foreground, as
 * noise_instrument_model_mcmc (noise/src/glass_noise_sampler.c:559-568) and
 * the coarse wavelet covariances (:923, :983) combine them.  FP64.  Device
 * pointers, asynchronous; _host forms: host pointers, synchronous.  The
 * forms without _sgwb are these with sgwb = NULL.
 */
int glass_gpu_noise_sgwb_setup(glass_gpu_ctx *ctx, int type, int nresp, const double *resp);

/*
 * One- and two-channel data for the same batched likelihood:
 * nchannel 1 (d0 = Michelson X) or 2 (d0, d1 = A, E), 2 NFFT interleaved
 * doubles each, on the bins qmin/T + n/T (qmin >= 1); nchannel 3 is
 * glass_gpu_noise_setup(d0, d1, d2).  With one or two channels
 * glass_gpu_noise_logl_batch[_host] gives noise_log_likelihood
 * (noise/src/glass_noise_model.c:1104-1134) of the covariance of
 * generate_instrument_noise_model's case 1 / case 2 (:450-461: XYZnoise_FF or
 * AEnoise_FF of the link levels sacc[0], soms[0]; the other ten link levels
 * are not read) plus, with sgal, the foreground's case 1 / case 2 (:635-641),
 * diagonal inverse (utils/src/glass_math.c:248-258); no 2 pi constant.  The
 * SGWB covariance is three-channel only (GLASS_ERR_ARG otherwise, where
 * generate_sgwb_model stops).
 */
int glass_gpu_noise_setup_channels(glass_gpu_ctx *ctx, int nchannel, double T, int qmin, int NFFT, const double *d0,
                                   const double *d1, const double *d2);
int glass_gpu_noise_logl_batch_sgwb(glass_gpu_ctx *ctx, int nprop, const double *inst, const double *sgal,
                                    const double *sgwb, double *logl);
int glass_gpu_noise_logl_batch_sgwb_host(glass_gpu_ctx *ctx, int nprop, const double *inst, const double *sgal,
                                         const double *sgwb, double *logl);

/*
 * The same likelihood in the wavelet domain, coarse-grained
 * (my_noise_log_likelihood_wavelet_coarse, noise/src/glass_noise_model.c:1211;
 * Q = 1 is the full-resolution my_noise_log_likelihood_wavelet, :1182).
 * glass_gpu_noise_wavelet_setup takes the wavelet data on layers lmin ..
 * lmin + Nlayer - 1 of an NF x NT grid with layer width df (X, Y, Z: pixel i
 * of layer j at i + j NT, Nlayer NT doubles each), forms the cells' sample
 * covariances over Q pixels (coarse_grain_wavelet_data, :1057), and keeps the
 * foreground modulation mod[6 (NT/Q)] = XX, YY, ZZ, XY, XZ, YZ per cell (the
 * cache galaxy_modulation_cache_for_Q fills, utils/src/glass_galaxy.c:773; may
 * be NULL when mode 2 is not used).  glass_gpu_noise_wavelet_logl_batch gives
 * logl[p] for the covariance of
 *   mode 0: the instrument (generate_instrument_noise_model_wavelet, :561),
 *   mode 1: plus the stationary foreground
 *           (generate_full_stationary_covariance_matrix_coarse, :983),
 *   mode 2: plus the modulated foreground
 *           (generate_full_dynamic_covariance_matrix_coarse, :923),
 * with inst, sgal as glass_gpu_noise_logl_batch (sgal unused in mode 0).
 * FP64.  Device pointers; asynchronous.  _host: host pointers, synchronous.
 */
int glass_gpu_noise_wavelet_setup(glass_gpu_ctx *ctx, int NF, int NT, double df, int lmin, int Nlayer, int Q,
                                  const double *X, const double *Y, const double *Z, const double *mod);
int glass_gpu_noise_wavelet_logl_batch(glass_gpu_ctx *ctx, int mode, int nprop, const double *inst, const double *sgal,
                                       double *logl);
int glass_gpu_noise_wavelet_logl_batch_host(glass_gpu_ctx *ctx, int mode, int nprop, const double *inst,
                                            const double *sgal, double *logl);
int glass_gpu_noise_wavelet_logl_batch_sgwb(glass_gpu_ctx *ctx, int mode, int nprop, const double *inst,
                                            const double *sgal, const double *sgwb, double *logl);
int glass_gpu_noise_wavelet_logl_batch_sgwb_host(glass_gpu_ctx *ctx, int mode, int nprop, const double *inst,
                                                 const double *sgal, const double *sgwb, double *logl);

/*
 * The noise module's one- and two-channel spline noise model
 * (noise_spline_model_mcmc / _rjmcmc, noise/src/glass_noise_sampler.c:213-393):
 * each model's noise spectrum per channel is the natural cubic spline through
 * its control points (CubicSplineGLASS with the binary-search lookup,
 * utils/src/glass_math.c:855-868) at f_n = qmin/T + n/T plus the transfer
 * function (generate_spline_noise_model, noise/src/glass_noise_model.c:366-387),
 * and logl[p] is noise_log_likelihood (:1104-1134) of the data for it:
 *   -sum_c sum_n |d_c[n]|^2 / C_c[n]  -  sum_n sum_c log C_c[n].
 * glass_gpu_spline_noise_setup keeps the grid, transfer[NFFT] and the data's
 * power |d_c|^2 (d0, d1: 2 NFFT interleaved doubles; d1 used when nchannel
 * is 2).  glass_gpu_spline_noise_logl_batch: model p has nknots[p] control
 * points (2 .. kmax, frequencies strictly increasing) at knot_f[p kmax + k],
 * values knot_C[(p nchannel + c) kmax + k]; kmax <= 512.  One launch, one CTA
 * per model.  FP64.  Device pointers, asynchronous (a knot count outside
 * 2 .. kmax gives NaN).  _host: host pointers, synchronous, and the knot
 * counts and orders are checked (GLASS_ERR_ARG).
 */
int glass_gpu_spline_noise_setup(glass_gpu_ctx *ctx, int nchannel, double T, int qmin, int NFFT,
                                 const double *transfer, const double *d0, const double *d1);
int glass_gpu_spline_noise_logl_batch(glass_gpu_ctx *ctx, int nprop, int kmax, const int *nknots,
                                      const double *knot_f, const double *knot_C, double *logl);
int glass_gpu_spline_noise_logl_batch_host(glass_gpu_ctx *ctx, int nprop, int kmax, const int *nknots,
                                           const double *knot_f, const double *knot_C, double *logl);

/* glass_gpu_dlogl_batch with each channel's share of term_y as well:
 * term_ch[2 i] (A) + term_ch[2 i + 1] (E) = term_y[i].  Device pointers. */
int glass_gpu_dlogl_batch_channels(glass_gpu_ctx *ctx, int precision, int nitems, const int *item_seg,
                                   const double *params, const double *term_x, double *dlogl, double *term_y,
                                   double *hh, int *status, double *term_ch);

/*
 * The UCB sampler's noise step (noise_model_mcmc, ucb/src/glass_ucb_sampler.c:29-73,
 * Fourier basis, A/E): for chain i whose model on segment item_seg[i] is the
 * bank's residual minus the template of params[8 i ..], the change of
 * logL + logLnorm when each channel's noise level moves from eta_x[2 i + c] to
 * eta_y[2 i + c] (c = 0 A, 1 E) with the residual unchanged
 * (generate_noise_model, ucb/src/glass_ucb_model.c:336; gaussian_log_likelihood
 * and gaussian_log_likelihood_model_norm, utils/src/glass_model.c:726, :788):
 *   dlogl_noise[i] = (logL + logLnorm)(eta_y) - (logL + logLnorm)(eta_x).
 * The sampler divides by the temperature and adds the prior as before.  The
 * template's per-channel power comes from the batched path in `precision`.
 * Device pointers, asynchronous; the _host form synchronises.
 */
int glass_gpu_noise_eta_batch(glass_gpu_ctx *ctx, int precision, int n, const int *item_seg, const double *params,
                              const double *eta_x, const double *eta_y, double *dlogl_noise, int *status);
int glass_gpu_noise_eta_batch_host(glass_gpu_ctx *ctx, int precision, int n, const int *item_seg,
                                   const double *params, const double *eta_x, const double *eta_y,
                                   double *dlogl_noise, int *status);

/* ------------------------------------------------ on-device sampler */
/*
 * The reference draws a chain's random numbers from the C library's rand_r on
 * that chain's seed (rand_r_U_0_1 = rand_r / RAND_MAX, utils/src/glass_utils.c:19;
 * chain->r[ic]).  These kernels advance the same seeds with the same
 * algorithm, so the decisions are the reference's; the seeds, like every other
 * argument, are DEVICE arrays updated in place.  Asynchronous.
 *
 * glass_gpu_rand_r_fill: out[i count + k] = the next count rand_r values of
 * seed[i] (a check of the stream).
 *
 * glass_gpu_mh_accept: the accept/reject tail of ucb_mcmc
 * (ucb/src/glass_ucb_sampler.c:141-172) for n chains: where logPy[i] is
 * finite, snr[i] < 5 (snr may be NULL) rejects as the reference does, logH =
 * dlogl[i]/temperature[i] + logPy - logPx + logQxy - logQyx, one draw
 * loga = log U(0,1), and acceptance when logH is finite and > loga; no draw
 * where logPy is -inf.  On acceptance params_x[8 i ..] = params_y[8 i ..] and
 * logL_x[i] += dlogl[i].  accepted[i] = 1/0 (may be NULL).
 *
 * glass_gpu_ptmcmc: ptmcmc (utils/src/glass_sampler.c:19-63) on nens ladders
 * of NC chains: ladder e's chain c at e NC + c of logL, logLnorm (may be
 * NULL), index (the ladder's permutation of 0..NC-1), seed and acceptance;
 * temperature[NC] shared.
 *
 * glass_gpu_fisher_draw: draw_from_fisher (ucb/src/glass_ucb_proposal.c:348-391)
 * for n chains: from params_x[8 i ..], the eigenvectors evec[64 i + 8 j + k]
 * (= source->fisher_evectr[j][k]) and eigenvalues evalue[8 i ..], eight
 * rand_r_N_0_1 amplitudes (utils/src/glass_utils.c:24-35) over sqrt(eigenvalue)
 * and one rand_r_U_0_1 choice of the eigenvector, the jump along it, a NaN jump
 * component replaced by 0.01 params_x, params_y = params_x + jump with the two
 * cosines reflected back where they reach +-1.  logQ[i] (may be NULL) is 0, or
 * -inf where a drawn parameter is NaN (the reference's return value);
 * status[i] (may be NULL) a GLASS_DRAW_* code.  The seeds advance exactly as
 * the reference's; the parameters agree with the C library's to within the
 * last bits of its log.  Where the choice draw is RAND_MAX the reference reads
 * one column past the matrix; the last column is used here.
 */
#define GLASS_DRAW_OK 0
#define GLASS_DRAW_NAN 1        /* a drawn parameter is NaN: logQ = -inf */
#define GLASS_DRAW_RNG_LIMIT 2  /* 4096 rejections in a row in the polar method (probability ~1e-2700) */
int glass_gpu_rand_r_fill(glass_gpu_ctx *ctx, int n, int count, unsigned int *seed, int *out);
int glass_gpu_mh_accept(glass_gpu_ctx *ctx, int n, const double *temperature, const double *dlogl, const double *logPx,
                        const double *logPy, const double *logQxy, const double *logQyx, const double *snr,
                        unsigned int *seed, double *logL_x, double *params_x, const double *params_y, int *accepted);
int glass_gpu_ptmcmc(glass_gpu_ctx *ctx, int nens, int NC, const double *temperature, const double *logL,
                     const double *logLnorm, int *index, unsigned int *seed, double *acceptance);
int glass_gpu_fisher_draw(glass_gpu_ctx *ctx, int n, const double *params_x, const double *evec, const double *evalue,
                          unsigned int *seed, double *params_y, double *logQ, int *status);

/*
 * glass_gpu_sym_eigen8: the eigen-decomposition matrix_eigenstuff
 * (utils/src/glass_math.c:475-499) gives a chain's Fisher matrix, for n
 * symmetric 8x8 matrices (matrix[64 i + 8 r + c]), so that
 * glass_gpu_grad_fisher_batch -> glass_gpu_sym_eigen8 -> glass_gpu_fisher_draw
 * runs without the host: evec[64 i + 8 j + k] = component j of eigenvector k,
 * evalue[8 i + k]; cyclic Jacobi rotations in FP64 (every eigenvalue to full
 * relative accuracy), pairs sorted by decreasing eigenvalue, each vector's
 * largest component positive (the drop-in matrix_eigenstuff's convention;
 * LAPACK's order and signs are not reproduced).
 *
 * glass_gpu_prior_draw: draw_from_uniform_prior (utils/src/glass_sampler.c:96-107)
 * for n chains: params[8 i + k] = prior[2 k] + rand_r_U_0_1 (prior[2 k + 1] -
 * prior[2 k]) in order k = 0..7, logQ[i] = -sum logPV[k]; prior[16 c ..] the
 * model's bounds and logPV[8 c ..] its log prior volumes, c = i prior_stride
 * (0: one model for all chains, 1: one per chain).  Seeds advance as the
 * reference's.
 *
 * glass_gpu_ucb_prior: evaluate_ucb_prior (ucb/src/glass_ucb_prior.c:536-556)
 * without the catalogue (GMM) prior: check_range (:400-438: NaN or a bound
 * violated gives -inf; longitude, polarisation and phase are wrapped into
 * range IN PLACE in params, as the reference does), the sky-location prior
 * (:590-639: skyhist[i nphi + j] over cells dcostheta x dphi from the lower
 * bounds when skyhist is given, else uniform) and evaluate_uniform_priors
 * (:560-588).  The wrapping loops stop after 64 turns (the reference's do not).
 * All pointers DEVICE pointers; asynchronous.
 */
int glass_gpu_sym_eigen8(glass_gpu_ctx *ctx, int n, const double *matrix, double *evec, double *evalue);
int glass_gpu_prior_draw(glass_gpu_ctx *ctx, int n, const double *prior, int prior_stride, const double *logPV,
                         unsigned int *seed, double *params, double *logQ);
int glass_gpu_ucb_prior(glass_gpu_ctx *ctx, int n, double *params, const double *prior, int prior_stride,
                        const double *logPV, const double *skyhist, double dcostheta, double dphi, int nphi,
                        double *logP);

/*
 * The trans-dimensional (birth/death) step of ucb_rjmcmc
 * (ucb/src/glass_ucb_sampler.c:454-566, rj_birth_death :175-249) for n
 * chains on device state, in two launches around the likelihood:
 *
 * glass_gpu_rj_propose: per chain, every draw in the reference's order: the
 * proposal by rejection on the rj weights (rjweight[9], host array: only
 * 0 = prior draw, draw_from_uniform_prior, and 1 = F-statistic draw,
 * draw_from_fstatistic with the grid of build_fstatistic_proposal, may be
 * non-zero: the reference's cocktail without the catalogue and covariance
 * proposals), the birth/death choice, then for a birth (move = +1) the new
 * source params_y[8 i ..] and logQyx (refused, logPy = -inf, when Nlive + 1 >=
 * Neff), for a death (move = -1) the source slot[i] to remove, copied to
 * params_y, and logQxy (its proposal density; refused when Nlive = 0).
 * kind[i] = the proposal, status[i] (may be NULL) a GLASS_RJ_* code.  Chain
 * i's live sources: src[(i maxsrc + s) 8 ..], s < Nlive[i] (maxsrc: the
 * reference's Nmax).
 *
 * The caller then evaluates the likelihood change of each proposal, e.g.
 * with glass_gpu_dlogl_batch on params_y against the chain's residual
 * (term_x = 0), which gives a birth's change directly and a death's as
 * -(term + hh) (dlogl_is_term = 1), and hh = (h|h) for the birth's SNR cut.
 *
 * glass_gpu_rj_accept: the birth's SNR cut (sqrt(hh) < 5, skipped with
 * prior_only or hh NULL), the priors of the current and proposed source
 * lists (evaluate_ucb_prior as glass_gpu_ucb_prior: sources wrapped in place),
 * logH = dlogl / temperature + logPy - logPx + logQxy - logQyx, one draw
 * loga = log U(0,1) (always), and on acceptance the source list (the new
 * source appended, or the removed one taken out with the rest moved down),
 * Nlive and logL_x += dlogl.  accepted[i] (may be NULL).  Not restated: the
 * split/merge and cluster-bomb moves (never chosen by the reference's
 * branch draws), the maximisation penalty and calibration, the Fisher
 * matrices the reference refreshes on acceptance.  All arrays DEVICE
 * arrays; asynchronous.
 */
typedef struct {
  const double *tensor; /* device: density of cell (i, j, k) at (i n_theta + j) n_phi + k */
  int n_f, n_theta, n_phi;
  double d_f, d_theta, d_phi; /* cell sizes: Hz, cos theta, phi */
  double maxp;                /* the largest density */
  int qmin;                   /* the segment's first bin */
  double T;
} glass_gpu_fstat_grid;
#define GLASS_RJ_OK 0
#define GLASS_RJ_RNG_EDGE 1  /* a draw of exactly 1 picked one past the end (the reference reads past its arrays) */
#define GLASS_RJ_RNG_LIMIT 2 /* 2^20 rejections in a row: the proposal is refused */
int glass_gpu_rj_propose(glass_gpu_ctx *ctx, int n, int maxsrc, const int *Nlive, const int *Neff, const double *src,
                         const double *prior, int prior_stride, const double *logPV, const double *rjweight,
                         const glass_gpu_fstat_grid *grid, unsigned int *seed, int *move, int *slot, int *kind,
                         double *params_y, double *logQxy, double *logQyx, double *logPy, int *status);
int glass_gpu_rj_accept(glass_gpu_ctx *ctx, int n, int maxsrc, int *Nlive, double *src, const int *move,
                        const int *slot, double *params_y, const double *logQxy, const double *logQyx,
                        const double *logPy, const double *temperature, const double *dlogl, const double *hh,
                        int dlogl_is_term, int prior_only, const double *prior, int prior_stride, const double *logPV,
                        const double *skyhist, double dcostheta, double dphi, int nphi, unsigned int *seed,
                        double *logL_x, int *accepted);

/* Number of kernels the last glass_gpu_dlogl_batch launched (for accounting). */
int glass_gpu_last_launch_count(glass_gpu_ctx *ctx);

/* Per-phase timing of glass_gpu_dlogl_batch (profiling aid; off by default).
 * With enable != 0 every later call records five timing events on the
 * context's stream: before the plan kernel, after it, after the slow-part
 * kernel, after the spectral (FFT + likelihood) kernels and after the
 * re-evaluations that follow them (see glass_gpu_set_mixed_tolerance; empty
 * in FP64 or with the tolerance off).  glass_gpu_last_phase_ms waits for the
 * last call's events and writes the four durations in milliseconds to
 * ms[0..3] (plan, slow part, spectral, re-evaluation); GLASS_ERR_STATE when no
 * call was made with timing on.  Events recorded while the stream is being
 * captured into a CUDA graph become graph nodes: read the durations after
 * launches made outside capture. */
int glass_gpu_set_phase_timing(glass_gpu_ctx *ctx, int enable);
int glass_gpu_last_phase_ms(glass_gpu_ctx *ctx, float *ms);

/*
 * Accuracy of GLASS_PREC_MIXED.  No counterpart in the reference, which is
 * FP64 throughout.  The FP32 template's rounding error enters delta logL
 * through the template's inner product with the residual r - h: a part
 * spread over the template's N bins, up to ~6e-7 sqrt(H R / N), and a part
 * along the template (the FP32 per-proposal constants), up to ~1.5e-7
 * |(h|r - h)|/2, H = (h|h)/2 and R = |r - h|^2 the whitened powers over the
 * template support (H of the whole template when the segment edge clips it).
 * That is below 1e-3 except for loud templates (near the data of an SNR ~ 300
 * source, or far from the data with a power of 1e6, as a jump of a weak
 * source's amplitude by e^6 gives).  The spectral kernel estimates each
 * proposal's error from sums it already has (with the constants 9e-7 and
 * 2e-7) and lists those above `tol`; the listed proposals are evaluated again
 * in double-float arithmetic (slow part, FFTs and sums; error ~1e-12) and the
 * results written over the mixed ones, in the same launch sequence (and CUDA
 * graph: a conditional node skips the re-evaluation when nothing is listed).
 * tol <= 0 turns the re-evaluation off (pure mixed precision); the default is
 * 1e-3.  Changing it drops the context's recorded host-path graphs.
 */
int glass_gpu_set_mixed_tolerance(glass_gpu_ctx *ctx, double tol);
/* Per-proposal tolerance: proposal i < n of every later batch uses
 * tol * scale[i] (HOST array, copied; scales finite and positive; n = 0
 * restores tol for all).  A parallel-tempering sampler passes its ladder
 * (scale[i] = the temperature of batch slot i): the error of the Hastings
 * ratio's likelihood part, delta logL / T, is then at most tol for every
 * proposal, and only the cold chains' proposals need delta logL itself to
 * tol.  Synchronises the context's stream. */
int glass_gpu_set_mixed_tolerance_scale(glass_gpu_ctx *ctx, int n, const double *scale);
/*
 * Launch shapes of the mixed-precision path, by name; the autotuner
 * (glass_gb300/tune.py) sweeps them on the target workload and records the
 * fastest per GPU model.  0 selects the built-in choice.
 *   "slow_block"        slow-part kernel threads per CTA: 128, 256 (default), 512
 *   "slow_ctas_per_sm"  cap on its resident CTAs per SM (0: occupancy limit)
 *   "spec_ctas_per_sm"  cap on the persistent spectral kernel's CTAs per SM
 *   "plan_per_cta"      proposals per plan CTA, 8..32 (0: ceil(n / SMs) in 16..32)
 * Changing a value drops the context's recorded host-path graphs; graphs the
 * caller captured keep the shapes they were captured with.
 */
int glass_gpu_set_tuning(glass_gpu_ctx *ctx, const char *key, int value);
int glass_gpu_get_tuning(glass_gpu_ctx *ctx, const char *key, int *value);

/* Number of proposals re-evaluated in double-float since the context's work
 * buffers were allocated.  Synchronises the context's stream. */
int glass_gpu_mixed_reevaluated(glass_gpu_ctx *ctx, unsigned long long *count);

/* ------------------------------------------- batch that allocates nothing */
/*
 * No counterpart in the reference.  For callers that cannot allocate GPU
 * memory once they are running -- a host that allocates everything at start-up
 * and forbids it later, code running inside someone else's memory pool, or code
 * that may not call the CUDA allocator at all -- this evaluates a batch with
 * the kernels glass_gpu_dlogl_batch runs for GLASS_PREC_FP64, on the caller's
 * stream, without calling cudaMalloc or any other allocating routine and
 * without a context.  The segment tables are built on the device here (on the
 * host there), so the two agree to about 1e-13 relative, not bit for bit.
 * All pointers are device pointers the caller owns; the segment inputs have
 * the layout of glass_gpu_bank_upload.
 *
 * Intermediate data live in fixed arrays compiled into the library (about
 * 41 MB of device memory, held by every GPU that loads the library until the
 * process exits), which bounds the sizes:
 *   nitems <= GLASS_NOALLOC_MAX_ITEMS, nseg * NFFT <= GLASS_NOALLOC_MAX_BINS,
 *   nitems * min(NFFT, 4096) <= GLASS_NOALLOC_MAX_SAMPLES;
 * larger inputs return GLASS_ERR_SIZE.  Every call on a device shares those
 * arrays, so calls that overlap on the GPU (other streams, other host threads)
 * race: serialise them.  The first call on a device looks up the arrays'
 * addresses; make it before any stream capture.  Asynchronous on `stream`.
 */
#define GLASS_NOALLOC_MAX_ITEMS 4096
#define GLASS_NOALLOC_MAX_BINS 65536
#define GLASS_NOALLOC_MAX_SAMPLES 524288
int glass_gpu_dlogl_fp64_noalloc(void *stream, int format, double T, double t0, int NFFT, int nseg, const int *qmin,
                                 const double *rA, const double *rE, const double *invCA, const double *invCE,
                                 int nitems, const int *item_seg, const double *params, const double *term_x,
                                 double *dlogl, double *term_y, double *hh, int *status);

/* ------------------------------------------------------ WDM transforms */
/*
 * Wilson-Daubechies-Meyer time-frequency transform on a grid of NF layers x
 * NT pixels, ND = NF NT samples, coefficient layout wdm[n + NT m] with the DC
 * (m = 0) and Nyquist (m = NF) layers in the even and odd pixels of row 0.
 * The window is the Meyer window with flat half-width A and exponent nx; the
 * reference fixes A = 0 and nx = 6 (WAVELET_FILTER_CONSTANT,
 * utils/src/glass_wavelet.h:21) and allocates NF = 1536 layers
 * (utils/src/glass_wavelet.c:210-271).
 *
 * glass_wdm_window replaces build_wdm_filter_freq
 * (utils/src/glass_wavelet.c:327, declared utils/src/glass_wavelet.h:122):
 * phif[0..NT/2], forward normalisation when forward != 0.  Host only.
 */
int glass_wdm_window(int NF, int NT, double A, double nx, int forward, double *phif);

/*
 * time (ND samples) -> wdm (ND coefficients).  Replaces
 * wavelet_transform_timefreq (utils/src/glass_wavelet.c:293, declared
 * utils/src/glass_wavelet.h:100), which is the real FFT
 * (utils/src/glass_math.c:808) followed by wavelet_transform_freq
 * (utils/src/glass_wavelet.c:410).  The reference transforms in place; here
 * time and wdm may be the same buffer or different ones.
 * precision GLASS_PREC_FP64 computes in FP64 (matches the reference to about
 * 1e-13 of the largest coefficient); GLASS_PREC_MIXED computes in FP32 (about
 * 1e-6).  Grid limits: NT even, 8 <= NT <= 4096, NT and ND/2 of the form
 * 2^a 3^b with ND/2 = M1 M2, M1, M2 <= 4096 (GLASS_ERR_SIZE otherwise).
 * Device pointers; asynchronous on the context's stream.  The first call on a
 * grid builds tables (synchronous, allocates); later calls on the same grid
 * reuse them.
 */
int glass_gpu_wdm_forward(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx,
                          const double *time, double *wdm);

/*
 * wdm -> time.  Replaces wavelet_transform_inverse_freq
 * (utils/src/glass_wavelet.c:351, declared utils/src/glass_wavelet.h:108)
 * followed by glass_inverse_real_fft_outplace (utils/src/glass_math.c:819).
 * Same arguments, precision and limits as glass_gpu_wdm_forward.
 */
int glass_gpu_wdm_inverse(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx,
                          const double *wdm, double *time);

/*
 * wdm -> the ND/2 + 1 complex bins (ND + 2 doubles, re/im interleaved) that
 * wavelet_transform_inverse_freq (utils/src/glass_wavelet.c:351) produces, and
 * bins -> wdm as wavelet_transform_freq (utils/src/glass_wavelet.c:410) does.
 * Same precision and grid limits as glass_gpu_wdm_forward; input and output
 * must not overlap.  Device pointers; asynchronous.
 */
int glass_gpu_wdm_to_freq(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx, const double *wdm,
                          double *freq);
int glass_gpu_wdm_from_freq(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx,
                            const double *freq, double *wdm);

/* The same two with HOST pointers: copy in, transform, copy out, synchronise. */
int glass_gpu_wdm_forward_host(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx,
                               const double *time, double *wdm);
int glass_gpu_wdm_inverse_host(glass_gpu_ctx *ctx, int precision, int NF, int NT, double A, double nx,
                               const double *wdm, double *time);

/*
 * wavelet_transform_timefreq_by_layers (utils/src/glass_wavelet.c:544-610,
 * glass_wavelet.h:119) on a HOST series of NT (nlayers + 1) samples, in place:
 * the real FFT of the series, then for each of the nlayers layers from jmin
 * the band around its centre weighted by window[0 .. NT/2] and an NT-point
 * inverse FFT, written to timedata[n nlayers + layer] (the rest zero).  FP64,
 * one CTA; NT a power of two and NT (nlayers + 1) / 2 of the form 2^a 3^b.
 */
int glass_gpu_wdm_by_layers_host(glass_gpu_ctx *ctx, int NF, int NT, int jmin, int nlayers, const double *window,
                                 double *timedata);

/* ------------------------------------------- wavelet-domain UCB waveform */
/*
 * The wavelet-domain UCB waveform (ucb_waveform_wavelet,
 * ucb/src/glass_ucb_waveform.c:1061, declared
 * ucb/src/glass_ucb_waveform.h:231) and the sparse-pixel likelihood
 * delta_log_likelihood (utils/src/glass_model.c:624, declared
 * utils/src/glass_model.h) for batches of sources, in FP64.
 *
 * glass_gpu_wavelet_setup fixes the segment: observation Tobs from t0, a WDM
 * grid of NF layers x NT pixels of duration wdt and bandwidth wdf (the
 * reference's struct Wavelets fields dt, df), Meyer window (A, nx; the
 * reference uses A = 0, nx = 6), and the data pixels [kmin, kmax) (whole
 * layers, as the reference's kmin/kmax are).  The orbit is given as norb node
 * times orbit_t and positions orbit_pos[(3 s + d) norb + n] in metres (the
 * arrays struct Orbit holds, utils/src/glass_lisa.h:60-109), or, with both
 * NULL, is initialize_interpolated_analytic_orbits (utils/src/glass_lisa.c:271).
 * Limits: NT even, of the form 2^a 3^b, 8 <= NT <= 4096; 20 <= norb <= 2048.
 * Host pointers; synchronous; allocates the grid tables and a work area.
 */
int glass_gpu_wavelet_setup(glass_gpu_ctx *ctx, double Tobs, double t0, int NF, int NT, double wdt, double wdf,
                            double A, double nx, int kmin, int kmax, int norb, const double *orbit_t,
                            const double *orbit_pos);

/* The segment's residual X, Y, Z (N = kmax - kmin pixels each, pixel k - kmin)
 * and inverse noise covariance invC[(3 i + j) N + k] (the reference's
 * noise->invC[i][j][k]).  Host pointers; synchronous. */
int glass_gpu_wavelet_set_data(glass_gpu_ctx *ctx, const double *rX, const double *rY, const double *rZ,
                               const double *invC);

/*
 * precision GLASS_PREC_FP64: everything in FP64 with the reference's order
 * of operations (delta logL to 1e-10 of the reference).  GLASS_PREC_MIXED: the
 * sample phase (carrier at S/C 1 minus the heterodyne, plus the channel's
 * relative phase) to FP64 accuracy (FP64 per-interval constants, double-float
 * per sample) and reduced mod 2 pi, the amplitude spline, FFTs and
 * layer transforms in FP32, the likelihood from FP32 products with
 * double-float sums, per pixel in the form (residual or direct) with the
 * smaller rounding error.  Its error against FP64 is set by the FP32 template
 * (relative ~4e-7 rms): measured below 1e-7 sqrt((h|h) (r - h|r - h)), below
 * 1e-3 where the residual holds noise and the source's own signal, and growing
 * where a loud template meets data that do not contain it.  With the
 * context's mixed tolerance (glass_gpu_set_mixed_tolerance, default 1e-3;
 * the per-proposal scale is not applied here) every source whose estimate
 * 2e-7 sqrt((h|h) (r - h|r - h)) exceeds it, or whose mixed result is not
 * finite, is evaluated again in FP64 in the same launch sequence (two more
 * launches), so that |delta logL error| stays below the tolerance; tol <= 0
 * gives the mixed values alone.  glass_gpu_wavelet_reevaluated counts those
 * sources over the context's life (synchronises the stream).
 *
 * For each of nitems parameter vectors params[8 i ..] (the reference's UCB
 * params array), the wavelet waveform on its pixel list and
 *   term_y[i] = (h|h) - 2 (r|h)     (nine XYZ cross terms, as delta_log_likelihood)
 *   hh[i]     = (h|h)               (snr_wavelet squared, utils/src/glass_math.c:428)
 *   dlogl[i]  = -(term_y[i] - term_x[i]) / 2
 * so that dlogl is delta_log_likelihood of replacing a source whose term is
 * term_x[i] (NULL: 0) by this one against the residual r.  status[i]: 0, or
 * GLASS_ITEM_NONFINITE for invalid parameters (outputs NaN), or
 * GLASS_ITEM_OUTSIDE when no pixel of the source falls in the segment.
 * Device pointers (any may be NULL except params); asynchronous.
 */
int glass_gpu_wavelet_dlogl_batch(glass_gpu_ctx *ctx, int precision, int nitems, const double *params,
                                  const double *term_x, double *dlogl, double *term_y, double *hh, int *status);
int glass_gpu_wavelet_dlogl_batch_host(glass_gpu_ctx *ctx, int precision, int nitems, const double *params,
                                       const double *term_x, double *dlogl, double *term_y, double *hh, int *status);
int glass_gpu_wavelet_reevaluated(glass_gpu_ctx *ctx, unsigned long long *count);

/*
 * The waveforms themselves: info[4 i ..] = first layer, layer count, first
 * layer inside the segment (jlo), layers inside the segment (c; -1 for invalid
 * parameters); xyz[(3 i + ch) 3 NT + q] = channel ch (X, Y, Z) at list entry q
 * < NT c, whose pixel is k - kmin = q / c + (jlo + q % c) NT - kmin.  This is
 * ucb_waveform_wavelet's wavelet_list / X[list[q]] output in compact form
 * (including its rule that the q-th listed pixel takes the q-th coefficient
 * of the per-layer transform).  Device pointers; asynchronous.
 */
int glass_gpu_wavelet_waveform_batch(glass_gpu_ctx *ctx, int precision, int nitems, const double *params, int *info,
                                     double *xyz, int *status);
int glass_gpu_wavelet_waveform_batch_host(glass_gpu_ctx *ctx, int precision, int nitems, const double *params,
                                          int *info, double *xyz, int *status);

/*
 * Wavelet-domain Fisher matrices, batched: ucb_fisher_wavelet
 * (ucb/src/glass_ucb_waveform.c:524-640) for nitems sources params[8 i ..]
 * against the noise of glass_gpu_wavelet_set_data.  Central differences with
 * the reference's step (each parameter +-5e-7, the cosine parameters clamped
 * to [-1, 1], divided by 1e-6) of FP64 wavelet waveforms, on the pixels of
 * each + waveform's list whose time index t has imin < t < imax (the
 * reference's wdm->imin, wdm->imax), and the nine XYZ cross terms of invC per
 * pixel (wavelet_nwip).  fisher[64 i + 8 k + l] = (dh/dp_k | dh/dp_l); a NaN
 * element becomes 10, as in the reference; status[i] (may be NULL) is 0, or
 * the status of an invalid perturbed parameter set (fisher then NaN).  The
 * eigen-decomposition the reference does next (matrix_eigenstuff) stays with
 * the caller.  Device pointers; asynchronous on the context's stream.  The
 * reference's own ucb_fisher_wavelet also runs unchanged on the drop-in
 * ucb_waveform_wavelet below, one source at a time.
 */
int glass_gpu_wavelet_fisher_batch(glass_gpu_ctx *ctx, int nitems, const double *params, int imin, int imax,
                                   double *fisher, int *status);
int glass_gpu_wavelet_fisher_batch_host(glass_gpu_ctx *ctx, int nitems, const double *params, int imin, int imax,
                                        double *fisher, int *status);

/* ------------------------------------ drop-ins for the wavelet headers */
/*
 * Same names and signatures as the reference, so that ucb_wavelet_mcmc and
 * global_fit link against this library instead of glass_wavelet.o /
 * glass_ucb_waveform.o.  Host arrays; one GPU context per calling thread
 * (device from GLASS_GPU_DEVICE, default 0), created on first use.  FP64,
 * window exponent 6 (WAVELET_FILTER_CONSTANT).  Errors print the reason and
 * exit(1), the reference's way of failing.
 *
 * build_wdm_filter_freq          utils/src/glass_wavelet.c:327 (glass_wavelet.h:122)
 * wavelet_transform_timefreq     utils/src/glass_wavelet.c:293 (glass_wavelet.h:100), in place
 * wavelet_transform_freq         utils/src/glass_wavelet.c:410 (glass_wavelet.h:105)
 * wavelet_transform_inverse_freq utils/src/glass_wavelet.c:351 (glass_wavelet.h:108)
 * wavelet_transform_timefreq_by_layers utils/src/glass_wavelet.c:544 (glass_wavelet.h:119), in place
 * ucb_waveform_wavelet           ucb/src/glass_ucb_waveform.c:1061 (glass_ucb_waveform.h:231);
 *                                the orbit nodes come from the caller's struct Orbit
 *                                (Norb, t, x, y, z), so interpolated analytic and
 *                                numeric orbits both work.
 * ucb_waveform_wavelet_tab / _slow (glass_ucb_waveform.h:237, :239) are not
 * built: the reference's lookup-table variant itself exits as "not
 * implemented", and _slow is a debugging variant that writes files.  They
 * report that and exit(1); glass_ucb_waveform_wavelet_tab/_slow return the
 * same as GLASS_ERR_STATE for callers that want a status.
 */
void build_wdm_filter_freq(double *phif, int Nf, int Nt, double A, bool forward);
void wavelet_transform_timefreq(struct Wavelets *wdm, double *timedata);
void wavelet_transform_freq(struct Wavelets *wdm, double *freqdata, double *wdmdata);
void wavelet_transform_inverse_freq(struct Wavelets *wdm, double *wdmdata, double *freqdata);
void wavelet_transform_timefreq_by_layers(struct Wavelets *wdm, int jmin, int Nlayers, double *window,
                                          double *timedata);
void ucb_waveform_wavelet(struct Orbit *orbit, struct Wavelets *wdm, double Tobs, double t0, double *params,
                          int *wavelet_list, int *Nwavelet, double *X, double *Y, double *Z);
void ucb_waveform_wavelet_tab(struct Orbit *orbit, struct Wavelets *wdm, double Tobs, double t0, double *params,
                              int *wavelet_list, int *Nwavelet, double *X, double *Y, double *Z);
void ucb_waveform_wavelet_slow(struct Orbit *orbit, struct Wavelets *wdm, double Tobs, double t0, double *params,
                               int *wavelet_list, int *Nwavelet, double *X, double *Y, double *Z);
int glass_ucb_waveform_wavelet_tab(void);
int glass_ucb_waveform_wavelet_slow(void);


#ifdef __cplusplus
}
#endif
#endif /* GLASS_GB300_H */
