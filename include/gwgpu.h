/*
 * gwgpu.h -- C ABI of the GB300 likelihood engine for gw_analysis_tools.
 *
 * Plain C types only (pointers, sizes, ints, doubles).  Host buffers unless a
 * name ends in _device.  Complex arrays are interleaved (re, im) doubles, the
 * memory layout of std::complex<double>.  Every entry point returns a
 * GWGPU_* status code unless documented otherwise; waveform entry points that
 * mirror the reference return 1 on success like the reference does.
 *
 * Each declaration names the reference interface it replaces
 * (file:line in gw_analysis_tools).
 */
#ifndef GWGPU_H
#define GWGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define GWGPU_OK 0
#define GWGPU_EINVAL 1      /* bad argument (null pointer, length < 2, unknown detector/method) */
#define GWGPU_ECUDA 2       /* CUDA runtime error; see gwgpu_last_error_string */
#define GWGPU_ENOMEM 3      /* HBM budget of the context exceeded */
#define GWGPU_EDOMAIN 4     /* request outside the model domain (NaN, eta > 1/4, spin out of table) */
#define GWGPU_ETIMEDOUT 5   /* a bounded wait gave up */
#define GWGPU_EBUSY 6       /* queue full / resource in use */
#define GWGPU_ENOTFOUND 7   /* unknown handle or ticket */
#define GWGPU_ETOOLARGE 8   /* size beyond a fixed maximum */
#define GWGPU_ESINGULAR 9   /* Fisher matrix not positive definite in FP64: matrix returned, covariance NaN */

/* ---- approximants and precision forms ---- */
#define GWGPU_IMRPHENOMD 0
#define GWGPU_IMRPHENOMPV2 1
#define GWGPU_PREC_FP64 0   /* the reference arithmetic in FP64 on the device */
#define GWGPU_PREC_MIXED 1  /* FP32 amplitude/projection/products, FP64 phase, compensated sums */

/* ---- Fisher parameterisations (unpack_parameters, fisher.cpp:1841-1961) ---- */
#define GWGPU_FISHER_IMRPHENOMD 0        /* "IMRPhenomD": 11 params, D_L and M_c as log factors */
#define GWGPU_FISHER_MCMC_IMRPHENOMD 1   /* "MCMC_IMRPhenomD": 11 MCMC params */
#define GWGPU_FISHER_STEP_ABSOLUTE 0     /* epsilon added to each parameter (the reference: 1e-8, fisher.cpp:158) */
#define GWGPU_FISHER_STEP_RELATIVE 1     /* epsilon * |theta_i| (epsilon when theta_i == 0) */

typedef struct gwgpu_context gwgpu_context;
typedef struct gwgpu_server gwgpu_server;

/* POD mirror of the gen_params_base<double> fields on the path
 * (include/gwat/util.h:121-378).  Solar masses, Mpc, seconds, radians, Hz.
 * chip = -1 selects the full in-plane-spin transform for Pv2
 * (waveform_generator.cpp:1272-1281).  equatorial_orientation: the detector
 * response and the Fisher entry points take the inclination and polarisation
 * from theta_l, phi_l (the equatorial direction of the orbital angular
 * momentum), as fourier_detector_response does (waveform_util.cpp:946-948);
 * the likelihood entry points ignore it, as MCMC_likelihood_extrinsic does. */
typedef struct {
  double mass1, mass2;
  double spin1[3], spin2[3];
  double Luminosity_Distance;
  double incl_angle, phiRef, f_ref, tc;
  double RA, DEC, psi, gmst;
  double chip, phip;
  int32_t shift_time, shift_phase, sky_average, dep_postmerger;
  double theta_l, phi_l;
  int32_t equatorial_orientation, reserved;
} gwgpu_gen_params;

void gwgpu_default_params(gwgpu_gen_params *p);
const char *gwgpu_status_string(int status);

/* ---- context: one device, one HBM budget, device-resident data registry ---- */
int gwgpu_context_create(int device, size_t hbm_budget_bytes, gwgpu_context **out);
int gwgpu_context_destroy(gwgpu_context *ctx);
const char *gwgpu_last_error_string(gwgpu_context *ctx);
/* The context's default stream (a cudaStream_t), for callers that time or
 * order work around the engine. */
void *gwgpu_context_stream(gwgpu_context *ctx);
size_t gwgpu_context_bytes_in_use(gwgpu_context *ctx);

/* ---- waveform and detector response ---- */
/* fourier_waveform(double*, int, std::complex<double>* hplus, hcross, std::string,
 * gen_params*)  (waveform_generator.h:70-74, waveform_generator.cpp:104-300).
 * generation_method: "IMRPhenomD" or "IMRPhenomPv2".  Returns 1 on success,
 * 0 on failure (reference convention). */
int gwgpu_fourier_waveform(gwgpu_context *ctx, const double *frequencies, int length, double *hplus,
                           double *hcross, const char *generation_method, const gwgpu_gen_params *params);

/* fourier_detector_response(T*, int, std::complex<T>*, std::string detector,
 * std::string method, gen_params_base<T>*, T *times)  (waveform_util.h:190-197,
 * waveform_util.cpp:1070-1088), ground detectors, equatorial coordinates.
 * Returns 1 on success, 0 on failure. */
int gwgpu_fourier_detector_response(gwgpu_context *ctx, const double *frequencies, int length, double *response,
                                    const char *detector, const char *generation_method,
                                    const gwgpu_gen_params *params);

/* transform_orientation_coords(gen_params_base<T>*, std::string
 * generation_method, std::string detector)  (waveform_util.h:229,
 * waveform_util.cpp:1523-1586) for a ground detector: sets incl_angle and psi
 * from theta_l, phi_l, RA, DEC (IMRPhenomPv2: psi of the total angular
 * momentum from chip, phip and the aligned spins).  Host only, no launch. */
int gwgpu_transform_orientation_coords(gwgpu_gen_params *params, const char *generation_method);

/* ---- data registry (replaces the process-global mcmc_data/mcmc_noise/
 * mcmc_frequencies pointers set at mcmc_gw.cpp:1464-1476) ---- */
int gwgpu_data_register(gwgpu_context *ctx, const char *detector, const double *frequencies, int length,
                        const double *data, const double *psd, int *handle);
/* The same for the "GAUSSLEG" integration of Log_Likelihood_internal
 * (mcmc_gw.cpp:820-833, 843-862): integral = 4 sum_i weights[i] integrand[i],
 * times frequencies[i] ln 10 when log10F (the sampler's GAUSS_QUAD option,
 * mcmc_gw.cpp:2608-2610).  Every form integrates such a stream with its
 * weights; the mixed form still needs a uniform grid with f0 a multiple of df. */
int gwgpu_data_register_weighted(gwgpu_context *ctx, const char *detector, const double *frequencies, int length,
                                 const double *data, const double *psd, const double *weights, int log10F,
                                 int *handle);
int gwgpu_data_release(gwgpu_context *ctx, int handle);

/* ---- plain form: FP64, one request per launch (the drop-in) ---- */
/* Log_Likelihood_internal(std::complex<double>* data, double* psd, double* freqs,
 * double* weights, std::complex<double>* response, int length, bool log10F,
 * std::string "SIMPSONS")  (mcmc_gw.h:276, mcmc_gw.cpp:801-873). */
int gwgpu_log_likelihood_internal(gwgpu_context *ctx, const double *data, const double *psd,
                                  const double *frequencies, const double *response, int length, double *out);
/* The "GAUSSLEG" branch of Log_Likelihood_internal (mcmc_gw.cpp:820-833,
 * 843-862): weights[i], times frequencies[i] ln 10 when log10F. */
int gwgpu_log_likelihood_internal_weighted(gwgpu_context *ctx, const double *data, const double *psd,
                                           const double *frequencies, const double *weights, const double *response,
                                           int length, int log10F, double *out);

/* MCMC_likelihood_extrinsic(bool save_waveform, gen_params_base<double>*, std::string
 * method, int* lengths, double** freqs, std::complex<double>** data, double** psd,
 * double** weights, std::string "SIMPSONS", bool log10F, std::string* detectors,
 * int num_detectors)  (mcmc_gw.h:473, mcmc_gw.cpp:2374-2487), over registered
 * data.  T_segment is the value the reference forms at mcmc_gw.cpp:2466 before
 * t_c <- T_segment - t_c; params is not mutated. */
int gwgpu_mcmc_likelihood_extrinsic(gwgpu_context *ctx, const gwgpu_gen_params *params,
                                    const char *generation_method, const int *handles, int num_detectors,
                                    double T_segment, double *loglik);

/* No counterpart in the reference.  The same plain FP64 likelihood for callers
 * that may not allocate memory while it runs (a fixed memory budget, or code
 * that must not call an allocator on this path): it allocates nothing, enqueues one launch on
 * `stream` (0: the legacy default stream) and writes log L to the device
 * pointer d_loglik without synchronising.  Its scratch is one fixed device
 * array sized for grids of up to 524,288 bins (4,096 blocks of 128 bins);
 * longer grids return GWGPU_ETOOLARGE.  Every call looks the array's device
 * address up again (cudaGetSymbolAddress, which allocates nothing), so the
 * entry point stays valid across a device reset; the first call on a device
 * also loads the kernels' module, so make one call before any stream capture
 * that later calls belong to.  Calls share the array:
 * overlapping calls (several host threads, or work in flight on several
 * streams) race, so issue them in order on one stream.  A request outside the
 * model domain returns GWGPU_EDOMAIN without a launch. */
int gwgpu_mcmc_likelihood_extrinsic_noalloc(gwgpu_context *ctx, const gwgpu_gen_params *params,
                                            const char *generation_method, const int *handles,
                                            int num_detectors, double T_segment, double *d_loglik, void *stream);

/* ---- likelihood maximised over arrival time and phase ---- */
/* maximized_Log_Likelihood_aligned_spin_internal(std::complex<double>* data,
 * double* psd, double* frequencies, std::complex<double>* response, size_t length,
 * fftw_outline* plan)  (mcmc_gw.h, mcmc_gw.cpp:595-658): 1/2 max_t |DFT(4 d* r / S)|^2
 * df^2 / HH, HH = 4 S(|r|^2 / S) by Simpson's rule.  Uniform grid. */
int gwgpu_maximized_log_likelihood_internal(gwgpu_context *ctx, const double *data, const double *psd,
                                            const double *frequencies, const double *response, int length,
                                            double *out);
/* maximized_Log_Likelihood_unaligned_spin_internal(std::complex<double>* data,
 * double* psd, double* frequencies, std::complex<double>* hplus,
 * std::complex<double>* hcross, size_t length, fftw_outline* plan)
 * (mcmc_gw.cpp:660-800): the maximum over arrival time, phase and polarisation
 * of 1/4 lambda built from the normalised h+ and hx transforms and their
 * overlap.  Uniform grid. */
int gwgpu_maximized_log_likelihood_unaligned_internal(gwgpu_context *ctx, const double *data, const double *psd,
                                                      const double *frequencies, const double *hplus,
                                                      const double *hcross, int length, double *out);
/* The sampler's intrinsic mode (MCMC_likelihood_wrapper, mcmc_gw.cpp:2611-2720):
 * for each request, the waveform with the extrinsic parameters fixed as there
 * (horizon frame theta = phi = psi = 0, inclination 0, phiRef 1, tc 1; f_ref
 * 10 for IMRPhenomD, 20 for IMRPhenomPv2), evaluated on the grid of the
 * request's first detector, and summed over its detectors: the aligned form
 * with r = h+ for GWGPU_IMRPHENOMD, the unaligned form for GWGPU_IMRPHENOMPV2.
 * One grid length for the whole batch (handles[i*num_detectors + d]).
 * status[i]: GWGPU_OK or GWGPU_EDOMAIN (loglik[i] NaN). */
int gwgpu_maximized_loglik_batch(gwgpu_context *ctx, const gwgpu_gen_params *params, int n, int approximant,
                                 const int *handles, int num_detectors, double *loglik, int *status);

/* ---- data and noise ingestion (the formats feeding the registered streams) ---- */
/* count_lines_data_file / count_lines_LOSC_data_file / count_lines_LOSC_PSD_file
 * (io_util.h:56-58, io_util.cpp:682-714): the file's line count as
 * std::getline yields lines, less the 3 (strain) or 1 (PSD) header lines.
 * GWGPU_ENOTFOUND when the file cannot be read. */
int gwgpu_count_lines_data_file(const char *path, int *count);
int gwgpu_count_lines_losc_data_file(const char *path, int *count);
int gwgpu_count_lines_losc_psd_file(const char *path, int *count);
/* read_LOSC_data_file(std::string filename, double* output, double*
 * data_start_time, double* duration, double* fs)  (io_util.h:27,
 * io_util.cpp:403-464): line 1's digit-led tokens give fs, line 2's the GPS
 * start and the duration, the comma-separated values from line 3 on are the
 * samples.  *count (may be null) gets the number of samples; capacity
 * bounds output (GWGPU_ETOOLARGE beyond it, with *count set).  GWGPU_EINVAL where a value does not parse (the
 * reference throws). */
int gwgpu_read_losc_data_file(const char *path, double *output, long long capacity, long long *count,
                              double *data_start_time, double *duration, double *fs);
/* read_LOSC_PSD_file(std::string filename, double** output, int rows, int cols)
 * (io_util.h:33, io_util.cpp:466-500): the first line skipped, then
 * white-space separated values into output[rows*cols] (row-major); rows the
 * file does not fill are zero. */
int gwgpu_read_losc_psd_file(const char *path, double *output, int rows, int cols);
/* populate_noise(double* frequencies, std::string detector, double*
 * noise_root, int length, double integration_time)  (detector_util.h:168,
 * detector_util.cpp:86-283) for the ground-detector curves: "aLIGO_analytic",
 * "Hanford_O1_fitted", and the tabulated curves ("AdLIGODesign", "CE2",
 * "ET-D", ... the reference's interp_PSD_models names) interpolated linearly
 * from their CSV file in noise_dir (the reference's share/noise_data).  The
 * LISA curves are not part of this library.  Frequencies outside a table give
 * NaN and GWGPU_EDOMAIN (the reference's GSL error). */
int gwgpu_populate_noise(const double *frequencies, const char *detector, double *noise_root, int length,
                         double integration_time, const char *noise_dir);
/* allocate_LOSC_data(std::string* data_files, std::string psd_file, int
 * num_detectors, int psd_length, int data_file_length, double trigger_time,
 * double post_merger_duration, std::complex<double>** data, double** psds,
 * double** freqs)  (io_util.h:38, io_util.cpp:523-664): the strain files are
 * parsed in parallel, then as gwgpu_losc_prepare.  Outputs flat:
 * data[num_detectors][psd_length] complex (interleaved), psds and freqs
 * [num_detectors][psd_length]. */
int gwgpu_allocate_losc_data(gwgpu_context *ctx, const char *const *data_files, const char *psd_file,
                             int num_detectors, int psd_length, int data_file_length, double trigger_time,
                             double post_merger_duration, double *data, double *psds, double *freqs);
/* The transform step of allocate_LOSC_data from strain already in memory:
 * series[num_detectors][series_length], psd_table[psd_length][num_detectors+1]
 * (frequency, then one PSD column per detector).  T_obs = 1/(f_1 - f_0) of the
 * table; the samples with trigger - (T_obs - post) < t <= trigger + post are
 * Tukey-windowed (alpha = 0.8/T_obs), transformed on the device (forward DFT,
 * times dt) and the bins k/T_obs inside the table's band kept.  psds and freqs
 * are filled first; GWGPU_EDOMAIN when the window does not fit in the file.
 * *bins_out (may be null) gets the number of data bins filled; the rest are
 * zero. */
int gwgpu_losc_prepare(gwgpu_context *ctx, const double *series, int num_detectors, long long series_length,
                       double file_start, double duration, double fs, const double *psd_table, int psd_length,
                       double trigger_time, double post_merger_duration, double *data, double *psds,
                       double *freqs, int *bins_out);

/* ---- batched form: n requests, one fused launch per step ---- */
/* n independent MCMC_likelihood_extrinsic evaluations (the sampler calls
 * mcmc_step -> sampler->ll once per chain, mcmc_sampler_internals.cpp:98).
 * approximants[i] is GWGPU_IMRPHENOMD or GWGPU_IMRPHENOMPV2; all detectors of
 * one request share one grid; requests may use different grids (handles per
 * request: handles[i*num_detectors + d]).  T_segment <= 0 selects 1/df of
 * each request's own grid.  status[i] is GWGPU_OK or GWGPU_EDOMAIN (loglik[i]
 * = NaN then). */
int gwgpu_loglik_batch(gwgpu_context *ctx, const gwgpu_gen_params *params, const int *approximants, int n,
                       const int *handles, int num_detectors, double T_segment, int precision, double *loglik,
                       int *status);
/* Same with params, approximants, log L and status arrays already on the
 * device (handles stay a host array), enqueued on `stream` (a cudaStream_t or
 * NULL for the context stream); asynchronous.  Repeated calls with the same
 * shape and pointers replay one captured CUDA graph. */
int gwgpu_loglik_batch_device(gwgpu_context *ctx, const gwgpu_gen_params *d_params, const int *d_approximants,
                              int n, const int *handles, int num_detectors, double T_segment, int precision,
                              double *d_loglik, int *d_status, void *stream);
/* MCMC_likelihood_wrapper(double *param, ...) (mcmc_gw.h:491, mcmc_gw.cpp:2569)
 * for n parameter vectors: MCMC_prep_params + repack_parameters (MCMC_IMRPhenomD
 * 11-dim, MCMC_IMRPhenomPv2 15-dim), then the batched likelihood. */
int gwgpu_mcmc_loglik_batch(gwgpu_context *ctx, const double *theta, int dim, int n, int approximant,
                            double gmst, const int *handles, int num_detectors, double T_segment, int precision,
                            double *loglik, int *status);

/* Tile (bins per work item, a multiple of 256; 0 = autotuned/default) of the
 * batched kernels, and whether repeated batch shapes replay a captured CUDA
 * graph (default on). */
int gwgpu_batch_set_tile(gwgpu_context *ctx, int tile);
/* Resident blocks per SM of the mixed form's fused kernel (3 or 4; 0 =
 * autotuned or default), the launch shape's second coordinate. */
int gwgpu_batch_set_blocks_per_sm(gwgpu_context *ctx, int blocks);
/* Launch shape of the last batch on the context stream: bin tile, resident
 * blocks per SM and grid of the fused kernel. */
int gwgpu_batch_last_launch_shape(gwgpu_context *ctx, int *tile, int *blocks_per_sm, int *grid);
int gwgpu_batch_use_graphs(gwgpu_context *ctx, int on);
/* Per-kernel timing of context-stream batches (graphs bypassed while on):
 * CUDA events around the prologue and the fused bin kernel of the last batch. */
int gwgpu_batch_timing(gwgpu_context *ctx, int on);
int gwgpu_batch_last_timing(gwgpu_context *ctx, float *prologue_ms, float *kernel_ms);
/* Autotuner: time the candidate launch shapes -- bin tile x resident blocks
 * per SM of the fused kernel (mixed form) -- on this batch (device arrays as
 * for gwgpu_loglik_batch_device; results are overwritten) and keep the
 * fastest for batches of the same precision, detector count, length class of
 * the longest grid and evenness (all requests on one grid length or not). */
int gwgpu_batch_autotune(gwgpu_context *ctx, const gwgpu_gen_params *d_params, const int *d_approximants, int n,
                         const int *handles, int num_detectors, double T_segment, int precision, double *d_loglik,
                         int *d_status, int *best_tile, float *best_ms);

/* ---- Fisher ---- */
/* fisher_numerical(double* freqs, int length, string method, string detector,
 * string reference_detector, double** output, int dimension, gen_params_base<double>*,
 * int order, int*, int*, double* noise)  (fisher.h:35-48, fisher.cpp:81-146).
 * method "IMRPhenomD" or "MCMC_IMRPhenomD"; output dimension*dimension row major;
 * order 2 or 4; epsilon 1e-8 absolute as the reference.  Returns GWGPU_OK. */
int gwgpu_fisher_numerical(gwgpu_context *ctx, const double *frequencies, int length, const char *generation_method,
                           const char *detector, const char *reference_detector, double *output, int dimension,
                           const gwgpu_gen_params *params, int order, const double *noise);
/* Batched network Fisher (MCMC_fisher_wrapper summing detectors,
 * mcmc_gw.cpp:2283-2317) for n sources over registered data: fisher[n][dim][dim]
 * and, if covariance != NULL, its FP64 inverse (gsl_cholesky_matrix_invert,
 * util.cpp:857-900).  Order 2, the moment form: FP64 waveform differences,
 * weights and Gram moment sums per bin (gwgpu_fisher_batch_ex with
 * GWGPU_FISHER_MOMENTS and GWGPU_PREC_FP64).  A source whose matrix that form
 * cannot invert is recomputed with the FP64 reference algorithm.  status[i]:
 * GWGPU_OK, GWGPU_EDOMAIN, GWGPU_ESINGULAR (not invertible in FP64 either). */
int gwgpu_fisher_batch(gwgpu_context *ctx, const gwgpu_gen_params *params, int n, int method, const int *handles,
                       int num_detectors, double epsilon, int step_mode, double *fisher, double *covariance,
                       int *status);
#define GWGPU_FISHER_REFERENCE 0   /* the reference's algorithm: every perturbed response in FP64 (orders 2 and 4) */
#define GWGPU_FISHER_MOMENTS 1     /* order 2: analytic extrinsic derivatives, per-bin waveform differences, moment sums */
typedef struct {
  int method;     /* GWGPU_FISHER_IMRPHENOMD or GWGPU_FISHER_MCMC_IMRPHENOMD */
  int order;      /* 2 (central) or 4 (five-point, fisher.cpp:426-458) */
  double epsilon; /* step (the reference: 1e-8) */
  int step_mode;  /* GWGPU_FISHER_STEP_* */
  int precision;  /* GWGPU_PREC_FP64; the moment form also takes GWGPU_PREC_MIXED (FP32 values, compensated FP32 sums) */
  int add_prior;  /* add MCMC_fisher_transformations' prior diagonal (mcmc_gw.cpp:2136-2160) */
  int algorithm;  /* GWGPU_FISHER_REFERENCE (0) or GWGPU_FISHER_MOMENTS */
} gwgpu_fisher_options;
/* fisher_numerical (fisher.h:35-48, fisher.cpp:81-557, 2704-2781) for n
 * sources, summed over the detectors with the first as reference detector.
 * GWGPU_FISHER_REFERENCE runs the reference's algorithm itself on the device:
 * every perturbed response in FP64 (including the constant phase the +-2 eps
 * responses of the five-point rule carry at a non-reference detector,
 * fisher.cpp:426-458), derivatives and Simpson Gram sums in FP64.
 * GWGPU_FISHER_MOMENTS is the form of gwgpu_fisher_batch, its sums in the
 * given precision; at order 4 it takes the five-point rule with that constant
 * phase analytically (each derivative at a non-reference detector becomes
 * kappa r' + c r, kappa = (4 - e^{i phq}) / 3, phq = 2 pi DTOA f_ref, c from
 * the sky position's change of phq), and a source with a pair it takes bin by
 * bin (eta at 1/4, a waveform's cut between the steps) is computed with the
 * reference algorithm. */
int gwgpu_fisher_batch_ex(gwgpu_context *ctx, const gwgpu_gen_params *params, int n, const int *handles,
                          int num_detectors, const gwgpu_fisher_options *options, double *fisher, double *covariance,
                          int *status);
/* MCMC_fisher_wrapper(double *param, double **output, mcmc_data_interface*,
 * void*)  (mcmc_gw.h:486, mcmc_gw.cpp:2230-2340) for n sampler positions: the
 * 11-dim MCMC_IMRPhenomD vector repacked as MCMC_prep_params does (f_ref 20,
 * the given GMST), fisher_numerical("MCMC_IMRPhenomD", order 4 =
 * mcmc_deriv_order, mcmc_gw.h:45, epsilon 1e-8) summed over the detectors with
 * the first as reference, plus the prior diagonal of
 * MCMC_fisher_transformations, in the moment form with FP64 sums at order 4
 * (gwgpu_fisher_batch_ex, GWGPU_FISHER_MOMENTS).  fisher[n][11][11]; status
 * as above. */
int gwgpu_mcmc_fisher_batch(gwgpu_context *ctx, const double *theta, int dim, int n, int approximant, double gmst,
                            const int *handles, int num_detectors, double *fisher, int *status);

/* ---- serving: continuous batching of log-likelihood requests ----
 * The reference serves one chain per host thread (mcmc_sampler.cpp:4585-4590,
 * each calling MCMC_likelihood_wrapper).  Here requests from any number of
 * chains / temperatures / ensembles are submitted into request slots; a
 * scheduler keeps up to `lanes` fused batches in flight on separate streams
 * and admits queued requests into the next launch as lanes and HBM budget
 * free up.  Results are the same alone and in any mix.
 *
 * device_loop = 1 selects the device-resident request loop instead (mixed
 * precision): requests go into a ring in mapped pinned memory, and one
 * persistent kernel on every SM claims them as they are published, runs
 * their prologues, queues their items and evaluates them, writing each
 * result and a completion sequence number back into mapped memory.  The
 * ring's size is max_inflight, reduced to what hbm_budget_bytes admits
 * (per-slot device state allocated at creation); max_batch and lanes are
 * not used.  A launch's blocks leave after idle_us without work (and at the
 * latest one second after the launch); the host relaunches while requests
 * are outstanding.  Every request of one such server has the same number
 * of detectors, and grids no longer than the longest grid registered when
 * the server was created.  While its kernel is resident (requests flowing,
 * and idle_us after the last) it holds every SM: other kernels on the GPU,
 * including a second device-loop server's, start when its blocks leave, so
 * run one device loop per GPU and lower idle_us where other calls share it,
 * or give it fewer blocks per SM (blocks_per_sm) to leave room beside it. */
typedef struct {
  int max_inflight;          /* request slots (submitted, not yet collected) */
  int max_batch;             /* requests per fused launch */
  int lanes;                 /* batches in flight at once, 1..16 */
  int precision;             /* GWGPU_PREC_* */
  double T_segment;          /* as for gwgpu_mcmc_likelihood_extrinsic */
  size_t hbm_budget_bytes;   /* admission budget for in-flight scratch; 0 = the context budget */
  int device_loop;           /* 1: device-resident request loop (GWGPU_PREC_MIXED only) */
  int tile;                  /* device loop: bins per item, a multiple of 256 (0: 4096) */
  int idle_us;               /* device loop: idle time after which a launch's blocks leave (0: 20000) */
  int blocks_per_sm;         /* device loop: blocks it keeps on each SM, 1..3 (0: 3, the SM's capacity);
                                fewer leave room for other kernels while it is resident */
} gwgpu_server_config;
int gwgpu_server_create(gwgpu_context *ctx, const gwgpu_server_config *cfg, gwgpu_server **out);
int gwgpu_server_destroy(gwgpu_server *srv);
/* Queue one request; returns a ticket.  GWGPU_EBUSY when every slot is taken. */
int gwgpu_server_submit(gwgpu_server *srv, const gwgpu_gen_params *params, int approximant, const int *handles,
                        int num_detectors, uint64_t *ticket);
/* Non-blocking: GWGPU_OK with the result (the slot is freed), GWGPU_EBUSY while
 * still in flight, GWGPU_ENOTFOUND for an unknown or collected ticket. */
int gwgpu_server_poll(gwgpu_server *srv, uint64_t ticket, double *loglik, int *status);
/* Blocks until the ticket completes or timeout_ms passes (GWGPU_ETIMEDOUT). */
int gwgpu_server_wait(gwgpu_server *srv, uint64_t ticket, int timeout_ms, double *loglik, int *status);
/* Latency percentiles (seconds, submit -> result visible on host), counts. */
int gwgpu_server_stats(gwgpu_server *srv, double *p50, double *p99, uint64_t *completed, uint64_t *launches);
int gwgpu_server_reset_stats(gwgpu_server *srv);
/* Device loop state: info[0] ring slots, [1] bins per item, [2] items per
 * request at most, [3] blocks per launch, [4] launches, [5] blocks that left
 * idle, [6] on the host's stop, [7] at the end of a launch's life (counts
 * of finished launches), [8] and [9] p50 and p99 of the device service time
 * in ns (request claimed -> result written; since the last reset_stats),
 * [10] ns the blocks spent in items, [11] in prologues, [12] items,
 * [13] prologue claims, [14] requests claimed (since creation).
 * GWGPU_EINVAL for a host-scheduled server. */
int gwgpu_server_loop_info(gwgpu_server *srv, long long info[15]);
/* Load driver: submits request i at t0 + arrival_s[i] from the calling
 * thread (open loop, arrival time counted as submit time), collects every
 * result into loglik/status (request order) and the per-request latencies
 * (completion order); wall_s = time from t0 to the last result. */
int gwgpu_server_drive(gwgpu_server *srv, const gwgpu_gen_params *params, const int *approximants,
                       const int *handles, int num_detectors, const double *arrival_s, int n, double *loglik,
                       int *status, double *latency_s, double *wall_s);

#ifdef __cplusplus
}
#endif
#endif /* GWGPU_H */
