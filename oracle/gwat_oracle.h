/*
 * gwat_oracle.h -- FP64 CPU oracle for the gw_analysis_tools likelihood path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * IMRPhenomD / IMRPhenomPv2 waveform, detector projection, Simpson inner
 * product, extrinsic log-likelihood and numerical Fisher matrix.  It is the
 * checker the CUDA path is compared against (tests/, the smoke check and the
 * CPU-baseline leg of bench.py); no product code links it.
 *
 * Each function cites the reference file:line it restates.  The restatement
 * is pinned against the reference's own IMRPhenomD.cpp / IMRPhenomP.cpp,
 * compiled here against test-only shim headers (oracle/ref_build.sh ->
 * oracle/_ref/), see tests/test_oracle_pins.py.
 */
#ifndef GWAT_ORACLE_H
#define GWAT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { GWO_IMRPHENOMD = 0, GWO_IMRPHENOMPV2 = 1 };

/* Mirror of the gen_params_base<double> fields the path reads
 * (reference include/gwat/util.h:121-378).  Units: solar masses, Mpc,
 * seconds, radians, Hz. */
typedef struct {
  double mass1, mass2;
  double spin1[3], spin2[3];
  double Luminosity_Distance;
  double incl_angle, phiRef, f_ref, tc;
  double RA, DEC, psi, gmst;
  double chip, phip;          /* reduced Pv2 spins; chip = -1 selects the full transform */
  int shift_time, shift_phase, sky_average, dep_postmerger;
  /* equatorial spherical angles of the orbital angular momentum, read when
   * equatorial_orientation is set (util.h:166-172) */
  double theta_l, phi_l;
  int equatorial_orientation, reserved;
} gwo_gen_params;

void gwo_default_params(gwo_gen_params *p);

/* fourier_waveform (waveform_generator.cpp:104-300), D and Pv2 branches.
 * hplus/hcross: interleaved complex128 [2*length].  Returns 1 (reference
 * convention) or 0 on bad input. */
int gwo_fourier_waveform(const double *freqs, int length, double *hplus, double *hcross,
                         int approximant, const gwo_gen_params *p);

/* Detector index from name (Hanford, Livingston, Virgo, Kagra, Indigo, CE,
 * ET1..3 and lower-case forms; detector_util.cpp:1037-1160).  -1 if unknown. */
int gwo_detector_index(const char *name);
/* F+, Fx for one detector (detector_util.cpp:901-1015, geometric factor :1160). */
void gwo_antenna(int det, double ra, double dec, double psi, double gmst, double *fplus, double *fcross);
/* DTOA_DETECTOR (detector_util.cpp:677-790). */
double gwo_dtoa(double ra, double dec, double gmst, int det1, int det2);

/* transform_orientation_coords (waveform_util.cpp:1523-1586) for a ground
 * detector: incl_angle and psi from theta_l, phi_l (and, for IMRPhenomPv2, the
 * total angular momentum from chip, phip and the aligned spins). */
void gwo_transform_orientation_coords(gwo_gen_params *p, int approximant);

/* fourier_detector_response, equatorial (waveform_util.cpp:1070-1088 ->
 * :936-985 -> :725-905); with equatorial_orientation set, the orientation
 * transform is applied to a copy of p first. */
int gwo_fourier_detector_response(const double *freqs, int length, double *response, int det,
                                  int approximant, const gwo_gen_params *p);

/* Log_Likelihood_internal, SIMPSONS branch (mcmc_gw.cpp:801-873). */
double gwo_log_likelihood_internal(const double *data, const double *psd, const double *freqs,
                                   const double *response, int length);

/* The GAUSSLEG branch (mcmc_gw.cpp:820-833, 843-862): weights w_i, log10F
 * multiplies each term by f_i ln 10. */
double gwo_log_likelihood_internal_gl(const double *data, const double *psd, const double *freqs,
                                      const double *weights, const double *response, int length, int log10F);
double gwo_loglik_extrinsic_gl(const gwo_gen_params *p, int approximant, double T_segment, const double *freqs,
                               int length, int ndet, const int *dets, const double *const *data,
                               const double *const *psd, const double *const *weights, int log10F);

/* MCMC_likelihood_extrinsic (mcmc_gw.cpp:2374-2487) with save_waveform=true.
 * T_segment is the value the reference forms at mcmc_gw.cpp:2466 before
 * t_c <- T_segment - t_c; p is copied, not mutated.  data/psd are per detector,
 * all on the grid freqs (length). */
double gwo_loglik_extrinsic(const gwo_gen_params *p, int approximant, double T_segment,
                            const double *freqs, int length, int ndet, const int *dets,
                            const double *const *data, const double *const *psd);

/* MCMC parameter vector -> gen params, MCMC_prep_params (mcmc_gw.cpp:2492-2510)
 * + repack_parameters MCMC branches (fisher.cpp:2171-2284).  dim 11 (D) or
 * 15 (Pv2). */
void gwo_mcmc_repack(const double *theta, int dim, int approximant, double gmst, gwo_gen_params *out);

/* Batch of extrinsic log-likelihoods with OpenMP over requests (one request
 * per thread, as the reference sampler does). nthreads<=0: all cores. */
void gwo_loglik_batch(const gwo_gen_params *p, int n, const int *approximant, double T_segment,
                      const double *freqs, int length, int ndet, const int *dets,
                      const double *const *data, const double *const *psd, double *out, int nthreads);

/* fisher_numerical (fisher.cpp:81-146) -> calculate_derivatives (:148-557,
 * non-sky-averaged branch :337-545) -> calculate_fisher_elements (:2704-2781).
 * method: 0 = "IMRPhenomD" (11 params), 1 = "MCMC_IMRPhenomD" (11),
 * 2 = "IMRPhenomPv2" (13), 3 = "MCMC_IMRPhenomPv2" (15).
 * step_mode 0: absolute epsilon (the reference: 1e-8, fisher.cpp:158);
 * step_mode 1: epsilon * |theta_i| (relative, epsilon*1 when theta_i == 0).
 * out: dim*dim row major.  Returns dim or 0 on error. */
int gwo_fisher_numerical(const double *freqs, int length, int method, int det, int ref_det,
                         double *out, const gwo_gen_params *p, int order, const double *psd,
                         double epsilon, int step_mode);

/* Network Fisher: sum over detectors with ref = dets[0] (mcmc_gw.cpp:2283-2317). */
int gwo_fisher_network(const double *freqs, int length, int method, int ndet, const int *dets,
                       double *out, const gwo_gen_params *p, int order, const double *const *psd,
                       double epsilon, int step_mode);
void gwo_fisher_batch(const gwo_gen_params *p, int n, const double *freqs, int length, int method,
                      int ndet, const int *dets, const double *const *psd, double epsilon,
                      int step_mode, double *out, int nthreads);

/* Pivoted-Cholesky inverse of a symmetric positive definite matrix
 * (gsl_cholesky_matrix_invert, util.cpp:857-900).  Returns 0 on success. */
int gwo_cholesky_invert(const double *a, double *inv, int dim);

/* Natural cubic spline (GSL "cspline" boundary conditions): value and first
 * derivative.  Used for the QNM table (IMRPhenomD.cpp:1183-1217) and the Pv2
 * time shift (IMRPhenomP.cpp:551-606). */
void gwo_cspline_coeffs(const double *x, const double *y, int n, double *c);
double gwo_cspline_eval(const double *x, const double *y, const double *c, int n, double xv, int deriv);

/* Analytic PSD used by the benchmark workloads:
 * S(f) = 1e-49 [x^-4.14 - 5 x^-2 + 111 (1 - x^2 + x^4/2)/(1 + x^2/2)], x = f/215 Hz. */
double gwo_analytic_psd(double f);

#ifdef __cplusplus
}
#endif
#endif
