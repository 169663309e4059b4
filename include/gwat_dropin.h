// gwat_dropin.h -- the reference's C++ entry points of the likelihood path,
// same signatures, running on the GB300 engine (include/gwgpu.h).
//
// A maintainer links libgwat_dropin.so in place of the CPU definitions of
// these functions.  The parameter and polarisation types here are the subset
// of the reference's gen_params_base<T> (include/gwat/util.h:121-378) and
// waveform_polarizations<T> (include/gwat/waveform_generator.h:12-32) that the
// path reads; in the reference build the reference's own headers replace
// this block and the definitions in gwat_dropin.cpp are compiled against them.
#ifndef GWAT_DROPIN_H
#define GWAT_DROPIN_H

#include <complex>
#include <string>

#ifndef GWAT_DROPIN_USE_REFERENCE_HEADERS
template <class T>
class gen_params_base {
 public:
  T mass1 = 0, mass2 = 0;
  T spin1[3] = {0, 0, 0}, spin2[3] = {0, 0, 0};
  T Luminosity_Distance = 0;
  T incl_angle = 0, phiRef = 0, f_ref = 0, tc = 0;
  T RA = 0, DEC = 0, psi = 0;
  double gmst = 0;
  T chip = -1, phip = -1;
  bool shift_time = true, shift_phase = true, sky_average = false, dep_postmerger = false;
  bool equatorial_orientation = false, horizon_coord = false;
  T theta_l = 0, phi_l = 0;  // equatorial direction of L, read when equatorial_orientation is set
};
class gen_params : public gen_params_base<double> {};
template <class T>
struct waveform_polarizations {
  std::complex<T> *hplus = nullptr, *hcross = nullptr;
};
struct fftw_outline;  // the reference's FFTW plan holder (util.h:90); unused here
#endif

// fourier_waveform (waveform_generator.h:43-49, waveform_generator.cpp:104)
template <class T>
int fourier_waveform(T *frequencies, int length, waveform_polarizations<T> *wp, std::string generation_method,
                     gen_params_base<T> *parameters);
// fourier_waveform complex overload (waveform_generator.h:70-74)
int fourier_waveform(double *frequencies, int length, std::complex<double> *waveform_plus,
                     std::complex<double> *waveform_cross, std::string generation_method, gen_params *parameters);
// fourier_detector_response (waveform_util.h:190-197, waveform_util.cpp:1070)
template <class T>
int fourier_detector_response(T *frequencies, int length, std::complex<T> *response, std::string detector,
                              std::string generation_method, gen_params_base<T> *parameters, T *times = nullptr);
// Log_Likelihood_internal (mcmc_gw.h:276, mcmc_gw.cpp:801); SIMPSONS and GAUSSLEG
double Log_Likelihood_internal(std::complex<double> *data, double *psd, double *frequencies, double *weights,
                               std::complex<double> *detector_response, int length, bool log10F,
                               std::string integration_method);
// MCMC_likelihood_extrinsic (mcmc_gw.h:473, mcmc_gw.cpp:2374); SIMPSONS and
// GAUSSLEG, save_waveform = true (one waveform for every detector,
// waveform_util.cpp:153)
double MCMC_likelihood_extrinsic(bool save_waveform, gen_params_base<double> *parameters,
                                 std::string generation_method, int *data_length, double **frequencies,
                                 std::complex<double> **data, double **psd, double **weights,
                                 std::string integration_method, bool log10F, std::string *detectors,
                                 int num_detectors);
// maximized_Log_Likelihood_aligned_spin_internal (mcmc_gw.h:203-209,
// mcmc_gw.cpp:595) and maximized_Log_Likelihood_unaligned_spin_internal
// (mcmc_gw.h:219-226, mcmc_gw.cpp:660): the transform runs on the device, the
// plan argument is not used
double maximized_Log_Likelihood_aligned_spin_internal(std::complex<double> *data, double *psd, double *frequencies,
                                                      std::complex<double> *detector_response, size_t length,
                                                      fftw_outline *plan);
double maximized_Log_Likelihood_unaligned_spin_internal(std::complex<double> *data, double *psd, double *frequencies,
                                                        std::complex<double> *hplus, std::complex<double> *hcross,
                                                        size_t length, fftw_outline *plan);
// Data and noise ingestion (io_util.h:27-58, detector_util.h:168).  File
// errors keep the reference's behaviour: a missing file prints a message and
// exits, a value that does not parse throws std::invalid_argument.
void read_LOSC_data_file(std::string filename, double *output, double *data_start_time, double *duration,
                         double *fs);
void read_LOSC_PSD_file(std::string filename, double **output, int rows, int cols);
void allocate_LOSC_data(std::string *data_files, std::string psd_file, int num_detectors, int psd_length,
                        int data_file_length, double trigger_time, double post_merger_duration,
                        std::complex<double> **data, double **psds, double **freqs);
int count_lines_data_file(std::string file, int *count);
int count_lines_LOSC_PSD_file(std::string file, int *count);
int count_lines_LOSC_data_file(std::string file, int *count);
// populate_noise for the ground-detector curves; the tabulated curves are read
// from $GWGPU_NOISE_DIR (else GWAT_SHARE_DIR "noise_data/" when defined at
// build time, as the reference does)
void populate_noise(double *frequencies, std::string detector, double *noise_root, int length,
                    double integration_time = 48);
// fisher_numerical (fisher.h:35-48, fisher.cpp:81): "IMRPhenomD" / "MCMC_IMRPhenomD"
void fisher_numerical(double *frequency, int length, std::string generation_method, std::string detector,
                      std::string reference_detector, double **output, int dimension,
                      gen_params_base<double> *parameters, int order, int *amp_tapes = nullptr,
                      int *phase_tapes = nullptr, double *noise = nullptr);

// Engine behind the drop-in: GWGPU_DROPIN_DEVICE (default 0) and
// GWGPU_DROPIN_MODE = "plain" (default: one FP64 request per launch) or
// "served" (concurrent callers' requests served together, mixed precision);
// GWGPU_DROPIN_SERVER = "loop" (default: the device-resident request loop for
// the first segment length, host-scheduled batching for the rest) or "host"
// (host-scheduled batching only).  set_mode / set_server change them later.
namespace gwat_dropin {
void set_mode(const char *mode);
void set_server(const char *server);
}

#endif
