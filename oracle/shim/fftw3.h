/* Test-only FFTW type stand-ins for the oracle pin build. */
#ifndef GWO_SHIM_FFTW3_H
#define GWO_SHIM_FFTW3_H
typedef double fftw_complex[2];
typedef struct gwo_fftw_plan_s *fftw_plan;
#endif
