/* Test-only FFTW stand-ins for the oracle pin build: the types and
 * declarations the reference headers and sources name.  The functions are
 * defined, where the pinned path needs them, by oracle/ref_fftw.cpp (a direct
 * DFT), else by the generated link stubs. */
#ifndef GWO_SHIM_FFTW3_H
#define GWO_SHIM_FFTW3_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef double fftw_complex[2];
typedef struct gwo_fftw_plan_s *fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out);
void fftw_destroy_plan(fftw_plan p);
void fftw_cleanup(void);
#ifdef __cplusplus
}
#endif
#endif
