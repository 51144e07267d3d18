/*
 * Minimal FFTW3-API header, written for this project, so that the reference's
 * own src/galario.cpp (CPU back end) compiles unchanged in a container that
 * has no FFTW.  Only the symbols galario.cpp uses are declared
 * (src/galario.cpp:358-361,400,415-417,425,469,516-524,1335).  The transform
 * behind them is the oracle FFT (oracle/orc_fft_impl.h), itself checked
 * against numpy.fft by the tests.
 *
 * TEST INFRASTRUCTURE ONLY (builds the reference into oracle/_ref/).
 */
#pragma once
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

#define FFTW_ESTIMATE (1U << 6)

typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct orc_fftw_plan_s *fftw_plan;
typedef struct orc_fftw_plan_s *fftwf_plan;

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_2d(int n0, int n1, float *in, fftwf_complex *out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftwf_execute(const fftwf_plan p);
void fftw_destroy_plan(fftw_plan p);
void fftwf_destroy_plan(fftwf_plan p);
fftw_complex *fftw_alloc_complex(size_t n);
fftwf_complex *fftwf_alloc_complex(size_t n);
double *fftw_alloc_real(size_t n);
float *fftwf_alloc_real(size_t n);
void fftw_free(void *p);
void fftwf_free(void *p);
void fftw_plan_with_nthreads(int nthreads);
void fftwf_plan_with_nthreads(int nthreads);
int fftw_init_threads(void);
int fftwf_init_threads(void);
void fftw_cleanup_threads(void);
void fftwf_cleanup_threads(void);
void fftw_cleanup(void);
void fftwf_cleanup(void);

#ifdef __cplusplus
}
#endif
