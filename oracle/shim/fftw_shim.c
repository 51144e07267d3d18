/*
 * FFTW3-API shim for building the reference's src/galario.cpp here (see
 * shim/fftw3.h).  Plans only record the in-place R2C geometry; execution runs
 * the oracle's 2D R2C (oracle/orc_fft_impl.h) in double or float.
 *
 * TEST INFRASTRUCTURE ONLY.
 */
#define _GNU_SOURCE
#include <stdlib.h>
#include <string.h>
#include "fftw3.h"

#define REAL double
#define SFX(name) name##_d
#include "../orc_fft_impl.h"
#undef REAL
#undef SFX
#define REAL float
#define SFX(name) name##_f
#include "../orc_fft_impl.h"
#undef REAL
#undef SFX

struct orc_fftw_plan_s {
    int n0, n1, is_double;
    void *in, *out;
};

static struct orc_fftw_plan_s *make_plan(int n0, int n1, void *in, void *out, int is_double) {
    struct orc_fftw_plan_s *p = (struct orc_fftw_plan_s *)malloc(sizeof *p);
    if (!p) return NULL;
    p->n0 = n0; p->n1 = n1; p->in = in; p->out = out; p->is_double = is_double;
    return p;
}

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags) {
    (void)flags;
    return make_plan(n0, n1, in, out, 1);
}
fftwf_plan fftwf_plan_dft_r2c_2d(int n0, int n1, float *in, fftwf_complex *out, unsigned flags) {
    (void)flags;
    return make_plan(n0, n1, in, out, 0);
}

/* galario only plans in place: in == out (src/galario.cpp:515-519) */
static void run(const struct orc_fftw_plan_s *p) {
    if (!p || p->in != p->out) abort();
    if (p->is_double) {
        if (orc_rfft2_inplace_d(p->n0, p->n1, (double *)p->in)) abort();
    } else {
        if (orc_rfft2_inplace_f(p->n0, p->n1, (float *)p->in)) abort();
    }
}
void fftw_execute(const fftw_plan p) { run(p); }
void fftwf_execute(const fftwf_plan p) { run(p); }
void fftw_destroy_plan(fftw_plan p) { free(p); }
void fftwf_destroy_plan(fftwf_plan p) { free(p); }

static void *aligned(size_t bytes) {
    void *p = NULL;
    if (posix_memalign(&p, 64, bytes ? bytes : 64)) return NULL;
    return p;
}
fftw_complex *fftw_alloc_complex(size_t n) { return (fftw_complex *)aligned(n * sizeof(fftw_complex)); }
fftwf_complex *fftwf_alloc_complex(size_t n) { return (fftwf_complex *)aligned(n * sizeof(fftwf_complex)); }
double *fftw_alloc_real(size_t n) { return (double *)aligned(n * sizeof(double)); }
float *fftwf_alloc_real(size_t n) { return (float *)aligned(n * sizeof(float)); }
void fftw_free(void *p) { free(p); }
void fftwf_free(void *p) { free(p); }
void fftw_plan_with_nthreads(int nthreads) { (void)nthreads; }
void fftwf_plan_with_nthreads(int nthreads) { (void)nthreads; }
int fftw_init_threads(void) { return 1; }
int fftwf_init_threads(void) { return 1; }
void fftw_cleanup_threads(void) {}
void fftwf_cleanup_threads(void) {}
void fftw_cleanup(void) {}
void fftwf_cleanup(void) {}
