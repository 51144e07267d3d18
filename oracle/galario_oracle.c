/*
 * galario CPU oracle: a plain-C restatement of the reference CPU path
 * (galario v1.2.2 src/galario.cpp, FFTW + OpenMP back end) in double and
 * float.  Built by oracle/Makefile into oracle/_build/liboracle.so and loaded
 * with ctypes.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load this library, as the checker or the
 * timed CPU baseline.  The GPU product (galario_gb300/) never calls it.
 *
 * Status codes: 0 ok, 1 invalid argument (the reference throws
 * std::invalid_argument -> ValueError), 2 out of memory (std::bad_alloc ->
 * MemoryError).  orc_last_error() returns the message of the calling thread.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define ORC_API __attribute__((visibility("default")))
#define ORC_EINVAL 1
#define ORC_ENOMEM 2

static __thread char orc_errbuf[512];

static int orc_oom(void) {
    snprintf(orc_errbuf, sizeof orc_errbuf, "std::bad_alloc");
    return ORC_ENOMEM;
}

/* reference CHECK_INPUT, src/galario.cpp:101-105 */
static int orc_check_input(int nx) {
    if (nx < 2) {
        snprintf(orc_errbuf, sizeof orc_errbuf, "Error in check input image: x dimension = %d is less than 2", nx);
        return ORC_EINVAL;
    }
    if (nx % 2 != 0) {
        snprintf(orc_errbuf, sizeof orc_errbuf, "Error in check input image: x dimension = %d is odd", nx);
        return ORC_EINVAL;
    }
    return 0;
}

/* reference CHECK_INPUTXY, src/galario.cpp:107-111 */
static int orc_check_square(int nx, int ny) {
    if (nx != ny) {
        snprintf(orc_errbuf, sizeof orc_errbuf,
                 "Error in check input image: Expect a square image but got shape (%d, %d)", nx, ny);
        return ORC_EINVAL;
    }
    return orc_check_input(nx);
}

ORC_API const char *orc_last_error(void) { return orc_errbuf; }

/* reference threads(), src/galario.cpp:367-390 (OpenMP branch) */
ORC_API int orc_threads(int num) {
#ifdef _OPENMP
    static int nthreads = 0;
    if (nthreads == 0) nthreads = omp_get_max_threads();
    if (num > 0) {
        nthreads = num;
        omp_set_dynamic(0);
        omp_set_num_threads(num);
    }
    return nthreads;
#else
    (void)num;
    return 1;
#endif
}

/* ---- double instantiation ---- */
#define REAL double
#define SFX(name) name##_d
#include "orc_fft_impl.h"
#include "orc_galario_impl.h"
#undef REAL
#undef SFX

/* ---- float instantiation ---- */
#define REAL float
#define SFX(name) name##_f
#include "orc_fft_impl.h"
#include "orc_galario_impl.h"
#undef REAL
#undef SFX
