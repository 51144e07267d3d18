/*
 * Oracle FFT: the 2D real-to-complex transform the galario CPU path gets
 * from FFTW (fftw_plan_dft_r2c_2d, FFTW_ESTIMATE, forward sign -1, no
 * normalisation; reference src/galario.cpp:514-525), restated as plain C.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is part of the CPU oracle: it is used
 * by the tests, by __graft_entry__.smoke() and by the CPU-baseline leg of
 * bench.py, never by the GPU product path.
 *
 * Included twice by galario_oracle.c and by shim/fftw_shim.c, with
 *   REAL = double / float   and   SFX(name) = name##_d / name##_f.
 *
 * Algorithms (published, textbook):
 *  - power-of-two lengths: iterative radix-2 decimation-in-time
 *    (Cooley & Tukey 1965) after a bit-reversal permutation;
 *  - other lengths: direct DFT with twiddles indexed by (j*k mod n), so each
 *    twiddle is one correctly rounded table value;
 *  - real rows of power-of-two length n >= 4: the half-length complex FFT of
 *    z[m] = x[2m] + i x[2m+1] followed by the even/odd split
 *    X[k] = E[k] + exp(-2 pi i k/n) O[k]  (e.g. Press et al., Numerical
 *    Recipes 12.3).
 * Twiddles are evaluated in long double and rounded once to REAL, so the
 * transform agrees with numpy.fft to ~1e-16 relative (double).
 *
 * The 2D transform works in place on the FFTW padded layout: nx rows of
 * 2*(ny/2+1) REALs, the real input in the first ny slots of each row, the
 * complex output (nx x (ny/2+1), interleaved re/im) in the same memory.
 */

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef ORC_FFT_COMMON_DEFINED
#define ORC_FFT_COMMON_DEFINED
static int orc_is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
static const long double ORC_TWO_PI_L = 6.283185307179586476925286766559005768L;
#endif

/* tw[2k], tw[2k+1] = cos, sin of (-2 pi k / n), k in [0, count) */
static void SFX(orc_twiddles)(int n, int count, REAL *tw) {
    for (int k = 0; k < count; ++k) {
        long double a = -ORC_TWO_PI_L * (long double)k / (long double)n;
        tw[2 * k] = (REAL)cosl(a);
        tw[2 * k + 1] = (REAL)sinl(a);
    }
}

/* In-place forward complex FFT of power-of-two length n on interleaved data.
 * tw holds n/2 twiddles of exp(-2 pi i k / n). */
static void SFX(orc_fft_pow2)(int n, REAL *x, const REAL *tw) {
    /* bit reversal */
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            REAL tr = x[2 * i], ti = x[2 * i + 1];
            x[2 * i] = x[2 * j]; x[2 * i + 1] = x[2 * j + 1];
            x[2 * j] = tr; x[2 * j + 1] = ti;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1, step = n / len;
        for (int b = 0; b < n; b += len) {
            for (int j = 0; j < half; ++j) {
                REAL wr = tw[2 * j * step], wi = tw[2 * j * step + 1];
                REAL *p = x + 2 * (b + j), *q = x + 2 * (b + j + half);
                REAL tr = q[0] * wr - q[1] * wi;
                REAL ti = q[0] * wi + q[1] * wr;
                q[0] = p[0] - tr; q[1] = p[1] - ti;
                p[0] = p[0] + tr; p[1] = p[1] + ti;
            }
        }
    }
}

/* Direct forward DFT of any length n; tw holds n twiddles, tmp 2n REALs. */
static void SFX(orc_dft_direct)(int n, REAL *x, const REAL *tw, REAL *tmp) {
    for (int k = 0; k < n; ++k) {
        long double sr = 0.0L, si = 0.0L;
        for (int j = 0; j < n; ++j) {
            int idx = (int)(((long long)j * k) % n);
            long double wr = tw[2 * idx], wi = tw[2 * idx + 1];
            sr += x[2 * j] * wr - x[2 * j + 1] * wi;
            si += x[2 * j] * wi + x[2 * j + 1] * wr;
        }
        tmp[2 * k] = (REAL)sr;
        tmp[2 * k + 1] = (REAL)si;
    }
    memcpy(x, tmp, sizeof(REAL) * 2 * (size_t)n);
}

/* Forward complex transform of length n, any n >= 1. tw: twiddle table for n
 * (n/2 entries if pow2, n entries otherwise); tmp: 2n REALs scratch. */
static void SFX(orc_fft_any)(int n, REAL *x, const REAL *tw, REAL *tmp) {
    if (n <= 1) return;
    if (orc_is_pow2(n)) SFX(orc_fft_pow2)(n, x, tw);
    else SFX(orc_dft_direct)(n, x, tw, tmp);
}

static int SFX(orc_tw_count)(int n) { return orc_is_pow2(n) ? (n / 2 > 0 ? n / 2 : 1) : n; }

/* In-place 2D R2C on the FFTW padded layout (see the file header).
 * Returns 0, or 2 on allocation failure. */
static int SFX(orc_rfft2_inplace)(int nx, int ny, REAL *buf) {
    const int ncol = ny / 2 + 1;
    const size_t rs = 2 * (size_t)ncol; /* REALs per row */
    const int half = ny / 2;
    const int use_pack = orc_is_pow2(ny) && ny >= 4;
    const int nrow_fft = use_pack ? half : ny;

    REAL *tw_row = (REAL *)malloc(sizeof(REAL) * 2 * (size_t)SFX(orc_tw_count)(nrow_fft));
    REAL *tw_split = (REAL *)malloc(sizeof(REAL) * 2 * (size_t)(half + 1));
    REAL *tw_col = (REAL *)malloc(sizeof(REAL) * 2 * (size_t)SFX(orc_tw_count)(nx));
    if (!tw_row || !tw_split || !tw_col) { free(tw_row); free(tw_split); free(tw_col); return 2; }
    SFX(orc_twiddles)(nrow_fft, SFX(orc_tw_count)(nrow_fft), tw_row);
    SFX(orc_twiddles)(ny, half + 1, tw_split);
    SFX(orc_twiddles)(nx, SFX(orc_tw_count)(nx), tw_col);
    int failed = 0;

    /* ---- row pass: real rows of length ny -> ncol complex ---- */
#pragma omp parallel
    {
        REAL *z = (REAL *)malloc(sizeof(REAL) * 2 * (size_t)(ny + 2));
        REAL *tmp = (REAL *)malloc(sizeof(REAL) * 2 * (size_t)(ny + 2));
        if (!z || !tmp) {
#pragma omp atomic write
            failed = 1;
        } else {
#pragma omp for schedule(static)
            for (int i = 0; i < nx; ++i) {
                REAL *row = buf + (size_t)i * rs;
                if (use_pack) {
                    /* the first ny reals of the row are z[m] = x[2m] + i x[2m+1] */
                    memcpy(z, row, sizeof(REAL) * (size_t)ny);
                    SFX(orc_fft_pow2)(half, z, tw_row);
                    for (int k = 0; k <= half; ++k) {
                        int a = k % half, b = (half - k) % half;
                        REAL zr = z[2 * a], zi = z[2 * a + 1];
                        REAL cr = z[2 * b], ci = -z[2 * b + 1]; /* conj(Z[M-k]) */
                        REAL er = (REAL)0.5 * (zr + cr), ei = (REAL)0.5 * (zi + ci);
                        /* O = (Z - conj)/(2i) = (dz)/(2i): (p + iq)/(2i) = (q - ip)/2 */
                        REAL pr = zr - cr, pi = zi - ci;
                        REAL or_ = (REAL)0.5 * pi, oi = (REAL)-0.5 * pr;
                        REAL wr = tw_split[2 * k], wi = tw_split[2 * k + 1];
                        row[2 * k] = er + (or_ * wr - oi * wi);
                        row[2 * k + 1] = ei + (or_ * wi + oi * wr);
                    }
                } else {
                    for (int j = 0; j < ny; ++j) { z[2 * j] = row[j]; z[2 * j + 1] = 0; }
                    SFX(orc_fft_any)(ny, z, tw_row, tmp);
                    memcpy(row, z, sizeof(REAL) * 2 * (size_t)ncol);
                }
            }
        }
        free(z); free(tmp);
    }

    /* ---- column pass: ncol complex columns of length nx, 8 at a time ---- */
    const int CB = 8;
    const int nblk = (ncol + CB - 1) / CB;
#pragma omp parallel
    {
        REAL *col = (REAL *)malloc(sizeof(REAL) * 2 * (size_t)nx * CB);
        REAL *tmp = (REAL *)malloc(sizeof(REAL) * 2 * (size_t)nx);
        if (!col || !tmp) {
#pragma omp atomic write
            failed = 1;
        } else {
#pragma omp for schedule(dynamic, 1)
            for (int blk = 0; blk < nblk; ++blk) {
                int k0 = blk * CB, nk = ncol - k0 < CB ? ncol - k0 : CB;
                for (int i = 0; i < nx; ++i) {
                    const REAL *src = buf + (size_t)i * rs + 2 * (size_t)k0;
                    for (int c = 0; c < nk; ++c) {
                        col[2 * ((size_t)c * nx + i)] = src[2 * c];
                        col[2 * ((size_t)c * nx + i) + 1] = src[2 * c + 1];
                    }
                }
                for (int c = 0; c < nk; ++c) SFX(orc_fft_any)(nx, col + 2 * (size_t)c * nx, tw_col, tmp);
                for (int i = 0; i < nx; ++i) {
                    REAL *dst = buf + (size_t)i * rs + 2 * (size_t)k0;
                    for (int c = 0; c < nk; ++c) {
                        dst[2 * c] = col[2 * ((size_t)c * nx + i)];
                        dst[2 * c + 1] = col[2 * ((size_t)c * nx + i) + 1];
                    }
                }
            }
        }
        free(col); free(tmp);
    }
    free(tw_row); free(tw_split); free(tw_col);
    return failed ? 2 : 0;
}
