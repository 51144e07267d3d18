/*
 * Oracle restatement of galario's CPU back end (reference: src/galario.cpp,
 * galario v1.2.2), one function per reference stage, in plain C with OpenMP.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU product path and the
 * CPU baseline timed beside it.  Nothing in galario_gb300/ calls this code.
 *
 * Included twice by galario_oracle.c with REAL = double / float and
 * SFX(name) = name##_d / name##_f.  Complex arrays are interleaved (re, im)
 * REAL pairs, the memory layout of std::complex<REAL>.  The arithmetic
 * follows the reference's operation order so that the double build agrees
 * with the reference to rounding.
 */

/* ---------------------------------------------------------------------- */
/* fftshift of a real nx x ny image stored in the padded R2C buffer        */
/* reference: shift_core src/galario.cpp:565-589, shift_h :615-623         */
/* ---------------------------------------------------------------------- */
static void SFX(orc_shift)(int nx, int ny, REAL *a) {
    const size_t rowsize = 2 * (size_t)(ny / 2 + 1);
#pragma omp parallel for
    for (int x = 0; x < nx / 2; ++x) {
        for (int y = 0; y < ny / 2; ++y) {
            size_t src_ul = (size_t)x * rowsize + y;
            size_t src_ur = src_ul + ny / 2;
            size_t tgt_ul = src_ur + (size_t)(nx / 2) * rowsize;
            size_t tgt_ur = tgt_ul - ny / 2;
            REAL t = a[src_ul]; a[src_ul] = a[tgt_ul]; a[tgt_ul] = t;
            t = a[src_ur]; a[src_ur] = a[tgt_ur]; a[tgt_ur] = t;
        }
    }
}

/* swap upper and lower halves of an nrow x ncol complex matrix            */
/* reference: shift_axis0_core src/galario.cpp:657-668, shift_axis0_h :691-698 */
static void SFX(orc_shift_axis0)(int nrow, int ncol, REAL *m) {
#pragma omp parallel for
    for (int x = 0; x < nrow / 2; ++x) {
        for (int y = 0; y < ncol; ++y) {
            size_t s = 2 * ((size_t)x * ncol + y);
            size_t t = s + 2 * (size_t)(nrow / 2) * ncol;
            REAL r = m[s], i = m[s + 1];
            m[s] = m[t]; m[s + 1] = m[t + 1];
            m[t] = r; m[t + 1] = i;
        }
    }
}

/* pad a real nx x ny image into the R2C in-place layout                    */
/* reference: copy_input src/galario.cpp:460-487                           */
static REAL *SFX(orc_copy_input)(int nx, int ny, const REAL *img) {
    const size_t rowsize = 2 * (size_t)(ny / 2 + 1);
    REAL *buf = (REAL *)calloc((size_t)nx * rowsize, sizeof(REAL));
    if (!buf) return NULL;
#pragma omp parallel for
    for (int i = 0; i < nx; ++i) memcpy(buf + (size_t)i * rowsize, img + (size_t)i * ny, sizeof(REAL) * (size_t)ny);
    return buf;
}

/* ---------------------------------------------------------------------- */
/* bilinear amplitude/phase interpolation on the half-plane spectrum       */
/* reference: interpolate_core src/galario.cpp:749-815, interpolate_h :832-838 */
/* ---------------------------------------------------------------------- */
static void SFX(orc_interpolate)(int nrow, int ncol, const REAL *data, REAL v_origin, int nd,
                                 const REAL *u, const REAL *v, REAL duv, REAL *vis) {
#pragma omp parallel for
    for (int idx = 0; idx < nd; ++idx) {
        const int half_nrow = nrow / 2;
        REAL indu = (REAL)fabs(u[idx]) / duv;
        REAL sign_u = (REAL)copysign(1., u[idx]);
        REAL indv = half_nrow + v_origin * sign_u * v[idx] / duv;
        int fl_u = (int)floor(indu);
        int fl_v = (int)floor(indv);
        REAL t = indv - fl_v;
        REAL q = indu - fl_u;
        long base = (long)fl_u + (long)fl_v * ncol;
        const REAL *y0 = data + 2 * base;
        const REAL *y1 = data + 2 * (base + ncol);
        const REAL *y2 = data + 2 * (base + ncol + 1);
        const REAL *y3 = data + 2 * (base + 1);
        /* t*q*(y0 - y1 + y2 - y3) + t*(y1 - y0) + q*(y3 - y0) + y0, as complex */
        REAL df1r = (y0[0] + y2[0]) - (y1[0] + y3[0]);
        REAL df1i = (y0[1] + y2[1]) - (y1[1] + y3[1]);
        REAL term1r = t * (q * df1r), term1i = t * (q * df1i);
        REAL term2r = t * (y1[0] - y0[0]), term2i = t * (y1[1] - y0[1]);
        REAL term3r = q * (y3[0] - y0[0]), term3i = q * (y3[1] - y0[1]);
        REAL fr = term1r + (term2r + term3r), fi = term1i + (term2i + term3i);
        REAL zr = fr + y0[0], zi = fi + y0[1];
        REAL interp_phase = (REAL)atan2(zi, zr) * sign_u;
        REAL y0r = (REAL)hypot(y0[0], y0[1]);
        REAL y1r = (REAL)hypot(y1[0], y1[1]);
        REAL y2r = (REAL)hypot(y2[0], y2[1]);
        REAL y3r = (REAL)hypot(y3[0], y3[1]);
        REAL amp = y0r;
        amp += (y3r - y0r) * q;
        amp += (y1r - y0r) * t;
        amp += (y0r - y1r + y2r - y3r) * t * q;
        vis[2 * idx] = amp * (REAL)cos(interp_phase);
        vis[2 * idx + 1] = amp * (REAL)sin(interp_phase);
    }
}

/* phase shift of the sampled visibilities                                  */
/* reference: apply_phase_sampled_core :877-884, apply_phase_sampled_h :908-921 */
static void SFX(orc_apply_phase)(REAL dRA, REAL dDec, int nd, const REAL *u, const REAL *v, REAL *vis) {
    if (dRA == 0 && dDec == 0) return;
    dRA *= (REAL)(2. * (REAL)M_PI);
    dDec *= (REAL)(2. * (REAL)M_PI);
#pragma omp parallel for schedule(static)
    for (int x = 0; x < nd; ++x) {
        REAL angle = u[x] * dRA + v[x] * dDec;
        REAL c = (REAL)cos(angle), s = (REAL)sin(angle);
        REAL a = vis[2 * x], b = vis[2 * x + 1];
        vis[2 * x] = a * c - b * s;
        vis[2 * x + 1] = a * s + b * c;
    }
}

/* rotation of (u, v) and of (dRA, dDec) by PA                              */
/* reference: uv_rotate_core :955-960, uv_rotate_h :976-999                 */
static void SFX(orc_uv_rotate)(REAL PA, REAL dRA, REAL dDec, REAL *dRArot, REAL *dDecrot, int nd,
                               const REAL *u, const REAL *v, REAL *urot, REAL *vrot) {
    if (PA == 0) {
        *dRArot = dRA; *dDecrot = dDec;
        memcpy(urot, u, sizeof(REAL) * (size_t)nd);
        memcpy(vrot, v, sizeof(REAL) * (size_t)nd);
        return;
    }
    const REAL c = (REAL)cos(PA), s = (REAL)sin(PA);
#pragma omp parallel for
    for (int i = 0; i < nd; ++i) {
        urot[i] = u[i] * c - v[i] * s;
        vrot[i] = u[i] * s + v[i] * c;
    }
    *dRArot = dRA * c - dDec * s;
    *dDecrot = dRA * s + dDec * c;
}

/* ---------------------------------------------------------------------- */
/* radial profile -> image (sweep + central pixel)                          */
/* reference: sweep_core :1048-1071, create_image_h :1186-1235               */
/* ---------------------------------------------------------------------- */
static int SFX(orc_create_image)(int nr, const REAL *I, REAL Rmin, REAL dR, int nxy, REAL dxy, REAL inc, REAL *image) {
    REAL ratio = (dxy / (REAL)2. - Rmin) / dR;
    if (ratio < 5) {
        snprintf(orc_errbuf, sizeof orc_errbuf,
                 "Error in create image: Expect (dxy/2-Rmin)/dR > 5, i.e. dR small enough to ensure reliable "
                 "interpolation the inside central pixel but got (dxy/2-Rmin)/dR = %f. Try reducing dR.", (double)ratio);
        return ORC_EINVAL;
    }
    const int ncol = nxy / 2 + 1;
    const size_t rowsize = 2 * (size_t)ncol;
    memset(image, 0, sizeof(REAL) * rowsize * (size_t)nxy);
    const REAL cos_inc = (REAL)cos(inc);
    int rmax = (int)ceil((Rmin + nr * dR) / dxy);
    if (rmax > nxy / 2) rmax = nxy / 2;
    const REAL sr_to_px = dxy * dxy;
    const int off = nxy / 2 - rmax;
#pragma omp parallel for
    for (int i = 0; i < 2 * rmax; ++i) {
        for (int j = 0; j < 2 * rmax; ++j) {
            REAL x = (rmax - j) * dxy;
            REAL y = (rmax - i) * dxy;
            REAL r = (REAL)sqrt(pow(x / cos_inc, 2) + pow(y, 2));
            int iR = (int)floor((r - Rmin) / dR);
            if (iR < 0) iR = 0;
            size_t base = (size_t)(i + off) * rowsize + (size_t)(j + off);
            if (iR > nr - 2) image[base] = 0;
            else image[base] = sr_to_px * (I[iR] + (r - iR * dR - Rmin) * (I[iR + 1] - I[iR]) / dR);
        }
    }
    /* central pixel: trapezoid-rule mean intensity inside dxy/2 (reference :1209-1232) */
    const int iIN = (int)floor((dxy / 2 - Rmin) / dR);
    REAL flux = 0;
    for (int i = 1; i < iIN; ++i) flux += (Rmin + dR * i) * I[i];
    flux *= 2;
    flux += Rmin * I[0] + (Rmin + iIN * dR) * I[iIN];
    flux *= dR;
    REAL I_interp = (I[iIN + 1] - I[iIN]) / dR * (dxy / (REAL)2. - (Rmin + dR * iIN)) + I[iIN];
    flux += ((Rmin + iIN * dR) * I[iIN] + dxy / (REAL)2. * I_interp) * (dxy / (REAL)2. - (Rmin + iIN * dR));
    REAL area = (REAL)(pow(dxy / 2., 2) - pow(Rmin, 2));
    image[(size_t)(nxy / 2) * rowsize + nxy / 2] = sr_to_px * flux / area;
    return 0;
}

/* ---------------------------------------------------------------------- */
/* chi2 reduction (accumulated in REAL, as the reference CPU path does)     */
/* reference: diff_weighted_core :1453-1461, reduce_chi2 CPU :1519-1529     */
/* ---------------------------------------------------------------------- */
static REAL SFX(orc_reduce)(int nd, const REAL *re, const REAL *im, const REAL *vis, const REAL *w) {
    REAL chi2 = 0;
#pragma omp parallel for reduction(+ : chi2)
    for (int i = 0; i < nd; ++i) {
        REAL sw = (REAL)sqrt(w[i]);
        REAL a = (vis[2 * i] - re[i]) * sw;
        REAL b = (vis[2 * i + 1] - im[i]) * sw;
        chi2 += a * a + b * b;
    }
    return chi2;
}

/* ---------------------------------------------------------------------- */
/* stage orchestration: shift -> FFT -> shift_axis0 -> rotate -> interp -> phase */
/* reference: sample_h :1324-1350                                           */
/* ---------------------------------------------------------------------- */
static int SFX(orc_sample_buffer)(int nx, int ny, REAL *data, REAL v_origin, REAL dRA, REAL dDec, int nd, REAL duv,
                                  REAL PA, const REAL *u, const REAL *v, REAL *vis) {
    const int ncol = ny / 2 + 1;
    SFX(orc_shift)(nx, ny, data);
    if (SFX(orc_rfft2_inplace)(nx, ny, data)) return orc_oom();
    SFX(orc_shift_axis0)(nx, ncol, data);
    REAL *urot = (REAL *)malloc(sizeof(REAL) * (size_t)(nd > 0 ? nd : 1));
    REAL *vrot = (REAL *)malloc(sizeof(REAL) * (size_t)(nd > 0 ? nd : 1));
    if (!urot || !vrot) { free(urot); free(vrot); return orc_oom(); }
    REAL dRArot, dDecrot;
    SFX(orc_uv_rotate)(PA, dRA, dDec, &dRArot, &dDecrot, nd, u, v, urot, vrot);
    SFX(orc_interpolate)(nx, ncol, data, v_origin, nd, urot, vrot, duv, vis);
    SFX(orc_apply_phase)(dRArot, dDecrot, nd, urot, vrot, vis);
    free(urot); free(vrot);
    return 0;
}

/* ======================= exported entry points ========================= */
/* Mirrors of the reference's void* wrappers (src/galario_py.h:30-46).      */

ORC_API int SFX(orc_sample_image)(int nx, int ny, const REAL *img, REAL v_origin, REAL dRA, REAL dDec, REAL duv,
                                  REAL PA, int nd, const REAL *u, const REAL *v, REAL *vis) {
    orc_errbuf[0] = 0;
    if (orc_check_input(nx)) return ORC_EINVAL; /* reference :1364 checks nx only */
    REAL *data = SFX(orc_copy_input)(nx, ny, img);
    if (!data) return orc_oom();
    int st = SFX(orc_sample_buffer)(nx, ny, data, v_origin, dRA, dDec, nd, duv, PA, u, v, vis);
    free(data);
    return st;
}

ORC_API int SFX(orc_sample_profile)(int nr, const REAL *I, REAL Rmin, REAL dR, REAL dxy, int nxy, REAL inc, REAL dRA,
                                    REAL dDec, REAL duv, REAL PA, int nd, const REAL *u, const REAL *v, REAL *vis) {
    orc_errbuf[0] = 0;
    if (orc_check_input(nxy)) return ORC_EINVAL;
    const size_t nb = (size_t)nxy * 2 * (size_t)(nxy / 2 + 1);
    REAL *data = (REAL *)malloc(sizeof(REAL) * nb);
    if (!data) return orc_oom();
    int st = SFX(orc_create_image)(nr, I, Rmin, dR, nxy, dxy, inc, data);
    if (!st) st = SFX(orc_sample_buffer)(nxy, nxy, data, (REAL)1, dRA, dDec, nd, duv, PA, u, v, vis);
    free(data);
    return st;
}

ORC_API int SFX(orc_chi2_image)(int nx, int ny, const REAL *img, REAL v_origin, REAL dRA, REAL dDec, REAL duv,
                                REAL PA, int nd, const REAL *u, const REAL *v, const REAL *re, const REAL *im,
                                const REAL *w, REAL *chi2) {
    orc_errbuf[0] = 0;
    if (orc_check_square(nx, ny)) return ORC_EINVAL;
    REAL *vis = (REAL *)malloc(sizeof(REAL) * 2 * (size_t)(nd > 0 ? nd : 1));
    if (!vis) return orc_oom();
    int st = SFX(orc_sample_image)(nx, ny, img, v_origin, dRA, dDec, duv, PA, nd, u, v, vis);
    if (!st) *chi2 = SFX(orc_reduce)(nd, re, im, vis, w);
    free(vis);
    return st;
}

ORC_API int SFX(orc_chi2_profile)(int nr, const REAL *I, REAL Rmin, REAL dR, REAL dxy, int nxy, REAL inc, REAL dRA,
                                  REAL dDec, REAL duv, REAL PA, int nd, const REAL *u, const REAL *v, const REAL *re,
                                  const REAL *im, const REAL *w, REAL *chi2) {
    orc_errbuf[0] = 0;
    if (orc_check_input(nxy)) return ORC_EINVAL;
    REAL *vis = (REAL *)malloc(sizeof(REAL) * 2 * (size_t)(nd > 0 ? nd : 1));
    if (!vis) return orc_oom();
    int st = SFX(orc_sample_profile)(nr, I, Rmin, dR, dxy, nxy, inc, dRA, dDec, duv, PA, nd, u, v, vis);
    if (!st) *chi2 = SFX(orc_reduce)(nd, re, im, vis, w);
    free(vis);
    return st;
}

/* sweep into a padded complex buffer (reference: sweep :1240-1250) */
ORC_API int SFX(orc_sweep)(int nr, const REAL *I, REAL Rmin, REAL dR, int nxy, REAL dxy, REAL inc, REAL *image) {
    orc_errbuf[0] = 0;
    if (orc_check_input(nxy)) return ORC_EINVAL;
    return SFX(orc_create_image)(nr, I, Rmin, dR, nxy, dxy, inc, image);
}

ORC_API int SFX(orc_uv_rotate_api)(REAL PA, REAL dRA, REAL dDec, REAL *dRArot, REAL *dDecrot, int nd, const REAL *u,
                                   const REAL *v, REAL *urot, REAL *vrot) {
    orc_errbuf[0] = 0;
    SFX(orc_uv_rotate)(PA, dRA, dDec, dRArot, dDecrot, nd, u, v, urot, vrot);
    return 0;
}

ORC_API int SFX(orc_interpolate_api)(int nrow, int ncol, const REAL *data, REAL v_origin, int nd, const REAL *u,
                                     const REAL *v, REAL duv, REAL *vis) {
    orc_errbuf[0] = 0;
    SFX(orc_interpolate)(nrow, ncol, data, v_origin, nd, u, v, duv, vis);
    return 0;
}

ORC_API int SFX(orc_apply_phase_api)(REAL dRA, REAL dDec, int nd, const REAL *u, const REAL *v, REAL *vis) {
    orc_errbuf[0] = 0;
    SFX(orc_apply_phase)(dRA, dDec, nd, u, v, vis);
    return 0;
}

ORC_API int SFX(orc_reduce_chi2)(int nd, const REAL *re, const REAL *im, const REAL *vis, const REAL *w, REAL *chi2) {
    orc_errbuf[0] = 0;
    *chi2 = SFX(orc_reduce)(nd, re, im, vis, w);
    return 0;
}

/* padded in-place R2C of an nx x ny image, output nx x (ny/2+1) complex */
ORC_API int SFX(orc_fft2d)(int nx, int ny, REAL *data) {
    orc_errbuf[0] = 0;
    if (orc_check_square(nx, ny)) return ORC_EINVAL;
    if (SFX(orc_rfft2_inplace)(nx, ny, data)) return orc_oom();
    return 0;
}

ORC_API int SFX(orc_fftshift)(int nx, int ny, REAL *data) {
    orc_errbuf[0] = 0;
    if (orc_check_square(nx, ny)) return ORC_EINVAL;
    SFX(orc_shift)(nx, ny, data);
    return 0;
}

ORC_API int SFX(orc_fftshift_axis0)(int nrow, int ncol, REAL *data) {
    orc_errbuf[0] = 0;
    if (orc_check_input(nrow)) return ORC_EINVAL;
    SFX(orc_shift_axis0)(nrow, ncol, data);
    return 0;
}
