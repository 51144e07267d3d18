/*
 * galario_gb300.hpp -- C++ functional API of galario (reference
 * src/galario.h:24-59) as a header-only facade over the C ABI in
 * galario_gb300.h.
 *
 * Same namespace, function names, argument order and meaning as the
 * reference, so that a C++ program written against galario.h compiles
 * against this header and links against libgalario_gb300.so:
 *  - precision: define GALARIO_DOUBLE_PRECISION (the reference's
 *    DOUBLE_PRECISION, src/galario_defs.h:28-46) for dreal = double, else
 *    dreal = float; dcomplex = std::complex<dreal> (the reference's CPU build);
 *  - errors: a failed call throws what the reference throws --
 *    std::invalid_argument, std::bad_alloc or std::runtime_error -- with the
 *    library's message (src/galario.cpp:101-121);
 *  - every array is host memory; the library copies to the current GPU.
 */
#ifndef GALARIO_GB300_HPP
#define GALARIO_GB300_HPP

#include <complex>
#include <cstdlib>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>

#include "galario_gb300.h"

namespace galario {

#if defined(GALARIO_DOUBLE_PRECISION) || defined(DOUBLE_PRECISION)
typedef double dreal;
#define GALARIO_GB300_FN(name) galario_##name##_d
#else
typedef float dreal;
#define GALARIO_GB300_FN(name) galario_##name##_f
#endif
typedef std::complex<dreal> dcomplex;

namespace detail {
inline void check(int status) {
    if (status == GALARIO_OK) return;
    const char* m = galario_last_error();
    const std::string msg = m ? m : "galario_gb300 error";
    if (status == GALARIO_EINVAL) throw std::invalid_argument(msg);
    if (status == GALARIO_ENOMEM) throw std::bad_alloc();
    throw std::runtime_error(msg);
}
inline dreal* re(dcomplex* p) { return reinterpret_cast<dreal*>(p); }
inline const dreal* re(const dcomplex* p) { return reinterpret_cast<const dreal*>(p); }
}  // namespace detail

/* Main user functions (reference src/galario.h:27-36) */
inline void sample_profile(int nr, const dreal* intensity, dreal Rmin, dreal dR, dreal dxy, int nxy, dreal inc,
                           dreal dRA, dreal dDec, dreal duv, dreal PA, int nd, const dreal* u, const dreal* v,
                           dcomplex* vis_int) {
    detail::check(GALARIO_GB300_FN(sample_profile)(nr, intensity, Rmin, dR, dxy, nxy, inc, dRA, dDec, duv, PA, nd, u,
                                                   v, detail::re(vis_int)));
}
inline void sample_image(int nx, int ny, const dreal* image, const dreal v_origin, dreal dRA, dreal dDec, dreal duv,
                         dreal PA, int nd, const dreal* u, const dreal* v, dcomplex* vis_int) {
    detail::check(GALARIO_GB300_FN(sample_image)(nx, ny, image, v_origin, dRA, dDec, duv, PA, nd, u, v,
                                                 detail::re(vis_int)));
}
inline dreal chi2_profile(int nr, const dreal* intensity, dreal Rmin, dreal dR, dreal dxy, int nxy, dreal inc,
                          dreal dRA, dreal dDec, dreal duv, dreal PA, int nd, const dreal* u, const dreal* v,
                          const dreal* vis_obs_re, const dreal* vis_obs_im, const dreal* weights) {
    dreal chi2 = 0;
    detail::check(GALARIO_GB300_FN(chi2_profile)(nr, intensity, Rmin, dR, dxy, nxy, inc, dRA, dDec, duv, PA, nd, u, v,
                                                 vis_obs_re, vis_obs_im, weights, &chi2));
    return chi2;
}
inline dreal chi2_image(int nx, int ny, const dreal* image, const dreal v_origin, dreal dRA, dreal dDec, dreal duv,
                        dreal PA, int nd, const dreal* u, const dreal* v, const dreal* vis_obs_re,
                        const dreal* vis_obs_im, const dreal* weights) {
    dreal chi2 = 0;
    detail::check(GALARIO_GB300_FN(chi2_image)(nx, ny, image, v_origin, dRA, dDec, duv, PA, nd, u, v, vis_obs_re,
                                               vis_obs_im, weights, &chi2));
    return chi2;
}
/* image: the padded real-to-complex buffer of nxy x (nxy/2+1) complex */
inline void sweep(int nr, const dreal* intensity, dreal Rmin, dreal dR, int nxy, dreal dxy, dreal inc,
                  dcomplex* image) {
    detail::check(GALARIO_GB300_FN(sweep)(nr, intensity, Rmin, dR, nxy, dxy, inc, detail::re(image)));
}
inline void uv_rotate(dreal PA, dreal dRA, dreal dDec, dreal* dRArot, dreal* dDecrot, int nd, const dreal* u,
                      const dreal* v, dreal* urot, dreal* vrot) {
    detail::check(GALARIO_GB300_FN(uv_rotate)(PA, dRA, dDec, dRArot, dDecrot, nd, u, v, urot, vrot));
}

/* Interface for the experts (reference src/galario.h:39-51) */

/* nx x ny real image -> newly allocated padded buffer of nx x (ny/2+1)
 * complex (row i starts at complex i*(ny/2+1)); free with galario_free */
inline dcomplex* copy_input(int nx, int ny, const dreal* image) {
    if (nx < 2 || ny < 2 || (nx & 1) || (ny & 1))
        throw std::invalid_argument("Error in copy_input: nx, ny must be even and at least 2");
    const size_t ncol = (size_t)ny / 2 + 1;
    void* p = std::malloc(sizeof(dcomplex) * ncol * (size_t)nx);
    if (!p) throw std::bad_alloc();
    dreal* out = static_cast<dreal*>(p);
    for (int i = 0; i < nx; ++i) {
        std::memcpy(out + (size_t)i * 2 * ncol, image + (size_t)i * ny, sizeof(dreal) * (size_t)ny);
        out[(size_t)i * 2 * ncol + ny] = 0;
        out[(size_t)i * 2 * ncol + ny + 1] = 0;
    }
    return static_cast<dcomplex*>(p);
}
inline void galario_free(void* p) { std::free(p); }
inline void fft2d(int nx, int ny, dcomplex* image) { detail::check(GALARIO_GB300_FN(fft2d)(nx, ny, detail::re(image))); }
inline void fftshift(int nx, int ny, dcomplex* image) {
    detail::check(GALARIO_GB300_FN(fftshift)(nx, ny, detail::re(image)));
}
inline void fftshift_axis0(int nx, int ny, dcomplex* matrix) {
    detail::check(GALARIO_GB300_FN(fftshift_axis0)(nx, ny, detail::re(matrix)));
}
inline void interpolate(int nrow, int ncol, const dcomplex* image, const dreal v_origin, int nd, const dreal* u,
                        const dreal* v, const dreal duv, dcomplex* vis_int) {
    detail::check(GALARIO_GB300_FN(interpolate)(nrow, ncol, detail::re(image), v_origin, nd, u, v, duv,
                                                detail::re(vis_int)));
}
inline void apply_phase_sampled(dreal dRA, dreal dDec, int nd, const dreal* u, const dreal* v, dcomplex* vis_int) {
    detail::check(GALARIO_GB300_FN(apply_phase_sampled)(dRA, dDec, nd, u, v, detail::re(vis_int)));
}
inline dreal reduce_chi2(int nd, const dreal* vis_obs_re, const dreal* vis_obs_im, const dcomplex* vis_int,
                         const dreal* weights) {
    dreal chi2 = 0;
    detail::check(GALARIO_GB300_FN(reduce_chi2)(nd, vis_obs_re, vis_obs_im, detail::re(vis_int), weights, &chi2));
    return chi2;
}

/* Required for multithreading (reference src/galario.h:54-56) */
inline void init() { detail::check(galario_init()); }
inline void cleanup() { detail::check(galario_cleanup()); }
inline int threads(int num = 0) { return galario_threads(num); }

/* GPU related functions (reference src/galario.h:58-60) */
inline int ngpus() {
    int n = 0;
    detail::check(galario_ngpus(&n));
    return n;
}
inline void use_gpu(int device_id) { detail::check(galario_use_gpu(device_id)); }

}  // namespace galario

#undef GALARIO_GB300_FN
#endif /* GALARIO_GB300_HPP */
