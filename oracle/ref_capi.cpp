/*
 * extern "C" forwarding layer over the reference's void* wrappers
 * (src/galario_py.h:30-46), compiled against the reference sources where
 * they lie, so ctypes can call the unmodified reference CPU path.  C++
 * exceptions become status codes the way Cython's `except +` maps them
 * (python/galario_defs.pxd:24-46): invalid_argument -> 1 (ValueError),
 * bad_alloc -> 2 (MemoryError), anything else -> 3 (RuntimeError).
 *
 * TEST INFRASTRUCTURE ONLY (builds oracle/_ref/).
 */
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include "galario.h"
#include "galario_py.h"

namespace {
thread_local std::string g_msg;
template <class F> int guarded(F &&f) {
    try {
        f();
        g_msg.clear();
        return 0;
    } catch (const std::invalid_argument &e) {
        g_msg = e.what();
        return 1;
    } catch (const std::bad_alloc &e) {
        g_msg = e.what();
        return 2;
    } catch (const std::exception &e) {
        g_msg = e.what();
        return 3;
    }
}
}  // namespace

#define API extern "C" __attribute__((visibility("default")))

API const char *ref_last_error() { return g_msg.c_str(); }
API int ref_threads(int num) { return galario::threads(num); }
API int ref_init() { return guarded([] { galario::init(); }); }

API int ref_sample_image(int nx, int ny, void *img, dreal v_origin, dreal dRA, dreal dDec, dreal duv, dreal PA, int nd,
                         void *u, void *v, void *vis) {
    return guarded([&] { galario::_sample_image(nx, ny, img, v_origin, dRA, dDec, duv, PA, nd, u, v, vis); });
}
API int ref_chi2_image(int nx, int ny, void *img, dreal v_origin, dreal dRA, dreal dDec, dreal duv, dreal PA, int nd,
                       void *u, void *v, void *re, void *im, void *w, dreal *chi2) {
    return guarded([&] { *chi2 = galario::_chi2_image(nx, ny, img, v_origin, dRA, dDec, duv, PA, nd, u, v, re, im, w); });
}
API int ref_sample_profile(int nr, void *I, dreal Rmin, dreal dR, dreal dxy, int nxy, dreal inc, dreal dRA, dreal dDec,
                           dreal duv, dreal PA, int nd, void *u, void *v, void *vis) {
    return guarded([&] { galario::_sample_profile(nr, I, Rmin, dR, dxy, nxy, inc, dRA, dDec, duv, PA, nd, u, v, vis); });
}
API int ref_chi2_profile(int nr, void *I, dreal Rmin, dreal dR, dreal dxy, int nxy, dreal inc, dreal dRA, dreal dDec,
                         dreal duv, dreal PA, int nd, void *u, void *v, void *re, void *im, void *w, dreal *chi2) {
    return guarded([&] {
        *chi2 = galario::_chi2_profile(nr, I, Rmin, dR, dxy, nxy, inc, dRA, dDec, duv, PA, nd, u, v, re, im, w);
    });
}
API int ref_sweep(int nr, void *I, dreal Rmin, dreal dR, int nxy, dreal dxy, dreal inc, void *image) {
    return guarded([&] { galario::_sweep(nr, I, Rmin, dR, nxy, dxy, inc, image); });
}
API int ref_uv_rotate(dreal PA, dreal dRA, dreal dDec, void *dRArot, void *dDecrot, int nd, void *u, void *v,
                      void *urot, void *vrot) {
    return guarded([&] { galario::_uv_rotate(PA, dRA, dDec, dRArot, dDecrot, nd, u, v, urot, vrot); });
}
API int ref_interpolate(int nrow, int ncol, void *data, dreal v_origin, int nd, void *u, void *v, dreal duv,
                        void *vis) {
    return guarded([&] { galario::_interpolate(nrow, ncol, data, v_origin, nd, u, v, duv, vis); });
}
API int ref_apply_phase(dreal dRA, dreal dDec, int nd, void *u, void *v, void *vis) {
    return guarded([&] { galario::_apply_phase_sampled(dRA, dDec, nd, u, v, vis); });
}
API int ref_reduce_chi2(int nd, void *re, void *im, void *vis, void *w, dreal *chi2) {
    return guarded([&] { *chi2 = galario::_reduce_chi2(nd, re, im, vis, w); });
}
/* _copy_input + _fft2d: padded in-place R2C; the result buffer is copied out
 * so the caller owns plain memory (nx * (ny/2+1) complex). */
API int ref_fft2d(int nx, int ny, void *img, void *out) {
    return guarded([&] {
        void *buf = galario::_copy_input(nx, ny, img);
        try {
            galario::_fft2d(nx, ny, buf);
        } catch (...) {
            galario::galario_free(buf);
            throw;
        }
        std::memcpy(out, buf, sizeof(dcomplex) * (size_t)nx * (ny / 2 + 1));
        galario::galario_free(buf);
    });
}
API int ref_fftshift(int nx, int ny, void *img, void *out) {
    return guarded([&] {
        void *buf = galario::_copy_input(nx, ny, img);
        galario::_fftshift(nx, ny, buf);
        std::memcpy(out, buf, sizeof(dcomplex) * (size_t)nx * (ny / 2 + 1));
        galario::galario_free(buf);
    });
}
API int ref_fftshift_axis0(int nrow, int ncol, void *data) {
    return guarded([&] { galario::_fftshift_axis0(nrow, ncol, data); });
}
