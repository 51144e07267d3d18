/*
 * galario_gb300 -- C ABI of the GB300 (sm_103a) implementation of galario's
 * synthetic-visibility and chi-squared path.
 *
 * Library: galario_gb300/_lib/libgalario_gb300.so (built by
 * __graft_entry__.build()).  Plain pointers and sizes only; no C++ or torch
 * types cross this boundary.
 *
 * Conventions shared by every entry point
 *  - Return value: GALARIO_OK (0) or an error status; the message for the
 *    calling thread is in galario_last_error().  The statuses correspond to
 *    the exceptions the reference throws (src/galario.cpp:89-198) and the
 *    Python exceptions Cython turns them into (python/galario_defs.pxd:24-46):
 *      GALARIO_EINVAL   std::invalid_argument -> ValueError
 *      GALARIO_ENOMEM   std::bad_alloc        -> MemoryError
 *      GALARIO_ERUNTIME std::runtime_error    -> RuntimeError
 *  - Suffix _d: every array and scalar is double (galario.double);
 *    suffix _f: float (galario.single), as the reference's `dreal`
 *    (src/galario_defs.h:28-46).
 *  - Complex arrays are interleaved (re, im) pairs, the layout of
 *    std::complex / numpy complex.
 *  - Units as in the reference: dxy, Rmin, dR, inc, PA, dRA, dDec in radians;
 *    u, v, duv in wavelengths; image in Jy/pixel; intensity in Jy/sr.
 *  - Host-pointer entry points copy their inputs to the current CUDA device
 *    (galario_use_gpu), run there and return when the results are back in
 *    host memory.  They are thread safe (one lock per device).
 *
 * Deviations from the reference, by design:
 *  - a (u, v) point whose bilinear corners fall outside the N x (N/2+1)
 *    spectrum returns GALARIO_EINVAL (the reference reads out of bounds);
 *  - sample_image rejects a non-square image with GALARIO_EINVAL (the
 *    reference passes ny = nx and misreads it, python/libcommon.pyx:441);
 *  - the profile entry points return GALARIO_EINVAL when the profile does
 *    not reach the edge of the central pixel (the reference reads past it).
 */
#ifndef GALARIO_GB300_H
#define GALARIO_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define GALARIO_OK 0
#define GALARIO_EINVAL 1
#define GALARIO_ENOMEM 2
#define GALARIO_ERUNTIME 3

/* Message of the last failed call on this thread. */
const char *galario_last_error(void);
const char *galario_version(void);

/* ---- runtime (reference src/galario.h:51-58, src/galario.cpp:366-428,1540-1554) ---- */
/* threads(num): replaces galario::threads (src/galario.cpp:367-390).  The value is
 * stored and returned for API compatibility; launch shapes are chosen by the library. */
int galario_threads(int num);
/* replaces galario::ngpus (src/galario.cpp:1540-1547) */
int galario_ngpus(int *count);
/* replaces galario::use_gpu (src/galario.cpp:1549-1554): cudaSetDevice for this thread */
int galario_use_gpu(int device_id);
/* replaces galario::init / galario::cleanup (src/galario.cpp:392-428) */
int galario_init(void);
int galario_cleanup(void);

/* ---- the four user functions ---- */

/* replaces galario::_sample_image (src/galario_py.h:31, src/galario.cpp:1359-1398).
 * image: nx*ny reals, row-major; u, v: nd; vis: 2*nd (output). */
int galario_sample_image_d(int nx, int ny, const double *image, double v_origin, double dRA, double dDec, double duv,
                           double PA, int nd, const double *u, const double *v, double *vis);
int galario_sample_image_f(int nx, int ny, const float *image, float v_origin, float dRA, float dDec, float duv,
                           float PA, int nd, const float *u, const float *v, float *vis);

/* replaces galario::_chi2_image (src/galario_py.h:34, src/galario.cpp:1556-1613).
 * chi2 = sum_k w_k |V_k - (re_k + i im_k)|^2, accumulated in double. */
int galario_chi2_image_d(int nx, int ny, const double *image, double v_origin, double dRA, double dDec, double duv,
                         double PA, int nd, const double *u, const double *v, const double *re, const double *im,
                         const double *w, double *chi2);
int galario_chi2_image_f(int nx, int ny, const float *image, float v_origin, float dRA, float dDec, float duv,
                         float PA, int nd, const float *u, const float *v, const float *re, const float *im,
                         const float *w, float *chi2);

/* replaces galario::_sample_profile (src/galario_py.h:29-30, src/galario.cpp:1404-1441).
 * intensity: nr samples on R = Rmin + i*dR; the image has origin 'upper'. */
int galario_sample_profile_d(int nr, const double *intensity, double Rmin, double dR, double dxy, int nxy, double inc,
                             double dRA, double dDec, double duv, double PA, int nd, const double *u, const double *v,
                             double *vis);
int galario_sample_profile_f(int nr, const float *intensity, float Rmin, float dR, float dxy, int nxy, float inc,
                             float dRA, float dDec, float duv, float PA, int nd, const float *u, const float *v,
                             float *vis);

/* replaces galario::_chi2_profile (src/galario_py.h:32-33, src/galario.cpp:1615-1664) */
int galario_chi2_profile_d(int nr, const double *intensity, double Rmin, double dR, double dxy, int nxy, double inc,
                           double dRA, double dDec, double duv, double PA, int nd, const double *u, const double *v,
                           const double *re, const double *im, const double *w, double *chi2);
int galario_chi2_profile_f(int nr, const float *intensity, float Rmin, float dR, float dxy, int nxy, float inc,
                           float dRA, float dDec, float duv, float PA, int nd, const float *u, const float *v,
                           const float *re, const float *im, const float *w, float *chi2);

/* ---- device-resident variants (no reference counterpart: the reference
 * re-uploads every input on every call, src/galario.cpp:1279-1280,1584-1589).
 * All *_dev pointers are device pointers; intensity_host is the same profile
 * in host memory (the central pixel is integrated on the host, as in the
 * reference :1136-1153).  The call only enqueues work on `stream` (a
 * cudaStream_t; NULL is CUDA's default stream) and writes chi2 as a double
 * to chi2_dev; galario_device_status() synchronises and reports device-side
 * errors.  Calls on one device share a workspace: issue them on one stream. */
int galario_chi2_profile_device_d(int nr, const double *intensity_host, const double *intensity_dev, double Rmin,
                                  double dR, double dxy, int nxy, double inc, double dRA, double dDec, double duv,
                                  double PA, int nd, const double *u_dev, const double *v_dev, const double *re_dev,
                                  const double *im_dev, const double *w_dev, double *chi2_dev, void *stream);
int galario_chi2_profile_device_f(int nr, const float *intensity_host, const float *intensity_dev, float Rmin,
                                  float dR, float dxy, int nxy, float inc, float dRA, float dDec, float duv, float PA,
                                  int nd, const float *u_dev, const float *v_dev, const float *re_dev,
                                  const float *im_dev, const float *w_dev, double *chi2_dev, void *stream);
int galario_chi2_image_device_d(int nx, int ny, const double *image_dev, double v_origin, double dRA, double dDec,
                                double duv, double PA, int nd, const double *u_dev, const double *v_dev,
                                const double *re_dev, const double *im_dev, const double *w_dev, double *chi2_dev,
                                void *stream);
int galario_chi2_image_device_f(int nx, int ny, const float *image_dev, float v_origin, float dRA, float dDec,
                                float duv, float PA, int nd, const float *u_dev, const float *v_dev,
                                const float *re_dev, const float *im_dev, const float *w_dev, double *chi2_dev,
                                void *stream);
/* Synchronise the device and return the error bits of the last device-resident call. */
int galario_device_status(unsigned int *err_bits);

/* ---- allocation-free chi2 reduction (no counterpart in the reference) ----
 * For callers that cannot let this library allocate GPU memory: device memory
 * owned by another allocator (PyTorch's caching allocator, a pool sized at
 * start-up) or loops that cannot afford the device-wide synchronisation of
 * cudaFree.  Computes chi2 = sum_k w_k |vis_k - (re_k + i im_k)|^2 (double,
 * accumulated in double) of caller-owned DEVICE arrays and writes it to
 * chi2_dev (device memory); only enqueues work on `stream` (NULL: CUDA's
 * default stream).  It calls no cudaMalloc/cudaFree: its scratch is a fixed
 * 32 KiB array inside the library's device image, held by every GPU that
 * loads the library until exit.
 *  - re_dev, im_dev, w_dev: nd doubles; vis_dev: nd interleaved (re, im)
 *    doubles, 16-byte aligned (as a complex128 array), otherwise
 *    GALARIO_EINVAL;
 *  - nd <= 16,777,216, otherwise GALARIO_EINVAL; nd == 0 writes 0;
 *  - the first call on a device (with it current) looks up the scratch
 *    address once; make that first call before any stream capture;
 *    galario_cleanup() forgets the addresses (needed after cudaDeviceReset);
 *  - all calls share the scratch: calls whose kernels overlap on the GPU
 *    race; order them on one stream. */
int galario_reduce_chi2_noalloc_d(int nd, const double *re_dev, const double *im_dev, const double *vis_dev,
                                  const double *w_dev, double *chi2_dev, void *stream);

/* ---- measurement helper (no reference counterpart) ----
 * FP64 fused multiply-add throughput of the current device in GFLOP/s (two
 * flops per FMA; independent chains, 8 blocks of 256 threads per SM, best of
 * five timed launches): the FP64-pipe peak that the double-precision kernels'
 * roofline is quoted against.  Allocates and frees a small buffer. */
int galario_measure_fp64_peak(double *gflops);

/* ---- stage timing (no reference counterpart; the reference's compile-time
 * GALARIO_TIMING prints, src/galario.cpp:64-87,275-315, become queryable
 * CUDA-event times).  With timing enabled every pipeline stage of the calls
 * on this device is bracketed by CUDA events on its stream; stage ids:
 * 0 h2d, 1 extent, 2 rows, 3 cols, 4 vis, 5 d2h, 6 quad. ---- */
int galario_stage_timing(int enable);
const char *galario_stage_name(int stage);
/* Synchronise, then return per stage the summed milliseconds and the number of
 * timed launches since the previous query (arrays of nstages entries). */
int galario_stage_times(double *ms_sum, int *count, int nstages);

/* ---- expert stages (reference src/galario_py.h:36-46, python/libcommon.pyx:800-1082) ---- */

/* replaces galario::_sweep (src/galario.cpp:1240-1256): image is the padded
 * R2C buffer, nxy rows of 2*(nxy/2+1) reals (output). */
int galario_sweep_d(int nr, const double *intensity, double Rmin, double dR, int nxy, double dxy, double inc,
                    double *image);
int galario_sweep_f(int nr, const float *intensity, float Rmin, float dR, int nxy, float dxy, float inc, float *image);

/* replaces galario::_uv_rotate (src/galario.cpp:1002-1039) */
int galario_uv_rotate_d(double PA, double dRA, double dDec, double *dRArot, double *dDecrot, int nd, const double *u,
                        const double *v, double *urot, double *vrot);
int galario_uv_rotate_f(float PA, float dRA, float dDec, float *dRArot, float *dDecrot, int nd, const float *u,
                        const float *v, float *urot, float *vrot);

/* replaces galario::_interpolate (src/galario.cpp:841-873): data is nrow x ncol complex */
int galario_interpolate_d(int nrow, int ncol, const double *data, double v_origin, int nd, const double *u,
                          const double *v, double duv, double *vis);
int galario_interpolate_f(int nrow, int ncol, const float *data, float v_origin, int nd, const float *u,
                          const float *v, float duv, float *vis);

/* replaces galario::_apply_phase_sampled (src/galario.cpp:924-945): vis in place */
int galario_apply_phase_sampled_d(double dRA, double dDec, int nd, const double *u, const double *v, double *vis);
int galario_apply_phase_sampled_f(float dRA, float dDec, int nd, const float *u, const float *v, float *vis);

/* replaces galario::_reduce_chi2 (src/galario.cpp:1504-1538) */
int galario_reduce_chi2_d(int nd, const double *re, const double *im, const double *vis, const double *w,
                          double *chi2);
int galario_reduce_chi2_f(int nd, const float *re, const float *im, const float *vis, const float *w, float *chi2);

/* replaces galario::_copy_input + galario::_fft2d (src/galario.cpp:460-491,527-547):
 * in-place R2C on the padded layout (nx rows of 2*(ny/2+1) reals in,
 * nx x (ny/2+1) complex out), unnormalised, forward sign -1. */
int galario_fft2d_d(int nx, int ny, double *data);
int galario_fft2d_f(int nx, int ny, float *data);

/* replaces galario::_fftshift (src/galario.cpp:625-643): quadrant swap of the
 * real image held in the padded layout, in place */
int galario_fftshift_d(int nx, int ny, double *data);
int galario_fftshift_f(int nx, int ny, float *data);

/* replaces galario::_fftshift_axis0 (src/galario.cpp:700-717): nrow x ncol complex, in place */
int galario_fftshift_axis0_d(int nrow, int ncol, double *data);
int galario_fftshift_axis0_f(int nrow, int ncol, float *data);

/* ---- batched FP32 chi2 with gradient (no counterpart in the reference,
 * which evaluates one model per call and has no derivative).
 *
 * A dataset is a device-resident copy of nd visibilities (float32), made of
 * nsets visibility sets stored one after the other: set k holds the entries
 * [set_offsets[k], set_offsets[k+1]) of the input arrays (set_offsets has
 * nsets + 1 entries, starts at 0 and ends at nd; NULL with nsets == 1 means
 * one set).  on_device != 0: the five input pointers are device pointers.
 * The copy is reordered (Morton order of (u, v) within each set) and padded
 * with zero-weight entries; visibilities of weight 0 contribute nothing. */
int galario_dataset_create_f(int nd, const float *u, const float *v, const float *re, const float *im,
                             const float *w, int nsets, const int *set_offsets, int on_device, void **handle);
int galario_dataset_free(void *handle);
int galario_dataset_nvis(void *handle, int *nd);
int galario_dataset_nsets(void *handle, int *nsets);

/* chi2 of B radial-profile models against a dataset, on `stream` (a
 * cudaStream_t; NULL is CUDA's default stream).  Device pointers:
 *  intensity (B x nr) [Jy/sr] on R = Rmin + i dR, shared radial grid;
 *  params (B x 4): inc, PA, dRA, dDec [rad] per model;
 *  chi2 (B, double): total over the dataset's sets;
 *  chi2_sets (B x nsets, double) or NULL: chi2 of every set;
 *  grad_intensity (B x nr) and grad_params (B x 4), both or neither (NULL):
 *  d(total chi2)/d(intensity, params).
 * Geometry rules as chi2Profile (galario.cpp:101-121 checks), with nxy a
 * power of two in [16, 16384], or any even nxy in that range when the
 * spectrum passes run on the tensor cores (profiles with rmax+1 <= 2048,
 * K <= 2048, W <= 4096, nr <= 40960; GALARIO_TC=0 turns them off).
 * Arithmetic: FP32 FFTs and interpolation;
 * uv rotation, cell index and phase in double-float; chi2 and the parameter
 * gradients accumulated in double.  Calls on one device share a workspace
 * and are serialised by a lock. */
int galario_chi2_profile_batch_f(void *dataset, int B, int nr, const float *intensity, float Rmin, float dR,
                                 float dxy, int nxy, const float *params, double *chi2, double *chi2_sets,
                                 float *grad_intensity, float *grad_params, void *stream);

/* chi2 of B images against a dataset (chi2Image semantics per image, no
 * reference counterpart for the batch or the gradient).  Device pointers:
 *  images (B x nxy x nxy) [Jy/pixel], nxy a power of two in [16, 16384];
 *  params (B x 3): PA, dRA, dDec [rad] per image;
 *  v_origin: +1 ('upper') or -1 ('lower'), as the reference's origin;
 *  chi2, chi2_sets as galario_chi2_profile_batch_f;
 *  grad_images (B x nxy x nxy) and grad_params (B x 3), both or neither. */
int galario_chi2_image_batch_f(void *dataset, int B, int nxy, const float *images, float dxy, float v_origin,
                               const float *params, double *chi2, double *chi2_sets, float *grad_images,
                               float *grad_params, void *stream);

/* Synchronise the device and return the error bits of the last batched call
 * on the current device: 0, or 4 when a visibility's cell had to be clamped
 * to the spectrum window (the host-side checks of the dataset and of the
 * image's uv range rule this out). */
int galario_batch_status(unsigned int *err_bits);

#ifdef __cplusplus
}
#endif
#endif /* GALARIO_GB300_H */
