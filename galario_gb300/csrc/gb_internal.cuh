// Internal declarations shared by the galario_gb300 CUDA translation units.
//
// Data layout in HBM for one model evaluation (N = nxy, C = N/2 + 1):
//   image     N x N real, row-major (sampleImage/chi2Image input)        [optional]
//   zt        K x N complex, column-major ("transposed rows"): zt[k*N + i] is
//             the k-th real-FFT output of image row i times (-1)^i
//   window    K x W complex, column-major: window[k*W + (r - r0)] is the
//             fftshift-ed half-plane spectrum S[r][k] for rows r in [r0, r0+W)
//   u, v, re, im, w   nd reals each (structure of arrays)
// K (columns) and [r0, r0+W) (rows) are the part of the spectrum the uv
// points can touch; they follow from max(u^2+v^2) and are computed on the
// device by window_from_extent() so that no host round trip is needed.
#pragma once

#include <cuda_runtime.h>

#include <cstring>
#include <stdint.h>

namespace gbg {

template <typename T> struct Cplx;
template <> struct Cplx<double> { using type = double2; };
template <> struct Cplx<float> { using type = float2; };
template <typename T> using C2 = typename Cplx<T>::type;

// Device-side state of one pipeline run (lives in device memory, 64 bytes).
struct DevState {
    double rmax2;                 // max(u^2 + v^2) over the dataset (atomicMax on the bit pattern)
    double chi2;                  // final chi2 (written by the last reduction block)
    unsigned int err;             // error bits, see ERR_*
    unsigned int ticket;          // last-block-done counter of the chi2 reduction
    unsigned long long err_index; // first offending visibility index + 1 (best effort)
    int win_K, win_r0, win_W;     // spectrum window, written once by the extent pass
    unsigned int ticket_extent;   // last-block-done counter of the extent pass
    double pad[2];
};

enum : unsigned int {
    ERR_UV_OUTSIDE = 1u,     // a bilinear corner falls outside the N x (N/2+1) spectrum
    ERR_UV_NONFINITE = 2u,   // u or v is NaN/inf
    ERR_WINDOW = 4u,         // internal: corner outside the computed window (should not happen)
    ERR_SPIN = 8u,           // a bounded wait gave up
};

// The part of the half-plane spectrum that can be touched by uv points whose
// radius is at most sqrt(rmax2):  columns [0, K), rows [r0, r0 + W).
struct Window {
    int K, r0, W;
};

__host__ __device__ inline Window window_from_extent(double rmax2, double duv, int N) {
    const int C = N / 2 + 1;
    Window w;
    double ext = sqrt(rmax2) / duv;
    ext = ext * (1.0 + 2e-6) + 1e-6;           // rotation/rounding margin (covers a float-precision max)
    if (!(ext < 4.0 * N)) ext = 4.0 * N;       // NaN/inf/huge: clamp (points get flagged later)
    int fu = (int)floor(ext);
    int K = fu + 2;                             // fl_u and fl_u + 1
    if (K > C) K = C;
    int kv = (int)ceil(ext);
    int r0 = N / 2 - kv - 1;
    int r1 = N / 2 + kv + 3;                    // fl_v + 1, and fl_v + 2 for the row wrap at u column C-1
    if (r0 < 0) r0 = 0;
    if (r1 > N) r1 = N;
    w.K = K;
    w.r0 = r0;
    w.W = r1 - r0;
    return w;
}

// double-float value hi + lo (two floats, about 44 significant bits)
struct DF {
    float hi, lo;
};

// reals per cell record of the quad layout (8 for the corners, 4 moduli, 4 padding)
constexpr int QUAD_REC = 16;
// cells of the quad buffer (2^21: 128 MiB in FP32, 256 MiB in FP64)
constexpr long long QUAD_CAP = 1LL << 21;

// size of the table of the table-driven sin/cos of the phase shift (a power of two)
constexpr int PHASE_T = 1 << 20;

inline bool is_pow2(long long n) { return n > 0 && (n & (n - 1)) == 0; }

// ---------------------------------------------------------------------------
// Kernel launchers (gb_kernels.cu).  All are asynchronous on `stream`.
// ---------------------------------------------------------------------------
template <typename T> struct Launch {
    using CT = C2<T>;
    // dataset extent: state->rmax2 = max(u^2 + v^2)
    // ... and the window (state->win_*) derived from it for an N x N image with cell duv.
    // u_out, v_out (both or neither): also copy u, v there (u, v may then be
    // host memory the device reads directly)
    static cudaError_t extent(const T* u, const T* v, int nd, int N, double duv, DevState* state, cudaStream_t s,
                              T* u_out = nullptr, T* v_out = nullptr);
    // copy [0, n) of a, b, c into da, db, dc (the sources may be host memory the device reads directly)
    static cudaError_t stage3(const T* a, const T* b, const T* c, T* da, T* db, T* dc, int n, cudaStream_t s);
    // row pass on an image (rows [0, N)), output zt for columns [0, K) where
    // K = host_K if >= 0, else from state->rmax2 (window_from_extent).
    // row_sign: multiply row i by (-1)^i.
    // tw: exp(-2 pi i m / N), m in [0, N); stw: stage twiddles of the length-N/2 row FFT
    static cudaError_t rows_image(const T* image, int N, const CT* tw, const CT* stw, CT* zt, int host_K,
                                  const DevState* state, double duv, bool row_sign, cudaStream_t s);
    // row pass fused with the profile sweep: only rows [N/2 - rmax, N/2 + rmax) are nonzero.
    // Writes columns [0, kcols), or the device window's K columns when kcols < 0
    // (kcols >= 0 lets the pass run before the extent pass).
    static cudaError_t rows_profile(const T* intensity, int nr, double Rmin, double dR, double dxy, double cos_inc,
                                    int rmax, double central_value, int N, const CT* tw, const CT* stw, CT* zt,
                                    const DevState* state, double duv, cudaStream_t s, int kcols = -1,
                                    const CT* stw4 = nullptr);
    // column pass: column FFTs of zt (rows outside [band0, band1) are zero) and
    // write rows [r0, r0+W) of columns [0, K) to out[(r - r0)*s_row + k*s_col],
    // times (-1)^(r + k + N/2) if out_sign.  host_K/host_r0/host_W >= 0 override
    // the device-derived window.
    // amp_out (optional, same layout as out) receives |out|, so the visibility
    // pass gathers amplitudes instead of recomputing 4 moduli per point.
    // column pass of a swept profile (real, even columns): two columns per
    // complex transform; device window; output sign applied
    // stw4 (stage twiddles of length N/4; row pass too): the even-sequence
    // transform of one column per block, for the N where even_dft_ok holds
    static cudaError_t cols_profile(const CT* zt, int N, int band0, int band1, const CT* tw, const CT* stw, CT* out,
                                    T* amp_out, long long s_row, long long s_col, const DevState* state, double duv,
                                    cudaStream_t s, const CT* stw4 = nullptr);
    // stw: stage twiddles of the length-N column FFT
    static cudaError_t cols(const CT* zt, int N, int band0, int band1, const CT* tw, const CT* stw, CT* out,
                            T* amp_out, long long s_row, long long s_col, int host_K, int host_r0, int host_W,
                            const DevState* state, double duv, bool out_sign, cudaStream_t s);
    // fused rotation + interpolation + phase + (vis out) + (chi2 reduction)
    struct VisArgs {
        const CT* spec;      // spectrum window
        const T* amp;        // |spec| in the same layout, or null (computed on the fly)
        const T* quads;      // cell-major records (see Launch::quads), or null: gather from spec/amp
        bool real_quads = false;  // quads hold 4 real corners per cell (real spectrum of a swept profile)
        long long quad_cap;  // capacity of quads in cells; larger windows gather from spec/amp
        const double2* phase_tab;  // exp(2 pi i j / PHASE_T), j in [0, PHASE_T); FP64 path
        long long s_row, s_col;
        int nrow, ncol;      // logical N and C of the full spectrum (flat-index semantics)
        int host_K, host_r0, host_W;  // window (>= 0) or derive from state
        double duv, v_origin, cos_pa, sin_pa;
        bool rotate;         // PA != 0
        double dra, ddec;    // rotated offsets (radians, not yet times 2 pi)
        bool phase;          // dra != 0 || ddec != 0
        // derived on the host by finalize(): no per-thread FP64 set-up in the kernels
        double inv_duv, half_nrow;
        // FP64 path: grid coordinates (a, c) = (u', v') / duv from (u, v) with
        // cu = cos(PA)/duv, su = sin(PA)/duv; the phase u' dra + v' ddec as
        // a dra_g + c ddec_g; vo_sign flips the sign bit of c for v_origin < 0
        double cu_d, su_d, dra_g, ddec_g;
        long long vo_sign, lim_bits;  // lim_bits: bit pattern of 4 N (coarse range check)
        float half_nrow_f, v_origin_f;
        DF inv_duv_df, cpa, spa, dra_df, ddec_df;  // double-float copies for the FP32 path
        void finalize() {
            auto split = [](double x) {
                DF r;
                r.hi = (float)x;
                r.lo = (float)(x - (double)r.hi);
                return r;
            };
            inv_duv = 1.0 / duv;
            half_nrow = (double)(nrow / 2);
            cu_d = cos_pa * inv_duv;
            su_d = sin_pa * inv_duv;
            dra_g = dra * duv;
            ddec_g = ddec * duv;
            vo_sign = v_origin < 0 ? (long long)0x8000000000000000ULL : 0LL;
            const double lim = 4.0 * nrow;
            std::memcpy(&lim_bits, &lim, sizeof(lim));
            half_nrow_f = (float)(nrow / 2);
            v_origin_f = (float)v_origin;
            inv_duv_df = split(inv_duv);
            cpa = split(cos_pa);
            spa = split(sin_pa);
            dra_df = split(dra);
            ddec_df = split(ddec);
        }
        const T *u, *v, *re, *im, *w;
        // observations of visibilities [split, nd) come from re2/im2/w2 (same
        // indexing) instead: the caller's host arrays, read in place, when
        // re/im/w hold device copies of the first `split` only
        const T *re2 = nullptr, *im2 = nullptr, *w2 = nullptr;
        int split = 0x7fffffff;
        int nd;
        CT* vis_out;         // may be null
        double* partials;    // chi2 partials (null: no chi2)
        double* chi2_out;    // optional extra copy of the final chi2 (device)
        DevState* state;
        // one chunk of a set of launches over the visibilities: u..w and
        // vis_out point at the chunk, `base` is its first visibility's index,
        // `part_off` the first chi2 partial slot of this launch and
        // `parts_total` the blocks of all the set's launches (0: this launch alone)
        int base = 0;
        int part_off = 0;
        int parts_total = 0;
    };
    // pdl: launch as a programmatic dependent of the stream's previous kernel
    // (the kernels wait with griddepcontrol.wait before reading its output)
    static cudaError_t vis(const VisArgs& a, cudaStream_t s, bool pdl = false);
    // Cell-major copy of the window for the visibility gather: one record of
    // QUAD_REC reals per cell (k, r), k in [0, K), r in [r0, r0 + W), at
    // quads + (k * W + (r - r0)) * QUAD_REC, holding the cell's 4 bilinear
    // corners y0 = S[r][k], y1 = S[r+1][k], y2 = S[r+1][k+1], y3 = S[r][k+1]
    // (complex, re/im) then their 4 moduli.  At k = C-1 the corners k+1 are
    // taken from column 0 of the next rows, as the reference's flat indexing
    // does.  Cells whose corners fall outside the window are left unwritten
    // and never read.
    // A window of more than `cap` cells is not converted (the gather then falls back to spec/amp).
    static cudaError_t quads(const CT* spec, const T* amp, long long s_row, long long s_col, int C,
                             const DevState* state, T* quads, long long cap, int host_K, int host_r0, int host_W,
                             cudaStream_t s);
    // records of a real spectrum: FP32, the 4 real corners of every cell (16
    // bytes); FP64, the 4 coefficients of the bilinear modulus and the 4
    // corners as FP32 (48 bytes; see quad_real_kernel)
    static cudaError_t quads_real(const CT* spec, long long s_row, long long s_col, int C, const DevState* state,
                                  T* quads, long long cap, cudaStream_t s, bool pdl = false);
    static int vis_grid(int nd);
    // expert-stage kernels
    static cudaError_t fftshift_real(T* padded, int N, cudaStream_t s);
    static cudaError_t fftshift_axis0(CT* m, int nrow, int ncol, cudaStream_t s);
    static cudaError_t apply_phase(const T* u, const T* v, CT* vis, int nd, double dra, double ddec, cudaStream_t s);
    static cudaError_t rotate(const T* u, const T* v, T* urot, T* vrot, int nd, double c, double sn, cudaStream_t s);
    static cudaError_t reduce(const T* re, const T* im, const CT* vis, const T* w, int nd, double* partials,
                              DevState* state, cudaStream_t s);
    static cudaError_t sweep_image(const T* intensity, int nr, double Rmin, double dR, double dxy, double cos_inc,
                                   int rmax, double central_value, int N, T* padded, cudaStream_t s);
    // largest N the shared-memory FFT kernels handle for this precision
    static int max_fft_n();
};

int num_sms();

// ---------------------------------------------------------------------------
// Spectrum window of a swept FP64 profile as two FP64-grade cosine-matrix
// products on the tensor cores (gb_profile_tc.cu), per-device state.
// ---------------------------------------------------------------------------
struct ProfileTc;
ProfileTc* profile_tc_new();
void profile_tc_free(ProfileTc* t);
// quadrant size of the sweep: columns/rows c < nF of the folded image
int profile_tc_quadrant(int N, int rmax);
// the path applies: even N, a quadrant within the exact level sums
// (nF <= 511), tensor maps available, GALARIO_TC not 0
bool profile_tc_ok(int N, int rmax);
// the quadrant of the sweep as digits (independent of the window); prepares
// the geometry (cosine digits, buffers) on its first call for (N, nF)
cudaError_t profile_tc_fold(ProfileTc* t, const double* intensity, int nr, double Rmin, double dR, double dxy,
                            double cos_inc, int rmax, double central, int N, cudaStream_t s);
// after the extent pass: the window (out, amp: rows [r0, r0+W) of columns
// [0, K) at q * s_row + k * s_col); errors of bounded waits set ERR_SPIN in st
cudaError_t profile_tc_window(ProfileTc* t, int N, DevState* st, C2<double>* out, double* amp, long long s_row,
                              long long s_col, cudaStream_t s);

}  // namespace gbg
