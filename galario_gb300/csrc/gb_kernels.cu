// GB300 (sm_103a) kernels for galario's synthetic-visibility / chi2 path.
//
// Pipeline for one model (reference stage order: src/galario.cpp:1258-1321):
//   [profile] sweep fused into the row pass           (reference sweep_core :1048-1071)
//   row pass:   real FFT of each image row in shared memory, times (-1)^row,
//               only the K spectrum columns the uv points can touch are written
//   column pass: complex FFT of each needed column in shared memory, only the
//               window rows are written, times (-1)^(r + k + N/2)
//   vis pass:   rotation + Hermitian bilinear amp/phase interpolation + phase
//               shift + weighted residual + deterministic FP64 chi2 reduction
//
// The two fftshifts of the reference (shift_d :595-612 before the FFT and
// shift_axis0_d :674-688 after it) are folded into sign patterns:
//   fftshift_axis0(rfft2(fftshift(x)))[r, k] = rfft2(x * (-1)^i)[r, k] * (-1)^(r + k + N/2)
// which is exact (multiplication by +-1), so no extra pass over the data runs.
//
// FFTs are Stockham autosort radix-8/4/2 stages on a block of E complex values
// per thread (Govindaraju et al., "High performance discrete Fourier
// transforms on graphics processors", SC 2008), with twiddles read from an
// accurate table built on the host.  Other lengths use a direct DFT.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "gb_internal.cuh"

namespace gbg {

namespace {

// ---------------------------------------------------------------------------
// complex helpers
// ---------------------------------------------------------------------------
template <typename CT> __device__ __forceinline__ CT cadd(CT a, CT b) { return CT{a.x + b.x, a.y + b.y}; }
template <typename CT> __device__ __forceinline__ CT csub(CT a, CT b) { return CT{a.x - b.x, a.y - b.y}; }
template <typename CT> __device__ __forceinline__ CT cmul(CT a, CT b) {
    return CT{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// (-i) * a
template <typename CT> __device__ __forceinline__ CT cmul_mi(CT a) { return CT{a.y, -a.x}; }
template <typename CT> __device__ __forceinline__ CT cneg(CT a) { return CT{-a.x, -a.y}; }

template <typename T> __device__ __forceinline__ T sqrt_half();
template <> __device__ __forceinline__ double sqrt_half<double>() { return 0.70710678118654752440084436210485; }
template <> __device__ __forceinline__ float sqrt_half<float>() { return 0.70710678118654752440f; }

// in-register forward DFT of size R (natural order in and out)
template <typename T, int R> struct Dft;
template <typename T> struct Dft<T, 2> {
    using CT = C2<T>;
    __device__ __forceinline__ static void run(CT* v) {
        CT a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};
template <typename T> struct Dft<T, 4> {
    using CT = C2<T>;
    __device__ __forceinline__ static void run(CT* v) {
        CT t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        CT t2 = cadd(v[1], v[3]), t3 = cmul_mi(csub(v[1], v[3]));
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3);
        v[3] = csub(t1, t3);
    }
};
template <typename T> struct Dft<T, 8> {
    using CT = C2<T>;
    __device__ __forceinline__ static void run(CT* v) {
        CT e[4] = {v[0], v[2], v[4], v[6]};
        CT o[4] = {v[1], v[3], v[5], v[7]};
        Dft<T, 4>::run(e);
        Dft<T, 4>::run(o);
        const T c = sqrt_half<T>();
        // o[k] *= exp(-2 pi i k / 8)
        CT o1 = CT{c * (o[1].x + o[1].y), c * (o[1].y - o[1].x)};
        CT o2 = cmul_mi(o[2]);
        CT o3 = CT{c * (o[3].y - o[3].x), -c * (o[3].x + o[3].y)};
        v[0] = cadd(e[0], o[0]);
        v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], o1);
        v[5] = csub(e[1], o1);
        v[2] = cadd(e[2], o2);
        v[6] = csub(e[2], o2);
        v[3] = cadd(e[3], o3);
        v[7] = csub(e[3], o3);
    }
};

// One Stockham stage of radix R on buf[0, M) (in place, two barriers).
// Every thread owns E/R butterflies.  tw[m] = exp(-2 pi i m / twN), twN = tw_mul * M.
template <typename T, int E, int R>
__device__ __forceinline__ void stockham_stage(C2<T>* buf, int M, int Ns, const C2<T>* __restrict__ tw, int tw_mul) {
    using CT = C2<T>;
    constexpr int B = E / R;
    const int nt = blockDim.x, tid = threadIdx.x;
    const int stride = M / R;
    CT v[E];
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = tid + b * nt;
#pragma unroll
        for (int r = 0; r < R; ++r) v[b * R + r] = buf[j + r * stride];
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = tid + b * nt;
        const int k = j & (Ns - 1);
        if (Ns > 1) {
            const int step = k * tw_mul * (M / (Ns * R));
#pragma unroll
            for (int r = 1; r < R; ++r) v[b * R + r] = cmul(v[b * R + r], __ldg(&tw[r * step]));
        }
        Dft<T, R>::run(&v[b * R]);
        const int d = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) buf[d + r * Ns] = v[b * R + r];
    }
    __syncthreads();
}

template <typename T> struct Dft<T, 1> {
    __device__ __forceinline__ static void run(C2<T>*) {}
};

// Forward complex FFT of length M = E * blockDim.x (power of two) on shared
// memory, natural order in and out.
template <typename T, int E>
__device__ void block_fft(C2<T>* buf, int M, int log2M, const C2<T>* __restrict__ tw, int tw_mul) {
    int Ns = 1, bits = log2M;
    while (bits > 0) {
        if constexpr (E >= 8) {
            if (bits >= 3) {
                stockham_stage<T, E, 8>(buf, M, Ns, tw, tw_mul);
                Ns <<= 3;
                bits -= 3;
                continue;
            }
        }
        if constexpr (E >= 4) {
            if (bits >= 2) {
                stockham_stage<T, E, 4>(buf, M, Ns, tw, tw_mul);
                Ns <<= 2;
                bits -= 2;
                continue;
            }
        }
        if constexpr (E >= 2) {
            stockham_stage<T, E, 2>(buf, M, Ns, tw, tw_mul);
            Ns <<= 1;
            bits -= 1;
        } else {
            bits = 0;  // E == 1 means M == 1: nothing to do
        }
    }
}

__device__ __forceinline__ int ilog2(int n) { return 31 - __clz(n); }

template <typename T> __device__ __forceinline__ T tw_cast(double x) { return (T)x; }

// ---------------------------------------------------------------------------
// Real-row post-processing: X[k] = E[k] + exp(-2 pi i k/N) O[k], k in [0, K)
// from the length-M complex FFT Z of z[m] = x[2m] + i x[2m+1].
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ C2<T> real_split(const C2<T>* Z, int M, int k, const C2<T>* __restrict__ tw) {
    using CT = C2<T>;
    const CT za = Z[k == M ? 0 : k];
    const CT zb = Z[k == 0 ? 0 : M - k];
    // Ek = (za + conj(zb))/2 ; Ok = (za - conj(zb))/(2i)
    const T h = (T)0.5;
    const CT e = CT{h * (za.x + zb.x), h * (za.y - zb.y)};
    const T pr = za.x - zb.x, pi = za.y + zb.y;
    const CT o = CT{h * pi, -h * pr};
    const CT w = __ldg(&tw[k]);  // exp(-2 pi i k / N), N = 2M
    return cadd(e, cmul(o, w));
}

// ---------------------------------------------------------------------------
// row pass kernels
// ---------------------------------------------------------------------------
template <typename T, int E>
__global__ void __launch_bounds__(1024) rows_image_kernel(const T* __restrict__ image, int N, const C2<T>* __restrict__ tw,
                                                          C2<T>* __restrict__ zt, int host_K,
                                                          const DevState* __restrict__ st, double duv, int row_sign) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT* buf = reinterpret_cast<CT*>(smem_raw);
    const int M = N / 2;
    const int i = blockIdx.x;
    const CT* row = reinterpret_cast<const CT*>(image + (size_t)i * N);
    for (int m = threadIdx.x; m < M; m += blockDim.x) buf[m] = __ldg(&row[m]);
    __syncthreads();
    block_fft<T, E>(buf, M, ilog2(M), tw, 2);
    const int K = host_K >= 0 ? host_K : window_from_extent(st->rmax2, duv, N).K;
    const T sgn = (row_sign && (i & 1)) ? (T)-1 : (T)1;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        CT x = real_split<T>(buf, M, k, tw);
        zt[(size_t)k * N + i] = CT{sgn * x.x, sgn * x.y};
    }
}

// sweep of a radial profile (reference sweep_core, src/galario.cpp:1048-1071)
// evaluated for image pixel (I, J); zero outside the 2*rmax box.
template <typename T>
__device__ __forceinline__ T sweep_pixel(int I, int J, const T* __restrict__ intensity, int nr, T Rmin, T dR, T dxy,
                                         T inv_cos_inc, int rmax, int off, T sr_to_px) {
    const int i = I - off, j = J - off;
    if (i < 0 || j < 0 || i >= 2 * rmax || j >= 2 * rmax) return (T)0;
    const T x = (T)(rmax - j) * dxy;
    const T y = (T)(rmax - i) * dxy;
    const T xs = x * inv_cos_inc;
    const T r = sqrt(xs * xs + y * y);
    int iR = (int)floor((r - Rmin) / dR);
    if (iR < 0) iR = 0;
    if (iR > nr - 2) return (T)0;
    const T I0 = __ldg(&intensity[iR]), I1 = __ldg(&intensity[iR + 1]);
    return sr_to_px * (I0 + (r - (T)iR * dR - Rmin) * (I1 - I0) / dR);
}

template <typename T, int E>
__global__ void __launch_bounds__(1024) rows_profile_kernel(const T* __restrict__ intensity, int nr, T Rmin, T dR,
                                                            T dxy, T inv_cos_inc, int rmax, T central, int N,
                                                            const C2<T>* __restrict__ tw, C2<T>* __restrict__ zt,
                                                            const DevState* __restrict__ st, double duv) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT* buf = reinterpret_cast<CT*>(smem_raw);
    const int M = N / 2;
    const int off = N / 2 - rmax;
    const int I = off + blockIdx.x;  // image row
    const T sr_to_px = dxy * dxy;
    for (int m = threadIdx.x; m < M; m += blockDim.x) {
        const int J0 = 2 * m, J1 = 2 * m + 1;
        T a = sweep_pixel<T>(I, J0, intensity, nr, Rmin, dR, dxy, inv_cos_inc, rmax, off, sr_to_px);
        T b = sweep_pixel<T>(I, J1, intensity, nr, Rmin, dR, dxy, inv_cos_inc, rmax, off, sr_to_px);
        if (I == N / 2) {  // reference central_pixel_d :1075-1079
            if (J0 == N / 2) a = central;
            if (J1 == N / 2) b = central;
        }
        buf[m] = CT{a, b};
    }
    __syncthreads();
    block_fft<T, E>(buf, M, ilog2(M), tw, 2);
    const int K = window_from_extent(st->rmax2, duv, N).K;
    const T sgn = (I & 1) ? (T)-1 : (T)1;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        CT x = real_split<T>(buf, M, k, tw);
        zt[(size_t)k * N + I] = CT{sgn * x.x, sgn * x.y};
    }
}

// ---------------------------------------------------------------------------
// column pass
// ---------------------------------------------------------------------------
template <typename T, int E>
__global__ void __launch_bounds__(1024) cols_kernel(const C2<T>* __restrict__ zt, int N, int band0, int band1,
                                                    const C2<T>* __restrict__ tw, C2<T>* __restrict__ out,
                                                    long long s_row, long long s_col, int host_K, int host_r0,
                                                    int host_W, const DevState* __restrict__ st, double duv,
                                                    int out_sign) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT* buf = reinterpret_cast<CT*>(smem_raw);
    Window w;
    if (host_K >= 0) {
        w.K = host_K;
        w.r0 = host_r0;
        w.W = host_W;
    } else {
        w = window_from_extent(st->rmax2, duv, N);
    }
    const int k = blockIdx.x;
    if (k >= w.K) return;  // uniform for the whole block
    const CT* col = zt + (size_t)k * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x)
        buf[i] = (i >= band0 && i < band1) ? __ldg(&col[i]) : CT{(T)0, (T)0};
    __syncthreads();
    block_fft<T, E>(buf, N, ilog2(N), tw, 1);
    const int par = (k + N / 2) & 1;
    for (int q = threadIdx.x; q < w.W; q += blockDim.x) {
        const int r = w.r0 + q;
        CT x = buf[r];
        if (out_sign && ((r & 1) ^ par)) x = cneg(x);
        out[(long long)q * s_row + (long long)k * s_col] = x;
    }
}

// ---------------------------------------------------------------------------
// direct-DFT fallbacks for lengths the shared-memory FFT does not handle
// (non powers of two, or too long for shared memory); tw has N entries.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void rows_direct_kernel(const T* __restrict__ image, int N, int row0, const T* __restrict__ intensity,
                                   int nr, T Rmin, T dR, T dxy, T inv_cos_inc, int rmax, T central, int profile,
                                   const C2<T>* __restrict__ tw, C2<T>* __restrict__ zt, int host_K,
                                   const DevState* __restrict__ st, double duv, int row_sign) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* row = reinterpret_cast<T*>(smem_raw);
    const int I = row0 + blockIdx.x;
    const int off = N / 2 - rmax;
    const T sr_to_px = dxy * dxy;
    for (int J = threadIdx.x; J < N; J += blockDim.x) {
        T x;
        if (profile) {
            x = sweep_pixel<T>(I, J, intensity, nr, Rmin, dR, dxy, inv_cos_inc, rmax, off, sr_to_px);
            if (I == N / 2 && J == N / 2) x = central;
        } else {
            x = image[(size_t)I * N + J];
        }
        row[J] = x;
    }
    __syncthreads();
    const int K = host_K >= 0 ? host_K : window_from_extent(st->rmax2, duv, N).K;
    const T sgn = (row_sign && (I & 1)) ? (T)-1 : (T)1;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        double sr = 0.0, si = 0.0;
        long long idx = 0;  // (J * k) mod N, advanced incrementally
        for (int J = 0; J < N; ++J) {
            const CT wv = __ldg(&tw[idx]);
            sr += (double)row[J] * (double)wv.x;
            si += (double)row[J] * (double)wv.y;
            idx += k;
            if (idx >= N) idx -= N;
        }
        zt[(size_t)k * N + I] = CT{sgn * (T)sr, sgn * (T)si};
    }
}

template <typename T>
__global__ void cols_direct_kernel(const C2<T>* __restrict__ zt, int N, int band0, int band1,
                                   const C2<T>* __restrict__ tw, C2<T>* __restrict__ out, long long s_row,
                                   long long s_col, int host_K, int host_r0, int host_W,
                                   const DevState* __restrict__ st, double duv, int out_sign) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT* col = reinterpret_cast<CT*>(smem_raw);
    Window w;
    if (host_K >= 0) {
        w.K = host_K;
        w.r0 = host_r0;
        w.W = host_W;
    } else {
        w = window_from_extent(st->rmax2, duv, N);
    }
    const int k = blockIdx.x;
    if (k >= w.K) return;
    for (int i = threadIdx.x; i < N; i += blockDim.x)
        col[i] = (i >= band0 && i < band1) ? zt[(size_t)k * N + i] : CT{(T)0, (T)0};
    __syncthreads();
    const int par = (k + N / 2) & 1;
    for (int q = threadIdx.x; q < w.W; q += blockDim.x) {
        const int r = w.r0 + q;
        double sr = 0.0, si = 0.0;
        long long idx = 0;  // (i * r) mod N
        for (int i = 0; i < N; ++i) {
            const CT z = col[i];
            const CT wv = __ldg(&tw[idx]);
            sr += (double)z.x * wv.x - (double)z.y * wv.y;
            si += (double)z.x * wv.y + (double)z.y * wv.x;
            idx += r;
            if (idx >= N) idx -= N;
        }
        CT x = CT{(T)sr, (T)si};
        if (out_sign && ((r & 1) ^ par)) x = cneg(x);
        out[(long long)q * s_row + (long long)k * s_col] = x;
    }
}

// ---------------------------------------------------------------------------
// dataset extent
// ---------------------------------------------------------------------------
template <typename T>
__global__ void extent_kernel(const T* __restrict__ u, const T* __restrict__ v, int nd, DevState* st) {
    double m = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += gridDim.x * blockDim.x) {
        const double a = (double)__ldg(&u[i]), b = (double)__ldg(&v[i]);
        const double r2 = a * a + b * b;
        m = fmax(m, r2);  // NaN entries are ignored here and flagged by the vis pass
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0)
        atomicMax(reinterpret_cast<unsigned long long*>(&st->rmax2), (unsigned long long)__double_as_longlong(m));
}

// ---------------------------------------------------------------------------
// block reduction helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double block_sum(double x, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = x;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < nw; ++q) s += sh[q];
    return s;  // valid in thread 0
}

// Deterministic grid reduction: each block writes its partial, the last block
// to arrive sums the partials in block order.
__device__ __forceinline__ void grid_finish(double block_total, double* partials, DevState* st,
                                            double* extra_out = nullptr) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = block_total;
        __threadfence();
        const unsigned t = atomicAdd(&st->ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double s = 0.0;
        const volatile double* p = partials;
        for (unsigned b = 0; b < gridDim.x; ++b) s += p[b];
        st->chi2 = s;
        if (extra_out) *extra_out = s;
        st->ticket = 0u;
    }
}

// ---------------------------------------------------------------------------
// fused visibility kernel
// reference: uv_rotate_core :955-960, interpolate_core :749-815,
//            apply_phase_sampled_core :877-884, diff_weighted_core :1453-1461
// ---------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ void sincos2pi(double a, T* s, T* c);
template <> __device__ __forceinline__ void sincos2pi<double>(double a, double* s, double* c) {
    sincospi(2.0 * a, s, c);
}
template <> __device__ __forceinline__ void sincos2pi<float>(double a, float* s, float* c) {
    // exact range reduction in FP64, evaluation in FP32
    const double f = a - rint(a);
    sincospif((float)(2.0 * f), s, c);
}
template <typename T> __device__ __forceinline__ T rnorm2(T x, T y);
template <> __device__ __forceinline__ double rnorm2<double>(double x, double y) { return rsqrt(fma(x, x, y * y)); }
template <> __device__ __forceinline__ float rnorm2<float>(float x, float y) { return rsqrtf(fmaf(x, x, y * y)); }
template <typename T> __device__ __forceinline__ T cabs_(C2<T> a);
template <> __device__ __forceinline__ double cabs_<double>(double2 a) { return sqrt(fma(a.x, a.x, a.y * a.y)); }
template <> __device__ __forceinline__ float cabs_<float>(float2 a) { return sqrtf(fmaf(a.x, a.x, a.y * a.y)); }

template <typename T, bool CHI2, bool VISOUT>
__global__ void __launch_bounds__(256) vis_kernel(typename Launch<T>::VisArgs a) {
    using CT = C2<T>;
    __shared__ double sh[32];
    Window w;
    if (a.host_K >= 0) {
        w.K = a.host_K;
        w.r0 = a.host_r0;
        w.W = a.host_W;
    } else {
        w = window_from_extent(a.state->rmax2, a.duv, a.nrow);
    }
    const long long C = a.ncol;
    const long long NC = (long long)a.nrow * C;
    const double inv_duv = 1.0 / a.duv;
    const double half = (double)(a.nrow / 2);
    double acc = 0.0;
    unsigned err = 0u;
    long long err_idx = -1;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < a.nd; idx += gridDim.x * blockDim.x) {
        double ur = (double)__ldg(&a.u[idx]);
        double vr = (double)__ldg(&a.v[idx]);
        if (a.rotate) {
            const double u0 = ur, v0 = vr;
            ur = u0 * a.cos_pa - v0 * a.sin_pa;
            vr = u0 * a.sin_pa + v0 * a.cos_pa;
        }
        CT out = CT{(T)0, (T)0};
        bool ok = isfinite(ur) && isfinite(vr);
        if (!ok) {
            err |= ERR_UV_NONFINITE;
            if (err_idx < 0) err_idx = idx;
        }
        double indu = 0.0, indv = 0.0, sign_u = 1.0;
        if (ok) {
            indu = fabs(ur) * inv_duv;
            sign_u = copysign(1.0, ur);
            indv = half + a.v_origin * sign_u * vr * inv_duv;
            if (!(indu < 4.0 * a.nrow && indv > -4.0 * a.nrow && indv < 4.0 * a.nrow)) {
                ok = false;
                err |= ERR_UV_OUTSIDE;
                if (err_idx < 0) err_idx = idx;
            }
        }
        if (ok) {
            const double fu = floor(indu), fv = floor(indv);
            const long long base = (long long)fu + (long long)fv * C;
            // flat-index semantics of the reference's row-major N x C array (:774-780)
            const long long b[4] = {base, base + C, base + C + 1, base + 1};
            if (base < 0 || base + C + 1 >= NC) {
                ok = false;
                err |= ERR_UV_OUTSIDE;
                if (err_idx < 0) err_idx = idx;
            } else {
                CT y[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int row = (int)(b[c] / C), col = (int)(b[c] - (long long)row * C);
                    const int rr = row - w.r0;
                    if (col >= w.K || rr < 0 || rr >= w.W) {
                        ok = false;
                        err |= ERR_WINDOW;
                        y[c] = CT{(T)0, (T)0};
                    } else {
                        y[c] = __ldg(&a.spec[(long long)rr * a.s_row + (long long)col * a.s_col]);
                    }
                }
                if (!ok && err_idx < 0) err_idx = idx;
                const T t = (T)(indv - fv);
                const T q = (T)(indu - fu);
                // complex bilinear (:782-800): t*q*(y0-y1+y2-y3) + t*(y1-y0) + q*(y3-y0) + y0
                const T d1r = (y[0].x + y[2].x) - (y[1].x + y[3].x);
                const T d1i = (y[0].y + y[2].y) - (y[1].y + y[3].y);
                const T zr = t * (q * d1r) + (t * (y[1].x - y[0].x) + q * (y[3].x - y[0].x)) + y[0].x;
                const T zi = t * (q * d1i) + (t * (y[1].y - y[0].y) + q * (y[3].y - y[0].y)) + y[0].y;
                // amplitude bilinear of |y| (:804-812)
                const T a0 = cabs_<T>(y[0]), a1 = cabs_<T>(y[1]), a2 = cabs_<T>(y[2]), a3 = cabs_<T>(y[3]);
                T amp = a0;
                amp += (a3 - a0) * q;
                amp += (a1 - a0) * t;
                amp += (a0 - a1 + a2 - a3) * t * q;
                // cos/sin of arg(z) * sign(u) without atan2: (zr, sign_u*zi)/|z|
                T cph = (T)1, sph = (T)0;
                if (zr != (T)0 || zi != (T)0) {
                    const T rn = rnorm2<T>(zr, zi);
                    cph = zr * rn;
                    sph = (T)sign_u * zi * rn;
                }
                out = CT{amp * cph, amp * sph};
                if (a.phase) {
                    T s, c;
                    sincos2pi<T>(ur * a.dra + vr * a.ddec, &s, &c);
                    out = cmul(out, CT{c, s});
                }
            }
        }
        if (VISOUT) a.vis_out[idx] = out;
        if (CHI2) {
            const double dr = (double)out.x - (double)__ldg(&a.re[idx]);
            const double di = (double)out.y - (double)__ldg(&a.im[idx]);
            acc += (double)__ldg(&a.w[idx]) * (dr * dr + di * di);
        }
    }
    if (err) {
        atomicOr(&a.state->err, err);
        atomicCAS(&a.state->err_index, 0ull, (unsigned long long)(err_idx + 1));
    }
    if (CHI2) {
        const double tot = block_sum(acc, sh);
        grid_finish(tot, a.partials, a.state, a.chi2_out);
    }
}

// ---------------------------------------------------------------------------
// expert-stage kernels
// ---------------------------------------------------------------------------
// 2D quadrant swap of a real N x N image inside the padded R2C buffer
// (reference shift_core :565-589)
template <typename T> __global__ void fftshift_real_kernel(T* a, int N) {
    const long long rowsize = 2LL * (N / 2 + 1);
    const int h = N / 2;
    const long long total = (long long)h * h;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(e / h), y = (int)(e % h);
        const long long s_ul = x * rowsize + y, s_ur = s_ul + h;
        const long long t_ul = s_ur + h * rowsize, t_ur = t_ul - h;
        T t = a[s_ul];
        a[s_ul] = a[t_ul];
        a[t_ul] = t;
        t = a[s_ur];
        a[s_ur] = a[t_ur];
        a[t_ur] = t;
    }
}

// swap the upper and lower halves (reference shift_axis0_core :657-668)
template <typename CT> __global__ void fftshift_axis0_kernel(CT* m, int nrow, int ncol) {
    const long long total = (long long)(nrow / 2) * ncol;
    const long long off = (long long)(nrow / 2) * ncol;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        CT t = m[e];
        m[e] = m[e + off];
        m[e + off] = t;
    }
}

// (reference apply_phase_sampled_core :877-884; skipped by the caller when both offsets are 0)
template <typename T>
__global__ void apply_phase_kernel(const T* __restrict__ u, const T* __restrict__ v, C2<T>* vis, int nd, double dra,
                                   double ddec) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += gridDim.x * blockDim.x) {
        T s, c;
        sincos2pi<T>((double)u[i] * dra + (double)v[i] * ddec, &s, &c);
        vis[i] = cmul(vis[i], C2<T>{c, s});
    }
}

// (reference uv_rotate_core :955-960)
template <typename T>
__global__ void rotate_kernel(const T* __restrict__ u, const T* __restrict__ v, T* urot, T* vrot, int nd, double c,
                              double s) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += gridDim.x * blockDim.x) {
        const double a = (double)u[i], b = (double)v[i];
        urot[i] = (T)(a * c - b * s);
        vrot[i] = (T)(a * s + b * c);
    }
}

// chi2 of given visibilities (reference reduce_chi2_d :1481-1502), FP64 accumulation
template <typename T>
__global__ void __launch_bounds__(256) reduce_kernel(const T* __restrict__ re, const T* __restrict__ im,
                                                     const C2<T>* __restrict__ vis, const T* __restrict__ w, int nd,
                                                     double* partials, DevState* st) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += gridDim.x * blockDim.x) {
        const C2<T> z = vis[i];
        const double dr = (double)z.x - (double)re[i], di = (double)z.y - (double)im[i];
        acc += (double)w[i] * (dr * dr + di * di);
    }
    const double tot = block_sum(acc, sh);
    grid_finish(tot, partials, st);
}

// standalone sweep into the padded buffer (the buffer is zeroed by the caller)
template <typename T>
__global__ void sweep_image_kernel(const T* __restrict__ intensity, int nr, T Rmin, T dR, T dxy, T inv_cos_inc,
                                   int rmax, T central, int N, T* padded) {
    const long long rowsize = 2LL * (N / 2 + 1);
    const int off = N / 2 - rmax;
    const int side = 2 * rmax;
    const T sr_to_px = dxy * dxy;
    const long long total = (long long)side * side;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / side), j = (int)(e % side);
        const int I = i + off, J = j + off;
        T val = sweep_pixel<T>(I, J, intensity, nr, Rmin, dR, dxy, inv_cos_inc, rmax, off, sr_to_px);
        if (I == N / 2 && J == N / 2) val = central;
        padded[I * rowsize + J] = val;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && side == 0) padded[(long long)(N / 2) * rowsize + N / 2] = central;
}

template <typename T> int max_fft_n_impl() { return sizeof(T) == 8 ? 8192 : 16384; }

// dispatch helper: launch a shared-memory FFT kernel with E elements per thread
template <typename T> struct FftCfg {
    int E, threads;
    size_t smem;
};
template <typename T> FftCfg<T> fft_cfg(int M) {
    FftCfg<T> c;
    if (M >= 16384) c.E = 16;
    else if (M >= 8) c.E = 8;
    else c.E = M < 1 ? 1 : M;
    c.threads = M / c.E < 1 ? 1 : M / c.E;
    c.smem = sizeof(C2<T>) * (size_t)(M < 1 ? 1 : M);
    return c;
}

template <typename K> cudaError_t set_smem(K kernel, size_t smem) {
    if (smem > 48 * 1024) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return cudaSuccess;
}

}  // namespace

int num_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// ===========================================================================
// launchers
// ===========================================================================
template <typename T> int Launch<T>::max_fft_n() { return max_fft_n_impl<T>(); }

template <typename T>
cudaError_t Launch<T>::extent(const T* u, const T* v, int nd, DevState* state, cudaStream_t s) {
    if (nd <= 0) return cudaSuccess;
    int blocks = (nd + 255) / 256;
    const int cap = num_sms() * 8;
    if (blocks > cap) blocks = cap;
    extent_kernel<T><<<blocks, 256, 0, s>>>(u, v, nd, state);
    return cudaGetLastError();
}

#define GBG_DISPATCH_E(E_, ...)                                   \
    switch (E_) {                                                 \
        case 1: { constexpr int EE = 1; __VA_ARGS__; } break;     \
        case 2: { constexpr int EE = 2; __VA_ARGS__; } break;     \
        case 4: { constexpr int EE = 4; __VA_ARGS__; } break;     \
        case 8: { constexpr int EE = 8; __VA_ARGS__; } break;     \
        case 16: { constexpr int EE = 16; __VA_ARGS__; } break;   \
        default: return cudaErrorInvalidValue;                    \
    }

template <typename T>
cudaError_t Launch<T>::rows_image(const T* image, int N, const CT* tw, CT* zt, int host_K, const DevState* state,
                                  double duv, bool row_sign, cudaStream_t s) {
    if (is_pow2(N) && N <= max_fft_n_impl<T>() * 2) {
        const int M = N / 2;
        FftCfg<T> c = fft_cfg<T>(M);
        cudaError_t e = cudaSuccess;
        GBG_DISPATCH_E(c.E, {
            auto kern = rows_image_kernel<T, EE>;
            e = set_smem(kern, c.smem);
            if (e == cudaSuccess) {
                kern<<<N, c.threads, c.smem, s>>>(image, N, tw, zt, host_K, state, duv, row_sign ? 1 : 0);
                e = cudaGetLastError();
            }
        });
        return e;
    }
    const size_t sm = sizeof(T) * (size_t)N;
    cudaError_t e = set_smem(rows_direct_kernel<T>, sm);
    if (e != cudaSuccess) return e;
    rows_direct_kernel<T><<<N, 256, sm, s>>>(image, N, 0, nullptr, 0, (T)0, (T)1, (T)1, (T)1, 0, (T)0, 0, tw, zt,
                                             host_K, state, duv, row_sign ? 1 : 0);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::rows_profile(const T* intensity, int nr, double Rmin, double dR, double dxy, double cos_inc,
                                    int rmax, double central_value, int N, const CT* tw, CT* zt,
                                    const DevState* state, double duv, cudaStream_t s) {
    const int nrows = 2 * rmax;
    if (nrows <= 0) return cudaSuccess;
    const T inv_cos = (T)(1.0 / cos_inc);
    if (is_pow2(N) && N <= max_fft_n_impl<T>() * 2) {
        const int M = N / 2;
        FftCfg<T> c = fft_cfg<T>(M);
        cudaError_t e = cudaSuccess;
        GBG_DISPATCH_E(c.E, {
            auto kern = rows_profile_kernel<T, EE>;
            e = set_smem(kern, c.smem);
            if (e == cudaSuccess) {
                kern<<<nrows, c.threads, c.smem, s>>>(intensity, nr, (T)Rmin, (T)dR, (T)dxy, inv_cos, rmax,
                                                      (T)central_value, N, tw, zt, state, duv);
                e = cudaGetLastError();
            }
        });
        return e;
    }
    const size_t sm = sizeof(T) * (size_t)N;
    cudaError_t e = set_smem(rows_direct_kernel<T>, sm);
    if (e != cudaSuccess) return e;
    rows_direct_kernel<T><<<nrows, 256, sm, s>>>(nullptr, N, N / 2 - rmax, intensity, nr, (T)Rmin, (T)dR, (T)dxy,
                                                 inv_cos, rmax, (T)central_value, 1, tw, zt, -1, state, duv, 1);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::cols(const CT* zt, int N, int band0, int band1, const CT* tw, CT* out, long long s_row,
                            long long s_col, int host_K, int host_r0, int host_W, const DevState* state, double duv,
                            bool out_sign, cudaStream_t s) {
    const int C = N / 2 + 1;
    const int grid = host_K >= 0 ? host_K : C;
    if (grid <= 0) return cudaSuccess;
    if (is_pow2(N) && N <= max_fft_n_impl<T>()) {
        FftCfg<T> c = fft_cfg<T>(N);
        cudaError_t e = cudaSuccess;
        GBG_DISPATCH_E(c.E, {
            auto kern = cols_kernel<T, EE>;
            e = set_smem(kern, c.smem);
            if (e == cudaSuccess) {
                kern<<<grid, c.threads, c.smem, s>>>(zt, N, band0, band1, tw, out, s_row, s_col, host_K, host_r0,
                                                     host_W, state, duv, out_sign ? 1 : 0);
                e = cudaGetLastError();
            }
        });
        return e;
    }
    const size_t sm = sizeof(CT) * (size_t)N;
    cudaError_t e = set_smem(cols_direct_kernel<T>, sm);
    if (e != cudaSuccess) return e;
    cols_direct_kernel<T><<<grid, 256, sm, s>>>(zt, N, band0, band1, tw, out, s_row, s_col, host_K, host_r0, host_W,
                                                state, duv, out_sign ? 1 : 0);
    return cudaGetLastError();
}

template <typename T> int Launch<T>::vis_grid(int nd) {
    int blocks = (nd + 255) / 256;
    const int cap = num_sms() * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return blocks;
}

template <typename T> cudaError_t Launch<T>::vis(const VisArgs& a, cudaStream_t s) {
    const int blocks = vis_grid(a.nd);
    const bool chi2 = a.partials != nullptr, vo = a.vis_out != nullptr;
    if (chi2 && vo) vis_kernel<T, true, true><<<blocks, 256, 0, s>>>(a);
    else if (chi2) vis_kernel<T, true, false><<<blocks, 256, 0, s>>>(a);
    else if (vo) vis_kernel<T, false, true><<<blocks, 256, 0, s>>>(a);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

static int grid_1d(long long n) {
    long long b = (n + 255) / 256;
    const long long cap = (long long)num_sms() * 16;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

template <typename T> cudaError_t Launch<T>::fftshift_real(T* padded, int N, cudaStream_t s) {
    fftshift_real_kernel<T><<<grid_1d((long long)(N / 2) * (N / 2)), 256, 0, s>>>(padded, N);
    return cudaGetLastError();
}
template <typename T> cudaError_t Launch<T>::fftshift_axis0(CT* m, int nrow, int ncol, cudaStream_t s) {
    fftshift_axis0_kernel<CT><<<grid_1d((long long)(nrow / 2) * ncol), 256, 0, s>>>(m, nrow, ncol);
    return cudaGetLastError();
}
template <typename T>
cudaError_t Launch<T>::apply_phase(const T* u, const T* v, CT* vis, int nd, double dra, double ddec, cudaStream_t s) {
    if (nd <= 0) return cudaSuccess;
    apply_phase_kernel<T><<<grid_1d(nd), 256, 0, s>>>(u, v, vis, nd, dra, ddec);
    return cudaGetLastError();
}
template <typename T>
cudaError_t Launch<T>::rotate(const T* u, const T* v, T* urot, T* vrot, int nd, double c, double sn, cudaStream_t s) {
    if (nd <= 0) return cudaSuccess;
    rotate_kernel<T><<<grid_1d(nd), 256, 0, s>>>(u, v, urot, vrot, nd, c, sn);
    return cudaGetLastError();
}
template <typename T>
cudaError_t Launch<T>::reduce(const T* re, const T* im, const CT* vis, const T* w, int nd, double* partials,
                              DevState* state, cudaStream_t s) {
    reduce_kernel<T><<<vis_grid(nd), 256, 0, s>>>(re, im, vis, w, nd, partials, state);
    return cudaGetLastError();
}
template <typename T>
cudaError_t Launch<T>::sweep_image(const T* intensity, int nr, double Rmin, double dR, double dxy, double cos_inc,
                                   int rmax, double central_value, int N, T* padded, cudaStream_t s) {
    sweep_image_kernel<T><<<grid_1d(4LL * rmax * rmax), 256, 0, s>>>(intensity, nr, (T)Rmin, (T)dR, (T)dxy,
                                                                     (T)(1.0 / cos_inc), rmax, (T)central_value, N,
                                                                     padded);
    return cudaGetLastError();
}

template struct Launch<double>;
template struct Launch<float>;

}  // namespace gbg
