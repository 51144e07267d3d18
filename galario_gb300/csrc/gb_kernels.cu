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

// modulus sqrt(re^2 + im^2) (the reference uses cuCabs / std::abs, :806-809)
template <typename T> __device__ __forceinline__ T cabs_(C2<T> a);
template <> __device__ __forceinline__ double cabs_<double>(double2 a) { return sqrt(fma(a.x, a.x, a.y * a.y)); }
template <> __device__ __forceinline__ float cabs_<float>(float2 a) { return sqrtf(fmaf(a.x, a.x, a.y * a.y)); }

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

// the spectrum window: given by the host (host_K >= 0) or written by the extent pass
__device__ __forceinline__ Window get_window(int host_K, int host_r0, int host_W, const DevState* __restrict__ st) {
    Window w;
    if (host_K >= 0) {
        w.K = host_K;
        w.r0 = host_r0;
        w.W = host_W;
    } else {
        w.K = st->win_K;
        w.r0 = st->win_r0;
        w.W = st->win_W;
    }
    return w;
}

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
    const int K = get_window(host_K, 0, 0, st).K;
    const T sgn = (row_sign && (i & 1)) ? (T)-1 : (T)1;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        CT x = real_split<T>(buf, M, k, tw);
        zt[(size_t)k * N + i] = CT{sgn * x.x, sgn * x.y};
    }
}

// Float rounding without conversion instructions.  On GB300 the
// float<->int conversions and FRND share the slow FP64 pipe, so the FP32 path
// rounds with the magic-number method: for |x| < 2^22, x + 1.5*2^23 lands in
// [2^23, 2^24) where the float spacing is 1, so the addition rounds x to the
// nearest integer and the low mantissa bits hold that integer.
constexpr float kMagic = 12582912.0f;   // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;  // bit pattern of kMagic
__device__ __forceinline__ int rint_i(float x, float* xr) {  // |x| < 2^22
    const float r = __fadd_rn(x, kMagic);
    *xr = __fsub_rn(r, kMagic);
    return __float_as_int(r) - kMagicBits;
}
__device__ __forceinline__ int floor_i(float x, float* xf) {  // |x| < 2^22
    float f;
    int n = rint_i(x, &f);
    if (f > x) {
        n -= 1;
        f = __fsub_rn(f, 1.f);
    }
    *xf = f;
    return n;
}
__device__ __forceinline__ float i2f_small(int n) {  // exact for |n| < 2^22
    return __fsub_rn(__int_as_float(kMagicBits + n), kMagic);
}

// sweep of a radial profile (reference sweep_core, src/galario.cpp:1048-1071)
// evaluated for image pixel (I, J); zero outside the 2*rmax box.  The
// reference's divisions by cos(inc) and dR are multiplications by host-computed
// reciprocals here (a rounding-level change: the linear interpolation is
// continuous across the bin edges where floor() could flip).
template <typename T>
__device__ __forceinline__ T sweep_pixel(int I, int J, const T* __restrict__ intensity, int nr, T Rmin, T dR, T inv_dR,
                                         T dxy, T inv_cos_inc, int rmax, int off, T sr_to_px) {
    const int i = I - off, j = J - off;
    if (i < 0 || j < 0 || i >= 2 * rmax || j >= 2 * rmax) return (T)0;
    if constexpr (sizeof(T) == 4) {
        // FP32: int<->float conversions and floor without the conversion pipe
        const float x = i2f_small(rmax - j) * dxy;
        const float y = i2f_small(rmax - i) * dxy;
        const float xs = x * inv_cos_inc;
        const float r = sqrtf(xs * xs + y * y);
        const float tR = (r - Rmin) * inv_dR;
        if (!(tR < (float)(nr - 1))) return 0.f;  // floor(tR) > nr - 2
        int iR = 0;
        if (tR > 0.f) {
            float fl;
            iR = floor_i(tR, &fl);
        }
        const float I0 = __ldg(&intensity[iR]), I1 = __ldg(&intensity[iR + 1]);
        return sr_to_px * (I0 + (r - i2f_small(iR) * dR - Rmin) * ((I1 - I0) * inv_dR));
    } else {
        const T x = (T)(rmax - j) * dxy;
        const T y = (T)(rmax - i) * dxy;
        const T xs = x * inv_cos_inc;
        const T r = sqrt(xs * xs + y * y);
        int iR = (int)floor((r - Rmin) * inv_dR);
        if (iR < 0) iR = 0;
        if (iR > nr - 2) return (T)0;
        const T I0 = __ldg(&intensity[iR]), I1 = __ldg(&intensity[iR + 1]);
        return sr_to_px * (I0 + (r - (T)iR * dR - Rmin) * ((I1 - I0) * inv_dR));
    }
}

template <typename T, int E>
__global__ void __launch_bounds__(1024) rows_profile_kernel(const T* __restrict__ intensity, int nr, T Rmin, T dR,
                                                            T inv_dR, T dxy, T inv_cos_inc, int rmax, T central, int N,
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
        T a = sweep_pixel<T>(I, J0, intensity, nr, Rmin, dR, inv_dR, dxy, inv_cos_inc, rmax, off, sr_to_px);
        T b = sweep_pixel<T>(I, J1, intensity, nr, Rmin, dR, inv_dR, dxy, inv_cos_inc, rmax, off, sr_to_px);
        if (I == N / 2) {  // reference central_pixel_d :1075-1079
            if (J0 == N / 2) a = central;
            if (J1 == N / 2) b = central;
        }
        buf[m] = CT{a, b};
    }
    __syncthreads();
    block_fft<T, E>(buf, M, ilog2(M), tw, 2);
    const int K = st->win_K;
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
                                                    T* __restrict__ amp_out, long long s_row, long long s_col,
                                                    int host_K, int host_r0,
                                                    int host_W, const DevState* __restrict__ st, double duv,
                                                    int out_sign) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT* buf = reinterpret_cast<CT*>(smem_raw);
    const Window w = get_window(host_K, host_r0, host_W, st);
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
        const long long o = (long long)q * s_row + (long long)k * s_col;
        out[o] = x;
        if (amp_out) amp_out[o] = cabs_<T>(x);
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
            x = sweep_pixel<T>(I, J, intensity, nr, Rmin, dR, (T)1 / dR, dxy, inv_cos_inc, rmax, off, sr_to_px);
            if (I == N / 2 && J == N / 2) x = central;
        } else {
            x = image[(size_t)I * N + J];
        }
        row[J] = x;
    }
    __syncthreads();
    const int K = get_window(host_K, 0, 0, st).K;
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
                                   const C2<T>* __restrict__ tw, C2<T>* __restrict__ out, T* __restrict__ amp_out,
                                   long long s_row, long long s_col, int host_K, int host_r0, int host_W,
                                   const DevState* __restrict__ st, double duv, int out_sign) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT* col = reinterpret_cast<CT*>(smem_raw);
    const Window w = get_window(host_K, host_r0, host_W, st);
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
        const long long o = (long long)q * s_row + (long long)k * s_col;
        out[o] = x;
        if (amp_out) amp_out[o] = cabs_<T>(x);
    }
}

// ---------------------------------------------------------------------------
// dataset extent
// ---------------------------------------------------------------------------
template <typename T>
__global__ void extent_kernel(const T* __restrict__ u, const T* __restrict__ v, int nd, int N, double duv,
                              DevState* st) {
    // max(u^2 + v^2) in the input precision (NaN entries are ignored here and
    // flagged by the visibility pass); the window adds a relative margin
    // larger than the float rounding of this maximum
    T mt = (T)0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += gridDim.x * blockDim.x) {
        const T a = __ldg(&u[i]), b = __ldg(&v[i]);
        mt = fmax(mt, a * a + b * b);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mt = fmax(mt, __shfl_xor_sync(0xffffffffu, mt, o));
    double m = (double)mt;
    __shared__ double sh[32];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) m = fmax(m, sh[q]);
        if (m > 0.0)
            atomicMax(reinterpret_cast<unsigned long long*>(&st->rmax2), (unsigned long long)__double_as_longlong(m));
        __threadfence();
        const unsigned t = atomicAdd(&st->ticket_extent, 1u);
        if (t == gridDim.x - 1) {  // last block: derive the window once for every later kernel
            __threadfence();
            const double r2 = *((volatile double*)&st->rmax2);
            const Window w = window_from_extent(r2, duv, N);
            st->win_K = w.K;
            st->win_r0 = w.r0;
            st->win_W = w.W;
            st->ticket_extent = 0u;
        }
    }
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
// to arrive sums the partials with all its threads: thread i takes partials
// i, i + blockDim, ... in order, then a fixed-shape tree (block_sum).  The
// summation order depends only on the grid size, so results are reproducible.
__device__ __forceinline__ void grid_finish(double block_total, double* partials, DevState* st,
                                            double* extra_out = nullptr) {
    __shared__ bool last;
    __shared__ double sh2[32];
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = block_total;
        __threadfence();
        const unsigned t = atomicAdd(&st->ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s = 0.0;
    const volatile double* p = partials;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) s += p[b];
    s = block_sum(s, sh2);
    if (threadIdx.x == 0) {
        st->chi2 = s;
        if (extra_out) *extra_out = s;
        st->ticket = 0u;
    }
}

// ---------------------------------------------------------------------------
// double-float arithmetic for the FP32 path: a value is hi + lo with two
// floats (about 44 significant bits).  Error-free transformations of Dekker
// (1971) and Knuth (TAOCP vol. 2, 4.2.2): two_prod via fused multiply-add,
// two_sum by Knuth's six-operation form.  Intrinsics (_rn) keep the compiler
// from contracting or reassociating them.
// ---------------------------------------------------------------------------
__device__ __forceinline__ DF df_two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return DF{p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ DF df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ DF df_renorm(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.hi, -a.lo}; }
__device__ __forceinline__ DF df_mul_f(float x, DF y) {  // exact float x times y
    DF p = df_two_prod(x, y.hi);
    return df_renorm(p.hi, __fmaf_rn(x, y.lo, p.lo));
}
__device__ __forceinline__ DF df_mul(DF x, DF y) {
    DF p = df_two_prod(x.hi, y.hi);
    return df_renorm(p.hi, __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, p.lo)));
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
    DF s = df_two_sum(a.hi, b.hi);
    return df_renorm(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
// floor of x = hi + lo (|hi| < 2^22) as an integer and the fraction in [0, 1]
__device__ __forceinline__ void df_floor(DF x, int* fl, float* frac) {
    float f;
    int n = floor_i(x.hi, &f);
    float r = __fadd_rn(__fsub_rn(x.hi, f), x.lo);  // hi - floor(hi) is exact
    if (r < 0.f) {
        n -= 1;
        r = __fadd_rn(r, 1.f);
    } else if (r >= 1.f) {
        n += 1;
        r = __fsub_rn(r, 1.f);
    }
    *fl = n;
    *frac = r;
}

// sin/cos(2 pi f) in FP32 for |f| <= 1/2 + tiny, without conversion
// instructions: j = rint(4 f), d = f - j/4 (exact by Sterbenz), x = 2 pi d with
// |x| <= pi/4, Taylor series to x^9 (sin) and x^8 (cos), truncation error
// below 3e-8, then rotation by i^j.
__device__ __forceinline__ void sincos2pi_f32(float f, float* s, float* c) {
    float jf;
    const int j = rint_i(4.f * f, &jf);
    const float d = __fmaf_rn(jf, -0.25f, f);
    const float x = d * 6.28318530717958647692f;
    const float x2 = x * x;
    float sp = __fmaf_rn(x2, 2.7557319e-6f, -1.9841270e-4f);  // 1/9!, -1/7!
    sp = __fmaf_rn(x2, sp, 8.3333333e-3f);                     // 1/5!
    sp = __fmaf_rn(x2, sp, -1.6666667e-1f);                    // -1/3!
    const float sx = __fmaf_rn(x * x2, sp, x);
    float cp = __fmaf_rn(x2, 2.4801587e-5f, -1.3888889e-3f);  // 1/8!, -1/6!
    cp = __fmaf_rn(x2, cp, 4.1666667e-2f);                     // 1/4!
    cp = __fmaf_rn(x2, cp, -0.5f);
    const float cx = __fmaf_rn(x2, cp, 1.f);
    switch (j & 3) {  // multiply by i^j
        case 0: *s = sx; *c = cx; break;
        case 1: *s = cx; *c = -sx; break;
        case 2: *s = -sx; *c = -cx; break;
        default: *s = -cx; *c = sx; break;
    }
}

// ---------------------------------------------------------------------------
// fused visibility kernel
// reference: uv_rotate_core :955-960, interpolate_core :749-815,
//            apply_phase_sampled_core :877-884, diff_weighted_core :1453-1461
// ---------------------------------------------------------------------------
// sin/cos(2 pi a), a in cycles, FP64, table-driven (Tang's method): a = n +
// j/T + d with n integer, j in [-T/2, T/2], |d| <= 1/(2T); exp(2 pi i a) =
// E[j] * exp(2 pi i d) with the table E built on the host in long double and
// exp(2 pi i d) from its Taylor series: x = 2 pi d, |x| <= pi/T = 3.1e-3, so
// cos x = 1 - x^2/2 + x^4/24 and sin x = x - x^3/6 + x^5/120 are exact to
// < 1e-17 (the next terms x^6/720 and x^7/5040 are below 1.3e-18).
__device__ __forceinline__ void sincos2pi_tab(double a, const double2* __restrict__ tab, double* s, double* c) {
    const double f = a - rint(a);                         // exact, |f| <= 1/2
    const double jf = rint(f * (double)PHASE_T);          // f*T exact (power of two)
    const double d = fma(jf, -1.0 / (double)PHASE_T, f);  // exact
    const double x = d * 6.283185307179586476925286766559;
    const double x2 = x * x;
    const double cx = fma(x2, fma(x2, 1.0 / 24.0, -0.5), 1.0);
    const double sx = fma(x * x2, fma(x2, 1.0 / 120.0, -1.0 / 6.0), x);
    const double2 e = __ldg(&tab[(int)jf + PHASE_T / 2]);
    *c = e.x * cx - e.y * sx;
    *s = e.x * sx + e.y * cx;
}
// FP32 phase: argument in FP64 with exact range reduction, evaluated in FP32
template <typename T> __device__ __forceinline__ void sincos2pi(double a, T* s, T* c);
template <> __device__ __forceinline__ void sincos2pi<double>(double a, double* s, double* c) {
    sincospi(2.0 * a, s, c);
}
template <> __device__ __forceinline__ void sincos2pi<float>(double a, float* s, float* c) {
    const double f = a - rint(a);
    sincospif((float)(2.0 * f), s, c);
}
template <typename T> __device__ __forceinline__ T rnorm2(T x, T y);
template <> __device__ __forceinline__ double rnorm2<double>(double x, double y) { return rsqrt(fma(x, x, y * y)); }
template <> __device__ __forceinline__ float rnorm2<float>(float x, float y) { return rsqrtf(fmaf(x, x, y * y)); }

// Bilinear amplitude/phase interpolation at cell (fu, fv) with fractions
// (q, t) along u and v (reference interpolate_core :749-815).  Corners follow
// the reference's flat-index semantics of the row-major N x C spectrum
// (:774-780): a corner past the last column continues on the next row.
// Returns false (and sets err bits) when a corner is outside the spectrum.
template <typename T>
__device__ __forceinline__ bool interp_cell(const typename Launch<T>::VisArgs& a, const Window& w, int fu, int fv,
                                            T q, T t, T sign_u, C2<T>* out, unsigned* err) {
    using CT = C2<T>;
    const int C = a.ncol;
    int r0 = fv, c0 = fu;
    while (c0 >= C) {  // flat-index continuation on the next row; fu < 4N bounds the loop
        c0 -= C;
        r0 += 1;
    }
    const bool wrap = (c0 + 1 == C);
    const int r_last = wrap ? r0 + 2 : r0 + 1;
    if (r0 < 0 || r_last >= a.nrow) {
        *err |= ERR_UV_OUTSIDE;
        return false;
    }
    CT y[4];
    T am[4];
    const int qq = r0 - w.r0;
    if (a.quads && (long long)w.K * w.W <= a.quad_cap) {
        // one cell record: corners and moduli in 3 (FP32) or 6 (FP64) 16-byte loads
        const bool inside = wrap ? (w.K == C && qq >= 0 && qq < w.W - 2) : (c0 < w.K - 1 && qq >= 0 && qq < w.W - 1);
        if (!inside) {
            *err |= ERR_WINDOW;
            return false;
        }
        const T* rec = a.quads + ((long long)c0 * w.W + qq) * QUAD_REC;
        if constexpr (sizeof(T) == 4) {
            const float4 p0 = __ldg(reinterpret_cast<const float4*>(rec));
            const float4 p1 = __ldg(reinterpret_cast<const float4*>(rec) + 1);
            const float4 p2 = __ldg(reinterpret_cast<const float4*>(rec) + 2);
            y[0] = CT{p0.x, p0.y};
            y[1] = CT{p0.z, p0.w};
            y[2] = CT{p1.x, p1.y};
            y[3] = CT{p1.z, p1.w};
            am[0] = p2.x;
            am[1] = p2.y;
            am[2] = p2.z;
            am[3] = p2.w;
        } else {
            const double2* r2 = reinterpret_cast<const double2*>(rec);
#pragma unroll
            for (int c = 0; c < 4; ++c) y[c] = __ldg(&r2[c]);
            const double2 m0 = __ldg(&r2[4]), m1 = __ldg(&r2[5]);
            am[0] = m0.x;
            am[1] = m0.y;
            am[2] = m1.x;
            am[3] = m1.y;
        }
    } else {
        const int rr[4] = {r0, r0 + 1, r_last, wrap ? r0 + 1 : r0};
        const int cc[4] = {c0, c0, wrap ? 0 : c0 + 1, wrap ? 0 : c0 + 1};
        bool ok = true;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int qc = rr[c] - w.r0;
            if (cc[c] >= w.K || qc < 0 || qc >= w.W) {
                ok = false;
                y[c] = CT{(T)0, (T)0};
                am[c] = (T)0;
            } else {
                const long long o = (long long)qc * a.s_row + (long long)cc[c] * a.s_col;
                y[c] = __ldg(&a.spec[o]);
                am[c] = a.amp ? __ldg(&a.amp[o]) : cabs_<T>(y[c]);
            }
        }
        if (!ok) {
            *err |= ERR_WINDOW;
            return false;
        }
    }
    // complex bilinear (:782-800): t*q*(y0-y1+y2-y3) + t*(y1-y0) + q*(y3-y0) + y0
    const T d1r = (y[0].x + y[2].x) - (y[1].x + y[3].x);
    const T d1i = (y[0].y + y[2].y) - (y[1].y + y[3].y);
    const T zr = t * (q * d1r) + (t * (y[1].x - y[0].x) + q * (y[3].x - y[0].x)) + y[0].x;
    const T zi = t * (q * d1i) + (t * (y[1].y - y[0].y) + q * (y[3].y - y[0].y)) + y[0].y;
    // bilinear of the corner amplitudes (:804-812)
    T amp = am[0];
    amp += (am[3] - am[0]) * q;
    amp += (am[1] - am[0]) * t;
    amp += (am[0] - am[1] + am[2] - am[3]) * t * q;
    // amp * exp(i sign_u arg z) without atan2: (zr, sign_u * zi) / |z|
    T cph = (T)1, sph = (T)0;
    if (zr != (T)0 || zi != (T)0) {
        const T rn = rnorm2<T>(zr, zi);
        cph = zr * rn;
        sph = sign_u * zi * rn;
    }
    *out = CT{amp * cph, amp * sph};
    return true;
}

// One visibility: rotation, index, interpolation and phase shift.
template <typename T>
__device__ __forceinline__ C2<T> vis_point(const typename Launch<T>::VisArgs& a, const Window& w, T u_in, T v_in,
                                           unsigned* e) {
    using CT = C2<T>;
    CT out = CT{(T)0, (T)0};
    if constexpr (sizeof(T) == 8) {
        // FP64: index and phase in double, as the reference's double build
        double ur = u_in, vr = v_in;
        if (a.rotate) {
            ur = u_in * a.cos_pa - v_in * a.sin_pa;
            vr = u_in * a.sin_pa + v_in * a.cos_pa;
        }
        if (!(isfinite(ur) && isfinite(vr))) {
            *e = ERR_UV_NONFINITE;
            return out;
        }
        const double indu = fabs(ur) * a.inv_duv;
        const double sign_u = copysign(1.0, ur);
        const double indv = a.half_nrow + a.v_origin * sign_u * vr * a.inv_duv;
        if (!(indu < 4.0 * a.nrow && indv > -4.0 * a.nrow && indv < 4.0 * a.nrow)) {
            *e = ERR_UV_OUTSIDE;
            return out;
        }
        const double fu = floor(indu), fv = floor(indv);
        if (interp_cell<T>(a, w, (int)fu, (int)fv, (T)(indu - fu), (T)(indv - fv), (T)sign_u, &out, e) && a.phase) {
            double sn, cs;
            sincos2pi_tab(ur * a.dra + vr * a.ddec, a.phase_tab, &sn, &cs);
            out = cmul(out, CT{(T)cs, (T)sn});
        }
    } else {
        // FP32: index and phase argument in double-float, no FP64 instruction
        const float u = u_in, v = v_in;
        if (!(isfinite(u) && isfinite(v))) {
            *e = ERR_UV_NONFINITE;
            return out;
        }
        DF ur = DF{u, 0.f}, vr = DF{v, 0.f};
        if (a.rotate) {
            ur = df_add(df_mul_f(u, a.cpa), df_neg(df_mul_f(v, a.spa)));
            vr = df_add(df_mul_f(u, a.spa), df_mul_f(v, a.cpa));
        }
        const float sign_u = copysignf(1.f, ur.hi);
        const DF au = ur.hi < 0.f ? df_neg(ur) : ur;
        const DF indu = df_mul(au, a.inv_duv_df);
        const DF sv = (a.v_origin_f * sign_u < 0.f) ? df_neg(vr) : vr;
        const DF indv = df_add(DF{a.half_nrow_f, 0.f}, df_mul(sv, a.inv_duv_df));
        const float lim = 4.f * a.half_nrow_f * 2.f;
        if (!(indu.hi < lim && indv.hi > -lim && indv.hi < lim)) {
            *e = ERR_UV_OUTSIDE;
            return out;
        }
        int fu, fv;
        float q, t;
        df_floor(indu, &fu, &q);
        df_floor(indv, &fv, &t);
        if (interp_cell<T>(a, w, fu, fv, (T)q, (T)t, (T)sign_u, &out, e) && a.phase) {
            const DF ph = df_add(df_mul(ur, a.dra_df), df_mul(vr, a.ddec_df));
            float n;
            if (fabsf(ph.hi) < 4194304.f) rint_i(ph.hi, &n);
            else n = rintf(ph.hi);  // |phase| >= 2^22 cycles: not reached for physical offsets
            const float f = __fadd_rn(__fsub_rn(ph.hi, n), ph.lo);  // cycles, |f| <= 1/2 + tiny
            float sn, cs;
            sincos2pi_f32(f, &sn, &cs);
            out = cmul(out, CT{(T)cs, (T)sn});
        }
    }
    return out;
}

// Grid-stride over the visibilities, two independent points per iteration so
// their load -> gather chains overlap.
template <typename T, bool CHI2, bool VISOUT>
__global__ void __launch_bounds__(256) vis_kernel(typename Launch<T>::VisArgs a) {
    using CT = C2<T>;
    __shared__ double sh[32];
    const Window w = get_window(a.host_K, a.host_r0, a.host_W, a.state);
    T acc = (T)0;
    unsigned err = 0u;
    long long err_idx = -1;
    const int stride = gridDim.x * blockDim.x;
    for (int i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < a.nd; i0 += 2 * stride) {
        const int i1 = i0 + stride;
        const bool has1 = i1 < a.nd;
        const T u0 = __ldg(&a.u[i0]), v0 = __ldg(&a.v[i0]);
        const T u1 = has1 ? __ldg(&a.u[i1]) : (T)0, v1 = has1 ? __ldg(&a.v[i1]) : (T)0;
        T re0 = (T)0, im0 = (T)0, w0 = (T)0, re1 = (T)0, im1 = (T)0, w1 = (T)0;
        if (CHI2) {
            re0 = __ldg(&a.re[i0]);
            im0 = __ldg(&a.im[i0]);
            w0 = __ldg(&a.w[i0]);
            if (has1) {
                re1 = __ldg(&a.re[i1]);
                im1 = __ldg(&a.im[i1]);
                w1 = __ldg(&a.w[i1]);
            }
        }
        unsigned e0 = 0u, e1 = 0u;
        const CT o0 = vis_point<T>(a, w, u0, v0, &e0);
        const CT o1 = has1 ? vis_point<T>(a, w, u1, v1, &e1) : CT{(T)0, (T)0};
        if (e0 | e1) {
            err |= e0 | e1;
            if (err_idx < 0) err_idx = e0 ? i0 : i1;
        }
        if (VISOUT) {
            a.vis_out[i0] = o0;
            if (has1) a.vis_out[i1] = o1;
        }
        if (CHI2) {
            const T dr0 = o0.x - re0, di0 = o0.y - im0;
            const T dr1 = o1.x - re1, di1 = o1.y - im1;
            acc += w0 * (dr0 * dr0 + di0 * di0);
            acc += w1 * (dr1 * dr1 + di1 * di1);  // w1 == 0 when i1 is past the end
        }
    }
    if (err) {
        atomicOr(&a.state->err, err);
        atomicCAS(&a.state->err_index, 0ull, (unsigned long long)(err_idx + 1));
    }
    if (CHI2) {
        const double tot = block_sum((double)acc, sh);
        grid_finish(tot, a.partials, a.state, a.chi2_out);
    }
}

// cell-major records for the visibility gather (see Launch::quads)
template <typename T>
__global__ void quad_kernel(const C2<T>* __restrict__ spec, const T* __restrict__ amp, long long s_row,
                            long long s_col, int C, const DevState* __restrict__ st, T* __restrict__ quads,
                            long long cap, int host_K, int host_r0, int host_W) {
    const Window w = get_window(host_K, host_r0, host_W, st);
    const long long ncell = (long long)w.K * w.W;
    if (ncell > cap) return;  // the visibility pass gathers from spec/amp instead
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ncell;
         e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e / w.W), q = (int)(e - (long long)k * w.W);
        const bool wrap = (k + 1 == C);
        const int rr[4] = {q, q + 1, wrap ? q + 2 : q + 1, wrap ? q + 1 : q};
        const int cc[4] = {k, k, wrap ? 0 : k + 1, wrap ? 0 : k + 1};
        bool ok = true;
#pragma unroll
        for (int c = 0; c < 4; ++c) ok = ok && rr[c] < w.W && cc[c] < w.K;
        if (!ok) continue;
        T* rec = quads + e * QUAD_REC;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const long long o = (long long)rr[c] * s_row + (long long)cc[c] * s_col;
            const C2<T> y = spec[o];
            rec[2 * c] = y.x;
            rec[2 * c + 1] = y.y;
            rec[8 + c] = amp[o];
        }
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
        T val = sweep_pixel<T>(I, J, intensity, nr, Rmin, dR, (T)1 / dR, dxy, inv_cos_inc, rmax, off, sr_to_px);
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
cudaError_t Launch<T>::extent(const T* u, const T* v, int nd, int N, double duv, DevState* state, cudaStream_t s) {
    int blocks = (nd + 255) / 256;
    const int cap = num_sms() * 4;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    extent_kernel<T><<<blocks, 256, 0, s>>>(u, v, nd, N, duv, state);
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
                kern<<<nrows, c.threads, c.smem, s>>>(intensity, nr, (T)Rmin, (T)dR, (T)(1.0 / dR), (T)dxy,
                                                      inv_cos, rmax, (T)central_value, N, tw, zt, state, duv);
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
cudaError_t Launch<T>::cols(const CT* zt, int N, int band0, int band1, const CT* tw, CT* out, T* amp_out,
                            long long s_row, long long s_col, int host_K, int host_r0, int host_W,
                            const DevState* state, double duv, bool out_sign, cudaStream_t s) {
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
                kern<<<grid, c.threads, c.smem, s>>>(zt, N, band0, band1, tw, out, amp_out, s_row, s_col, host_K,
                                                     host_r0, host_W, state, duv, out_sign ? 1 : 0);
                e = cudaGetLastError();
            }
        });
        return e;
    }
    const size_t sm = sizeof(CT) * (size_t)N;
    cudaError_t e = set_smem(cols_direct_kernel<T>, sm);
    if (e != cudaSuccess) return e;
    cols_direct_kernel<T><<<grid, 256, sm, s>>>(zt, N, band0, band1, tw, out, amp_out, s_row, s_col, host_K, host_r0,
                                                host_W, state, duv, out_sign ? 1 : 0);
    return cudaGetLastError();
}

template <typename T> int Launch<T>::vis_grid(int nd) {
    int blocks = (nd + 255) / 256;
    const int cap = num_sms() * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return blocks;
}

template <typename T> cudaError_t Launch<T>::vis(const VisArgs& args, cudaStream_t s) {
    VisArgs a = args;
    a.finalize();
    const int blocks = vis_grid(a.nd);
    const bool chi2 = a.partials != nullptr, vo = a.vis_out != nullptr;
    if (chi2 && vo) vis_kernel<T, true, true><<<blocks, 256, 0, s>>>(a);
    else if (chi2) vis_kernel<T, true, false><<<blocks, 256, 0, s>>>(a);
    else if (vo) vis_kernel<T, false, true><<<blocks, 256, 0, s>>>(a);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::quads(const CT* spec, const T* amp, long long s_row, long long s_col, int C,
                             const DevState* state, T* q, long long cap, int host_K, int host_r0, int host_W,
                             cudaStream_t s) {
    quad_kernel<T><<<num_sms() * 4, 256, 0, s>>>(spec, amp, s_row, s_col, C, state, q, cap, host_K, host_r0,
                                                 host_W);
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
