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

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <mutex>
#include <type_traits>
#include <utility>
#include <vector>

#include "gb_device.cuh"
#include "gb_internal.cuh"
#include "gb_tc.cuh"

namespace gbg {

namespace {

// Launch on s; with pdl as a programmatic dependent of the stream's previous
// kernel (its CTAs may start while that kernel finishes; the kernel's
// griddepcontrol.wait precedes every read of the previous kernel's output).
template <typename... KArgs, typename... Args>
cudaError_t launch_on(void (*kern)(KArgs...), int grid, int block, cudaStream_t s, bool pdl, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

// ---------------------------------------------------------------------------
// row pass kernels
// ---------------------------------------------------------------------------
template <typename T, int E, int MAXT>
__global__ void __launch_bounds__(MAXT) rows_image_kernel(const T* __restrict__ image, int N, const C2<T>* __restrict__ tw,
                                                          const C2<T>* __restrict__ stw, C2<T>* __restrict__ zt,
                                                          int host_K,
                                                          const DevState* __restrict__ st, double duv, int row_sign) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT* buf = reinterpret_cast<CT*>(smem_raw);
    const int M = N / 2;
    const int i = blockIdx.x;
    const CT* row = reinterpret_cast<const CT*>(image + (size_t)i * N);
    for (int m = threadIdx.x; m < M; m += blockDim.x) buf[sp(m)] = __ldg(&row[m]);
    __syncthreads();
    block_fft<T, E>(buf, M, ilog2(M), stw);
    const int K = get_window(host_K, 0, 0, st).K;
    const T sgn = (row_sign && (i & 1)) ? (T)-1 : (T)1;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        CT x = real_split<T>(buf, M, k, tw);
        zt[(size_t)k * N + i] = CT{sgn * x.x, sgn * x.y};
    }
}

// FP32 image rows with the loads pipelined: persistent CTAs take the rows
// i = blockIdx.x, blockIdx.x + gridDim.x, ...; the next row is fetched by a 1D
// bulk copy (cp.async.bulk, completion counted on an mbarrier) into the other
// of two staging buffers while the current row is transformed, so HBM reads
// overlap the shared-memory FFT.  Needs N * 4 bytes a multiple of 16 and a
// 16-byte aligned image.  Waits are bounded: one that gives up sets ERR_SPIN,
// waits (bounded) for the copy it has in flight and ends the CTA.
template <int E, int MAXT>
__global__ void __launch_bounds__(MAXT) rows_image_tma_kernel(const float* __restrict__ image, int N,
                                                              const float2* __restrict__ tw,
                                                              const float2* __restrict__ stw,
                                                              float2* __restrict__ zt, int host_K, DevState* st,
                                                              int row_sign) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int M = N / 2;
    float* stg = reinterpret_cast<float*>(smem_raw);                  // [2][N]
    float2* buf = reinterpret_cast<float2*>(stg + 2 * (size_t)N);     // fft_slots(M)
    uint64_t* bar = reinterpret_cast<uint64_t*>(buf + fft_slots(M));  // [2]
    const uint32_t bytes = (uint32_t)N * 4u;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int K = get_window(host_K, 0, 0, st).K;
    int i = blockIdx.x;
    if (threadIdx.x == 0 && i < N) tc::bulk_load_1d(stg, image + (size_t)i * N, bytes, &bar[0]);
    for (int it = 0; i < N; ++it, i += gridDim.x) {
        const int cur = it & 1;
        const int nxt = i + gridDim.x;
        if (threadIdx.x == 0 && nxt < N) {
            // the other buffer was read through the generic proxy before the last barrier
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tc::bulk_load_1d(stg + (size_t)(cur ^ 1) * N, image + (size_t)nxt * N, bytes, &bar[cur ^ 1]);
        }
        const bool ok = tc::mbar_wait(&bar[cur], (uint32_t)((it >> 1) & 1));
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0) {
                atomicOr(&st->err, ERR_SPIN);
                if (nxt < N) (void)tc::mbar_wait(&bar[cur ^ 1], (uint32_t)(((it + 1) >> 1) & 1));
            }
            return;
        }
        const float2* row = reinterpret_cast<const float2*>(stg + (size_t)cur * N);
        for (int m = threadIdx.x; m < M; m += blockDim.x) buf[sp(m)] = row[m];
        __syncthreads();
        block_fft<float, E>(buf, M, ilog2(M), stw);
        const float sgn = (row_sign && (i & 1)) ? -1.f : 1.f;
        for (int k = threadIdx.x; k < K; k += blockDim.x) {
            const float2 x = real_split<float>(buf, M, k, tw);
            zt[(size_t)k * N + i] = make_float2(sgn * x.x, sgn * x.y);
        }
        __syncthreads();  // buf and this staging buffer are free again
    }
}

template <typename T, int E, int MAXT>
__global__ void __launch_bounds__(MAXT) rows_profile_kernel(const T* __restrict__ intensity, int nr, T Rmin, T dR,
                                                            T inv_dR, T dxy, T inv_cos_inc, int rmax, T central, int N,
                                                            const C2<T>* __restrict__ tw,
                                                            const C2<T>* __restrict__ stw, C2<T>* __restrict__ zt,
                                                            const DevState* __restrict__ st, double duv, int kcols) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT* buf = reinterpret_cast<CT*>(smem_raw);
    const int M = N / 2;
    const int off = N / 2 - rmax;
    // Block a transforms image row I = N/2 - a.  The swept image depends on
    // |y| only, so row N/2 + a (0 < a < rmax) holds the same pixels, and its
    // row sign (-1)^I has the same parity: the result is written to both.
    const int a_fold = blockIdx.x;
    const int I = off + rmax - a_fold;
    const bool mirror = a_fold > 0 && a_fold < rmax;
    const int I2 = off + rmax + a_fold;
    const T sr_to_px = dxy * dxy;
    for (int m = threadIdx.x; m < M; m += blockDim.x) {
        const int J0 = 2 * m, J1 = 2 * m + 1;
        T a = sweep_pixel<T>(I, J0, intensity, nr, Rmin, dR, inv_dR, dxy, inv_cos_inc, rmax, off, sr_to_px);
        T b = sweep_pixel<T>(I, J1, intensity, nr, Rmin, dR, inv_dR, dxy, inv_cos_inc, rmax, off, sr_to_px);
        if (I == N / 2) {  // reference central_pixel_d :1075-1079
            if (J0 == N / 2) a = central;
            if (J1 == N / 2) b = central;
        }
        buf[sp(m)] = CT{a, b};
    }
    __syncthreads();
    block_fft<T, E>(buf, M, ilog2(M), stw);
    const int K = kcols >= 0 ? kcols : st->win_K;
    const T sgn = (I & 1) ? (T)-1 : (T)1;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        CT x = real_split<T>(buf, M, k, tw);
        const CT y = CT{sgn * x.x, sgn * x.y};
        zt[(size_t)k * N + I] = y;
        if (mirror) zt[(size_t)k * N + I2] = y;
    }
}

// ---------------------------------------------------------------------------
// column pass
// ---------------------------------------------------------------------------
template <typename T, int E, int MAXT>
__global__ void __launch_bounds__(MAXT) cols_kernel(const C2<T>* __restrict__ zt, int N, int band0, int band1,
                                                    const C2<T>* __restrict__ stw, C2<T>* __restrict__ out,
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
        buf[sp(i)] = (i >= band0 && i < band1) ? __ldg(&col[i]) : CT{(T)0, (T)0};
    __syncthreads();
    block_fft<T, E>(buf, N, ilog2(N), stw);
    const int par = (k + N / 2) & 1;
    for (int q = threadIdx.x; q < w.W; q += blockDim.x) {
        const int r = w.r0 + q;
        CT x = buf[sp(r)];
        if (out_sign && ((r & 1) ^ par)) x = cneg(x);
        const long long o = (long long)q * s_row + (long long)k * s_col;
        out[o] = x;
        if (amp_out) amp_out[o] = cabs_<T>(x);
    }
}

// Column pass of a swept profile: the image is even in x and in y about its
// centre, so every row transform is real (x (-1)^k) and every column of zt is
// real and even about row N/2; its transform is real as well.  Two columns
// k1 = 2p, k2 = 2p + 1 are therefore transformed together as the real and the
// imaginary part of one complex column, and split after the transform:
// FFT(a + i b) = FFT(a) + i FFT(b) with both transforms real.  Half the
// column FFTs of cols_kernel.
template <typename T, int E, int MAXT>
__global__ void __launch_bounds__(MAXT) cols_pair_kernel(const C2<T>* __restrict__ zt, int N, int band0, int band1,
                                                         const C2<T>* __restrict__ stw, C2<T>* __restrict__ out,
                                                         T* __restrict__ amp_out, long long s_row, long long s_col,
                                                         const DevState* __restrict__ st) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT* buf = reinterpret_cast<CT*>(smem_raw);
    const Window w = get_window(-1, -1, -1, st);
    const int k1 = 2 * blockIdx.x, k2 = k1 + 1;
    if (k1 >= w.K) return;  // uniform for the whole block
    const bool two = k2 < w.K;
    const CT* c1 = zt + (size_t)k1 * N;
    const CT* c2 = zt + (size_t)k2 * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const bool in = i >= band0 && i < band1;
        buf[sp(i)] = CT{in ? __ldg(&c1[i]).x : (T)0, (in && two) ? __ldg(&c2[i]).x : (T)0};
    }
    __syncthreads();
    block_fft<T, E>(buf, N, ilog2(N), stw);
    const int par1 = (k1 + N / 2) & 1;
    for (int q = threadIdx.x; q < w.W; q += blockDim.x) {
        const int r = w.r0 + q;
        const CT x = buf[sp(r)];
        const T f1 = ((r & 1) ^ par1) ? -x.x : x.x;
        const long long o1 = (long long)q * s_row + (long long)k1 * s_col;
        out[o1] = CT{f1, (T)0};
        amp_out[o1] = fabs(f1);
        if (two) {  // k2 has the opposite output-sign parity
            const T f2 = ((r & 1) ^ par1) ? x.y : -x.y;
            const long long o2 = (long long)q * s_row + (long long)k2 * s_col;
            out[o2] = CT{f2, (T)0};
            amp_out[o2] = fabs(f2);
        }
    }
}

// ---------------------------------------------------------------------------
// Swept profiles as even sequences (even_dft_block): the swept image is even
// in x about column N/2 and in y about row N/2, so each image row and each
// spectrum column is a DCT-I of its half (n + 1 = N/2 + 1 values), computed
// with a complex FFT of length N/4 instead of N/2 (paired row transform) or
// N (paired column transform).  Shared memory: the FFT buffer, the half
// sequence (reused for the transform's output) and the Im Y scratch.
// ---------------------------------------------------------------------------
// Row pass: block a transforms image row I = N/2 - a (and its mirror N/2 + a):
// X[k] = sum_J x[J] exp(-2 pi i J k / N) = (-1)^k C_k, C the even transform
// of f(j) = sweep(|x| = j dxy), j in [0, n]; written times the row sign.
template <typename T, int E, int MAXT>
__global__ void __launch_bounds__(MAXT) rows_profile_dct_kernel(const T* __restrict__ intensity, int nr, T Rmin, T dR,
                                                                T inv_dR, T dxy, T inv_cos_inc, int rmax, T central,
                                                                int N, const C2<T>* __restrict__ tw,
                                                                const C2<T>* __restrict__ stw4, C2<T>* __restrict__ zt,
                                                                const DevState* __restrict__ st, int kcols) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = N / 2, M = N / 4;
    CT* buf = reinterpret_cast<CT*>(smem_raw);
    T* xs = reinterpret_cast<T*>(buf + fft_slots(M));  // n + 1 values, then the output C_k
    T* im = xs + (n + 1);
    const int off = N / 2 - rmax;
    const int a = blockIdx.x;
    const int I = N / 2 - a;
    const bool mirror = a > 0 && a < rmax;
    const int I2 = N / 2 + a;
    const T sr_to_px = dxy * dxy;
    const int nnz = rmax < n ? rmax : n;
    for (int j = threadIdx.x; j < nnz; j += blockDim.x) {
        T v = sweep_pixel<T>(I, N / 2 - j, intensity, nr, Rmin, dR, inv_dR, dxy, inv_cos_inc, rmax, off, sr_to_px);
        if (I == N / 2 && j == 0) v = central;  // reference central_pixel_d :1075-1079
        xs[j] = v;
    }
    // x_n: column 0 (x = n dxy) lies in the box only when rmax reaches n
    const T xn = rmax >= n ? sweep_pixel<T>(I, 0, intensity, nr, Rmin, dR, inv_dR, dxy, inv_cos_inc, rmax, off,
                                            sr_to_px)
                           : (T)0;
    __syncthreads();
    int K = kcols >= 0 ? kcols : st->win_K;
    if (K > n + 1) K = n + 1;
    if (K <= 0) return;  // uniform
    even_dft_block<T, E>(xs, nnz, xn, n, tw, stw4, buf, im, xs, K - 1);
    const T sgn = (I & 1) ? (T)-1 : (T)1;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const T c = (k & 1) ? -xs[k] : xs[k];
        const CT y = CT{sgn * c, (T)0};
        zt[(size_t)k * N + I] = y;
        if (mirror) zt[(size_t)k * N + I2] = y;
    }
}

// Column pass: column k (with the row signs of the row pass) is even about
// row N/2; undoing the signs gives the even sequence x'_j = zt[N/2 + j]
// (-1)^(N/2+j), and the window value at row r is (-1)^k C'_|r - N/2| (the
// output sign (-1)^(r+k+N/2) included).  One column per block.
template <typename T, int E, int MAXT>
__global__ void __launch_bounds__(MAXT) cols_profile_dct_kernel(const C2<T>* __restrict__ zt, int N, int rmax,
                                                                const C2<T>* __restrict__ tw,
                                                                const C2<T>* __restrict__ stw4, C2<T>* __restrict__ out,
                                                                T* __restrict__ amp_out, long long s_row,
                                                                long long s_col, const DevState* __restrict__ st) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Window w = get_window(-1, -1, -1, st);
    const int k = blockIdx.x;
    if (k >= w.K) return;  // uniform for the whole block
    const int n = N / 2, M = N / 4;
    CT* buf = reinterpret_cast<CT*>(smem_raw);
    T* xs = reinterpret_cast<T*>(buf + fft_slots(M));
    T* im = xs + (n + 1);
    const CT* col = zt + (size_t)k * N;
    const int nnz = rmax < n ? rmax : n;
    for (int j = threadIdx.x; j < nnz; j += blockDim.x) {
        const T v = __ldg(&col[N / 2 + j]).x;
        xs[j] = ((N / 2 + j) & 1) ? -v : v;
    }
    const T xn = rmax >= n ? __ldg(&col[0]).x : (T)0;  // row 0 = N/2 - n, sign (+1)
    __syncthreads();
    const int dmax = max(N / 2 - w.r0, w.r0 + w.W - 1 - N / 2);
    even_dft_block<T, E>(xs, nnz, xn, n, tw, stw4, buf, im, xs, dmax);
    const T ks = (k & 1) ? (T)-1 : (T)1;
    for (int q = threadIdx.x; q < w.W; q += blockDim.x) {
        const int d = abs(w.r0 + q - N / 2);
        const T f = ks * xs[d];
        const long long o = (long long)q * s_row + (long long)k * s_col;
        out[o] = CT{f, (T)0};
        amp_out[o] = fabs(f);
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
// mixed-radix (2, 3, 4, 5, 7) versions of the row and column passes for even
// lengths that are not powers of two (block_fft_mixed; ping-pong buffers in
// shared memory, no padding)
// ---------------------------------------------------------------------------
// Row I of the image (or of the swept profile): the M = N/2 complex values
// x[2m] + i x[2m+1] are transformed and split into the real transform
// X_k = E_k + exp(-2 pi i k / N) O_k (E, O the transforms of the even and odd
// samples), k < K.
template <typename T>
__global__ void rows_mixed_kernel(const T* __restrict__ image, int N, int row0, const T* __restrict__ intensity, int nr,
                                  T Rmin, T dR, T dxy, T inv_cos_inc, int rmax, T central, int profile,
                                  const C2<T>* __restrict__ tw, MixPlan plan, const C2<T>* __restrict__ mtab,
                                  C2<T>* __restrict__ zt, int host_K, const DevState* __restrict__ st, int row_sign) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int M = N / 2;
    CT* a = reinterpret_cast<CT*>(smem_raw);
    CT* b = a + M;
    const int I = row0 + blockIdx.x;
    const int off = N / 2 - rmax;
    const T sr_to_px = dxy * dxy;
    for (int m = threadIdx.x; m < M; m += blockDim.x) {
        T x[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int J = 2 * m + h;
            if (profile) {
                x[h] = sweep_pixel<T>(I, J, intensity, nr, Rmin, dR, (T)1 / dR, dxy, inv_cos_inc, rmax, off, sr_to_px);
                if (I == N / 2 && J == N / 2) x[h] = central;
            } else {
                x[h] = image[(size_t)I * N + J];
            }
        }
        a[m] = CT{x[0], x[1]};
    }
    __syncthreads();
    const CT* Z = block_fft_mixed<T>(a, b, plan, mtab);
    const int K = get_window(host_K, 0, 0, st).K;
    const T sgn = (row_sign && (I & 1)) ? (T)-1 : (T)1;
    const T h = (T)0.5;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const CT za = Z[k % M], zb = Z[(M - k % M) % M];
        const CT e = CT{h * (za.x + zb.x), h * (za.y - zb.y)};
        const CT o = CT{h * (za.y + zb.y), -h * (za.x - zb.x)};
        const CT x = cadd(e, cmul(o, __ldg(&tw[k])));
        zt[(size_t)k * N + I] = CT{sgn * x.x, sgn * x.y};
    }
}

// Column k of zt (rows outside [band0, band1) are zero): the length-N
// transform, window rows written as cols_kernel does
template <typename T>
__global__ void cols_mixed_kernel(const C2<T>* __restrict__ zt, int N, int band0, int band1, MixPlan plan,
                                  const C2<T>* __restrict__ mtab, C2<T>* __restrict__ out, T* __restrict__ amp_out,
                                  long long s_row, long long s_col, int host_K, int host_r0, int host_W,
                                  const DevState* __restrict__ st, int out_sign) {
    using CT = C2<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT* a = reinterpret_cast<CT*>(smem_raw);
    CT* b = a + N;
    const Window w = get_window(host_K, host_r0, host_W, st);
    const int k = blockIdx.x;
    if (k >= w.K) return;  // uniform for the whole block
    for (int i = threadIdx.x; i < N; i += blockDim.x)
        a[i] = (i >= band0 && i < band1) ? zt[(size_t)k * N + i] : CT{(T)0, (T)0};
    __syncthreads();
    const CT* col = block_fft_mixed<T>(a, b, plan, mtab);
    const int par = (k + N / 2) & 1;
    for (int q = threadIdx.x; q < w.W; q += blockDim.x) {
        const int r = w.r0 + q;
        CT x = col[r];
        if (out_sign && ((r & 1) ^ par)) x = cneg(x);
        const long long o = (long long)q * s_row + (long long)k * s_col;
        out[o] = x;
        if (amp_out) amp_out[o] = cabs_<T>(x);
    }
}

// Plan of a length L = 4^a 2^b 3^c 5^d 7^e (false for other lengths) and its
// table: per stage, exp(-2 pi i m k / (Ns R)) at off + (m-1) Ns + k, then the
// R-th roots of unity; long-double values rounded once to T.  Built once per
// (device, L, precision) and kept until exit.
bool mix_plan(int L, MixPlan* p) {
    if (L < 2) return false;
    MixPlan q{};
    q.L = L;
    int n = L, ns = 1, off = 0;
    for (int r : {4, 2, 3, 5, 7}) {
        while (n % r == 0) {
            if (q.nst >= kMixMaxStages) return false;
            q.R[q.nst] = r;
            q.Ns[q.nst] = ns;
            q.off[q.nst] = off;
            off += (r - 1) * ns;
            ns *= r;
            n /= r;
            ++q.nst;
        }
    }
    if (n != 1) return false;
    for (int r : {3, 5, 7}) {
        q.root_off[r] = off;
        off += r;
    }
    *p = q;
    return true;
}
int mix_table_size(const MixPlan& p) { return p.root_off[7] + 7; }

template <typename T> const C2<T>* mix_table(const MixPlan& p) {
    static std::mutex mu;
    static std::map<std::pair<int, int>, C2<T>*> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find({dev, p.L});
    if (it != cache.end()) return it->second;
    const long double two_pi = 6.283185307179586476925286766559005768L;
    std::vector<C2<T>> h((size_t)mix_table_size(p));
    for (int s = 0; s < p.nst; ++s) {
        const int R = p.R[s], Ns = p.Ns[s];
        for (int m = 1; m < R; ++m)
            for (int k = 0; k < Ns; ++k) {
                const long double a = -two_pi * (long double)(m * k) / (long double)(Ns * R);
                h[(size_t)p.off[s] + (size_t)(m - 1) * Ns + k] = C2<T>{(T)cosl(a), (T)sinl(a)};
            }
    }
    for (int r : {3, 5, 7})
        for (int j = 0; j < r; ++j) {
            const long double a = -two_pi * (long double)j / (long double)r;
            h[(size_t)p.root_off[r] + j] = C2<T>{(T)cosl(a), (T)sinl(a)};
        }
    C2<T>* d = nullptr;
    if (cudaMalloc(&d, sizeof(C2<T>) * h.size()) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, h.data(), sizeof(C2<T>) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    cache[{dev, p.L}] = d;
    return d;
}

// ---------------------------------------------------------------------------
// dataset extent
// ---------------------------------------------------------------------------
// An upper bound of |x| as a float from the high word of a double, without
// FP64 arithmetic: the exponent and the top 20 mantissa bits plus one unit of
// the 20th bit (relative slack at most 2^-19).  NaN and inf give 0 (the
// visibility pass flags them), |x| < 2^-126 gives 2^-126, |x| >= 2^128 gives inf.
__device__ __forceinline__ float abs_bound_f(double x) {
    const unsigned hi = (unsigned)__double2hiint(x) & 0x7fffffffu;
    const int e = (int)(hi >> 20);
    if (e == 2047) return 0.f;
    if (e < 1023 - 126) return 1.17549435e-38f;
    if (e > 1023 + 127) return __uint_as_float(0x7f800000u);
    return __uint_as_float((((unsigned)(e - 1023 + 127) << 23) | ((hi & 0xfffffu) << 3)) + 8u);
}

template <typename T>
__global__ void extent_kernel(const T* __restrict__ u, const T* __restrict__ v, int nd, int N, double duv,
                              DevState* st, T* __restrict__ u_out, T* __restrict__ v_out) {
    // max(u^2 + v^2) (NaN entries are ignored here and flagged by the
    // visibility pass), in FP32: for FP64 inputs as the sum of squares of
    // upper bounds of |u| and |v| (an upper bound itself: its rounding is far
    // below the bounds' slack); the window adds a relative margin larger than
    // the slack.  With u_out and v_out (both or neither) the pass also writes
    // a copy of u and v there: it stages arrays that sit in host memory.
    const bool copy = u_out != nullptr;
    float mt = 0.f;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    int done = 0;
    if ((reinterpret_cast<uintptr_t>(u) & 15) == 0 && (reinterpret_cast<uintptr_t>(v) & 15) == 0 &&
        (reinterpret_cast<uintptr_t>(u_out) & 15) == 0 && (reinterpret_cast<uintptr_t>(v_out) & 15) == 0) {
        // 16-byte vector loads
        using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
        constexpr int L = 16 / sizeof(T);
        const int nvec = nd / L;
        const V* uv = reinterpret_cast<const V*>(u);
        const V* vv = reinterpret_cast<const V*>(v);
        auto acc = [&](const V& a, const V& b) {
            if constexpr (sizeof(T) == 4) {
                mt = fmaxf(mt, fmaxf(fmaxf(a.x * a.x + b.x * b.x, a.y * a.y + b.y * b.y),
                                     fmaxf(a.z * a.z + b.z * b.z, a.w * a.w + b.w * b.w)));
            } else {
                const float ax = abs_bound_f(a.x), ay = abs_bound_f(a.y);
                const float bx = abs_bound_f(b.x), by = abs_bound_f(b.y);
                mt = fmaxf(mt, fmaxf(fmaf(ax, ax, bx * bx), fmaf(ay, ay, by * by)));
            }
        };
        int i = tid;
        for (; i + 3 * nth < nvec; i += 4 * nth) {  // four vectors of each array in flight
            V a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                a[r] = __ldg(&uv[i + r * nth]);
                b[r] = __ldg(&vv[i + r * nth]);
            }
#pragma unroll
            for (int r = 0; r < 4; ++r) acc(a[r], b[r]);
            if (copy) {
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    reinterpret_cast<V*>(u_out)[i + r * nth] = a[r];
                    reinterpret_cast<V*>(v_out)[i + r * nth] = b[r];
                }
            }
        }
        for (; i < nvec; i += nth) {
            const V a = __ldg(&uv[i]), b = __ldg(&vv[i]);
            acc(a, b);
            if (copy) {
                reinterpret_cast<V*>(u_out)[i] = a;
                reinterpret_cast<V*>(v_out)[i] = b;
            }
        }
        done = nvec * L;
    }
    for (int i = done + tid; i < nd; i += nth) {
        const T a = __ldg(&u[i]), b = __ldg(&v[i]);
        if (copy) {
            u_out[i] = a;
            v_out[i] = b;
        }
        if constexpr (sizeof(T) == 4) {
            mt = fmaxf(mt, a * a + b * b);
        } else {
            const float ab = abs_bound_f(a), bb = abs_bound_f(b);
            mt = fmaxf(mt, fmaf(ab, ab, bb * bb));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mt = fmaxf(mt, __shfl_xor_sync(0xffffffffu, mt, o));
    double m = (double)mt;
    __shared__ double sh[32];  // one per warp, blocks of up to 1024 threads
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

// Copy of [0, n) of three arrays (the observations' first visibilities, read
// from host memory) into device buffers; three 16-byte loads in flight per
// thread where all six pointers allow vectors.
template <typename T>
__global__ void stage3_kernel(const T* __restrict__ a, const T* __restrict__ b, const T* __restrict__ c,
                              T* __restrict__ da, T* __restrict__ db, T* __restrict__ dc, int n) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    int done = 0;
    const uintptr_t al = reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) |
                         reinterpret_cast<uintptr_t>(c) | reinterpret_cast<uintptr_t>(da) |
                         reinterpret_cast<uintptr_t>(db) | reinterpret_cast<uintptr_t>(dc);
    if ((al & 15) == 0) {
        using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
        constexpr int L = 16 / sizeof(T);
        const int nvec = n / L;
        for (int i = tid; i < nvec; i += nth) {
            const V x = __ldg(reinterpret_cast<const V*>(a) + i);
            const V y = __ldg(reinterpret_cast<const V*>(b) + i);
            const V z = __ldg(reinterpret_cast<const V*>(c) + i);
            reinterpret_cast<V*>(da)[i] = x;
            reinterpret_cast<V*>(db)[i] = y;
            reinterpret_cast<V*>(dc)[i] = z;
        }
        done = nvec * L;
    }
    for (int i = done + tid; i < n; i += nth) {
        da[i] = __ldg(&a[i]);
        db[i] = __ldg(&b[i]);
        dc[i] = __ldg(&c[i]);
    }
}

// ---------------------------------------------------------------------------
// fused visibility kernel
// reference: uv_rotate_core :955-960, interpolate_core :749-815,
//            apply_phase_sampled_core :877-884, diff_weighted_core :1453-1461
// ---------------------------------------------------------------------------
// Bilinear amplitude/phase interpolation at cell (fu, fv) with fractions
// (q, t) along u and v (reference interpolate_core :749-815).  Corners follow
// the reference's flat-index semantics of the row-major N x C spectrum
// (:774-780): a corner past the last column continues on the next row.
// Returns false (and sets err bits) when a corner is outside the spectrum.
// The same for the real spectrum of a swept profile (corners y real, z real):
// amp * exp(i sign_u arg z) = (amp * sign(z), 0).  Corners come from the real
// cell records, or from the window's real parts when it exceeds the record
// capacity.  Writes the real result to *out.
// t in [0, 1) (FP64) to FP32 by integer operations on its bit pattern
// (exponent rebiased, mantissa truncated to 23 bits: relative error below
// 2^-23); values below 2^-126 give 0.
__device__ __forceinline__ float frac_to_f(double t) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(t);
    const int e = (int)(b >> 52) - 1023;
    if (e < -126) return 0.f;
    return __uint_as_float(((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
}

// floor and fraction of x in [0, 2^30) by integer operations on the bit
// pattern, exactly (the FP64 pipe, the bound of this kernel, is not used):
// the integer part is the significand shifted right by 52 - e, the fraction
// the remaining bits, renormalised with a leading-zero count.  Returns false
// (and leaves the FP64 path to the caller) outside that range.
__device__ __forceinline__ bool floor_frac_bits(double x, int* fl, double* frac) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if (b >> 63) return false;  // negative (or -0)
    const int e = (int)(b >> 52) - 1023;
    if (e > 29) return false;
    if (e < 0) {  // x < 1 (and x = 0)
        *fl = 0;
        *frac = x;
        return true;
    }
    const unsigned long long m = (b & 0xfffffffffffffULL) | 0x10000000000000ULL;
    const int sh = 52 - e;
    *fl = (int)(m >> sh);
    const unsigned long long f = m & ((1ULL << sh) - 1ULL);  // fraction = f 2^-sh
    if (f == 0ULL) {
        *frac = 0.0;
        return true;
    }
    const int p = 63 - __clzll((long long)f);  // top bit of f: fraction in [2^(p-sh), 2^(p-sh+1))
    const unsigned long long mant = (f << (52 - p)) & 0xfffffffffffffULL;
    *frac = __longlong_as_double((long long)((((unsigned long long)(p - sh + 1023)) << 52) | mant));
    return true;
}

template <typename T>
__device__ __forceinline__ bool interp_cell_real(const typename Launch<T>::VisArgs& a, const Window& w, int fu,
                                                 int fv, T q, T t, T* out, unsigned* err) {
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
    const int qq = r0 - w.r0;
    T yr[4];
    float yf[4];
    bool have_f = false;
    T amp = (T)0;
    bool have_amp = false;  // FP64 records: modulus from their coefficients, signed corners from spec if needed
    bool have_y = false;    // FP32 records: the signed corners
    if ((long long)w.K * w.W <= a.quad_cap) {
        const bool inside = wrap ? (w.K == C && qq >= 0 && qq < w.W - 2) : (c0 < w.K - 1 && qq >= 0 && qq < w.W - 1);
        if (!inside) {
            *err |= ERR_WINDOW;
            return false;
        }
        const T* rec = a.quads + ((long long)c0 * w.W + qq) * real_rec<T>();
        if constexpr (sizeof(T) == 4) {
            const float4 p0 = __ldg(reinterpret_cast<const float4*>(rec));
            yr[0] = p0.x;
            yr[1] = p0.y;
            yr[2] = p0.z;
            yr[3] = p0.w;
            have_y = true;
        } else {
            // the reference's bilinear modulus (interpolate_core :804-812) from
            // the record's coefficients (see quad_real_kernel)
            const double2 p0 = __ldg(reinterpret_cast<const double2*>(rec));
            const double2 p1 = __ldg(reinterpret_cast<const double2*>(rec) + 1);
            const float4 pf = __ldg(reinterpret_cast<const float4*>(rec + 4));
            amp = fma(q, fma(t, p1.y, p1.x), fma(t, p0.y, p0.x));
            have_amp = true;
            yf[0] = pf.x;
            yf[1] = pf.y;
            yf[2] = pf.z;
            yf[3] = pf.w;
            have_f = true;
        }
    }
    // the four signed corners from the window (cells without a record, and
    // FP64 cells whose sign the FP32 estimate leaves open)
    auto corners = [&]() -> bool {
        const int rr[4] = {r0, r0 + 1, r_last, wrap ? r0 + 1 : r0};
        const int cc[4] = {c0, c0, wrap ? 0 : c0 + 1, wrap ? 0 : c0 + 1};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int qc = rr[c] - w.r0;
            if (cc[c] >= w.K || qc < 0 || qc >= w.W) return false;
            yr[c] = __ldg(&a.spec[(long long)qc * a.s_row + (long long)cc[c] * a.s_col]).x;
        }
        return true;
    };
    if (!have_amp && !have_y && !corners()) {
        *err |= ERR_WINDOW;
        return false;
    }
    // the reference's bilinear forms (interpolate_core :782-812),
    // y0 + t (y1 - y0) + q ((y3 - y0) + t (y0 - y1 + y2 - y3)), in fused
    // multiply-adds: the moduli, and the signed corners z of which only the
    // sign is used
    if (!have_amp) {
        const T m0 = fabs(yr[0]), m1 = fabs(yr[1]), m2 = fabs(yr[2]), m3 = fabs(yr[3]);
        const T e1 = m1 - m0, e3 = m3 - m0;
        amp = fma(q, fma(t, (m2 - m3) - e1, e3), fma(t, e1, m0));
    }
    bool neg;
    bool decided = false;
    if constexpr (sizeof(T) == 8) {
        if (have_f) {
            // FP32 estimate of z from the records' FP32 corners and the
            // fractions truncated to FP32: its error is below
            // (8 * 2^-24 + 2 * 2^-23) * sum|y| < 7.2e-7 sum|y|, so a value
            // beyond 4e-6 sum|y| has the sign of the FP64 z
            const float tf = frac_to_f(t), qf = frac_to_f(q);
            const float g1 = yf[1] - yf[0], g3 = yf[3] - yf[0];
            const float zf = fmaf(qf, fmaf(tf, (yf[2] - yf[3]) - g1, g3), fmaf(tf, g1, yf[0]));
            const float mag = (fabsf(yf[0]) + fabsf(yf[1])) + (fabsf(yf[2]) + fabsf(yf[3]));
            if (fabsf(zf) > 4e-6f * mag) {
                neg = zf < 0.f;
                decided = true;
            }
        }
    }
    if (!decided) {
        if (have_amp && !corners()) {
            *err |= ERR_WINDOW;
            return false;
        }
        const T f1 = yr[1] - yr[0], f3 = yr[3] - yr[0];
        const T zr = fma(q, fma(t, (yr[2] - yr[3]) - f1, f3), fma(t, f1, yr[0]));
        neg = zr < (T)0;
    }
    if constexpr (sizeof(T) == 8) {
        // the sign as a bit operation (no FP64 instruction)
        *out = __longlong_as_double(__double_as_longlong(amp) ^ (neg ? (long long)0x8000000000000000ULL : 0LL));
    } else {
        *out = neg ? -amp : amp;
    }
    return true;
}

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
// parts (FP64 real spectrum): receives (A, cos, sin) with V = A (cos, sin),
// so that the residual can be formed with fused multiply-adds
template <typename T, bool REALQ>
__device__ __forceinline__ C2<T> vis_point(const typename Launch<T>::VisArgs& a, const Window& w, T u_in, T v_in,
                                           unsigned* e, T* parts = nullptr) {
    using CT = C2<T>;
    CT out = CT{(T)0, (T)0};
    if constexpr (sizeof(T) == 8) {
        // FP64.  Grid coordinates of the rotated point, ga = u'/duv and
        // gc = v'/duv, with cos(PA)/duv and sin(PA)/duv from the host (the
        // reference divides u' by duv: same value to rounding).
        double ga = u_in * a.inv_duv, gc = v_in * a.inv_duv;
        if (a.rotate) {
            ga = fma(u_in, a.cu_d, -(v_in * a.su_d));
            gc = fma(u_in, a.su_d, v_in * a.cu_d);
        }
        // the Hermitian half: indu = |u'|/duv and v' -> v_origin sign(u') v'
        // (sign(u') = copysign(1, u'), as the reference), as sign-bit operations
        constexpr long long kSign = (long long)0x8000000000000000ULL, kExp = 0x7ff0000000000000LL;
        const long long ba = __double_as_longlong(ga), bc = __double_as_longlong(gc);
        const long long sa = ba & kSign;
        const long long bu = ba ^ sa, bv = bc ^ sa ^ a.vo_sign;
        // |indu|, |v'/duv| < 4 N as integer compares of the bit patterns of
        // non-negative doubles (NaN and inf compare above every finite value)
        if (!(bu < a.lim_bits && (bv & ~kSign) < a.lim_bits)) {
            *e = ((ba & kExp) == kExp || (bc & kExp) == kExp) ? ERR_UV_NONFINITE : ERR_UV_OUTSIDE;
            return out;
        }
        const double indu = __longlong_as_double(bu);
        const double indv = a.half_nrow + __longlong_as_double(bv);
        // cell and fractions: integer operations on the bit patterns (exact),
        // FP64 floor only for a negative indv (a point outside the spectrum)
        int ifu, ifv;
        double qf, tf;
        if (!floor_frac_bits(indu, &ifu, &qf)) {
            const double f = floor(indu);
            ifu = (int)f;
            qf = indu - f;
        }
        if (!floor_frac_bits(indv, &ifv, &tf)) {
            const double f = floor(indv);
            ifv = (int)f;
            tf = indv - f;
        }
        if constexpr (REALQ) {
            T amp;
            if (interp_cell_real<T>(a, w, ifu, ifv, (T)qf, (T)tf, &amp, e)) {
                out = CT{amp, (T)0};
                double sn = 0.0, cs = 1.0;
                if (a.phase) {
                    // u' dra + v' ddec = ga (dra duv) + gc (ddec duv) cycles
                    sincos2pi_tab(fma(ga, a.dra_g, gc * a.ddec_g), a.phase_tab, &sn, &cs);
                    out = CT{amp * (T)cs, amp * (T)sn};
                }
                if (parts) {
                    parts[0] = amp;
                    parts[1] = (T)cs;
                    parts[2] = (T)sn;
                }
            }
        } else if (interp_cell<T>(a, w, ifu, ifv, (T)qf, (T)tf, sa ? (T)-1 : (T)1, &out, e) &&
                   a.phase) {
            double sn, cs;
            sincos2pi_tab(fma(ga, a.dra_g, gc * a.ddec_g), a.phase_tab, &sn, &cs);
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
        bool ok;
        if constexpr (REALQ) {
            T amp;
            ok = interp_cell_real<T>(a, w, fu, fv, (T)q, (T)t, &amp, e);
            if (ok) out = CT{amp, (T)0};
        } else {
            ok = interp_cell<T>(a, w, fu, fv, (T)q, (T)t, (T)sign_u, &out, e);
        }
        if (ok && a.phase) {
            const DF ph = df_add(df_mul(ur, a.dra_df), df_mul(vr, a.ddec_df));  // cycles
            float sn, cs;
            sincos2pi_df(ph, &sn, &cs);
            if constexpr (REALQ) out = CT{out.x * (T)cs, out.x * (T)sn};
            else out = cmul(out, CT{(T)cs, (T)sn});
        }
    }
    return out;
}

// Grid-stride over the visibilities, two independent points per iteration so
// their load -> gather chains overlap.
// SPLIT: the observations of visibilities [a.split, nd) come from re2/im2/w2.
template <typename T, bool CHI2, bool VISOUT, bool REALQ, bool SPLIT = false>
__global__ void __launch_bounds__(256, (sizeof(T) == 8 && REALQ) ? 4 : 1) vis_kernel(typename Launch<T>::VisArgs a) {
    using CT = C2<T>;
    __shared__ double sh[32];
    asm volatile("griddepcontrol.wait;" ::: "memory");  // a no-op unless launched as a programmatic dependent
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
            const bool h0 = SPLIT && i0 >= a.split, h1 = SPLIT && i1 >= a.split;
            re0 = __ldg(&(h0 ? a.re2 : a.re)[i0]);
            im0 = __ldg(&(h0 ? a.im2 : a.im)[i0]);
            w0 = __ldg(&(h0 ? a.w2 : a.w)[i0]);
            if (has1) {
                re1 = __ldg(&(h1 ? a.re2 : a.re)[i1]);
                im1 = __ldg(&(h1 ? a.im2 : a.im)[i1]);
                w1 = __ldg(&(h1 ? a.w2 : a.w)[i1]);
            }
        }
        unsigned e0 = 0u, e1 = 0u;
        // FP64 real spectrum: V = A (cos, sin) kept in parts, the residual in fused multiply-adds
        constexpr bool kParts = CHI2 && REALQ && sizeof(T) == 8;
        T p0[3] = {(T)0, (T)1, (T)0}, p1[3] = {(T)0, (T)1, (T)0};
        const CT o0 = vis_point<T, REALQ>(a, w, u0, v0, &e0, kParts ? p0 : nullptr);
        const CT o1 = has1 ? vis_point<T, REALQ>(a, w, u1, v1, &e1, kParts ? p1 : nullptr) : CT{(T)0, (T)0};
        if (e0 | e1) {
            err |= e0 | e1;
            if (err_idx < 0) err_idx = (long long)a.base + (e0 ? i0 : i1);
        }
        if (VISOUT) {
            a.vis_out[i0] = o0;
            if (has1) a.vis_out[i1] = o1;
        }
        if (CHI2) {
            T dr0, di0, dr1, di1;
            if constexpr (kParts) {
                dr0 = fma(p0[0], p0[1], -re0);
                di0 = fma(p0[0], p0[2], -im0);
                dr1 = fma(p1[0], p1[1], -re1);
                di1 = fma(p1[0], p1[2], -im1);
            } else {
                dr0 = o0.x - re0;
                di0 = o0.y - im0;
                dr1 = o1.x - re1;
                di1 = o1.y - im1;
            }
            acc += w0 * (dr0 * dr0 + di0 * di0);
            acc += w1 * (dr1 * dr1 + di1 * di1);  // w1 == 0 when i1 is past the end
        }
    }
    if (err) {
        atomicOr(&a.state->err, err);
        atomicCAS(&a.state->err_index, 0ull, (unsigned long long)(err_idx + 1));
    }
    if (CHI2) {
        double tot;
        if constexpr (sizeof(T) == 4) tot = block_sum_df(acc, sh);
        else tot = block_sum((double)acc, sh);
        grid_finish(tot, a.partials, a.state, a.chi2_out, a.part_off, a.parts_total);
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

// Records of a real spectrum (a swept profile's), cell e = (k, q).  FP32: the
// 4 corners y_c at quads[4 e + c] (the moduli are their absolute values).
// FP64 (48 bytes): the coefficients of the bilinear modulus in the
// reference's algebraic form (interpolate_core :804-812), m0 = |y0|,
// e1 = |y1| - m0, e3 = |y3| - m0, e2 = (|y2| - |y3|) - e1, so that the
// visibility pass evaluates A = m0 + t e1 + q (e3 + t e2) with three fused
// multiply-adds (the same operations on the same values as evaluating it
// from the corners), then the 4 corners as FP32 for the sign estimate of z.
template <typename T>
__global__ void quad_real_kernel(const C2<T>* __restrict__ spec, long long s_row, long long s_col, int C,
                                 const DevState* __restrict__ st, T* __restrict__ quads, long long cap) {
    asm volatile("griddepcontrol.wait;" ::: "memory");  // a no-op unless launched as a programmatic dependent
    const Window w = get_window(-1, -1, -1, st);
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
        T* rec = quads + e * real_rec<T>();
        T y[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) y[c] = spec[(long long)rr[c] * s_row + (long long)cc[c] * s_col].x;
        if constexpr (sizeof(T) == 8) {
            const T m0 = fabs(y[0]), m1 = fabs(y[1]), m2 = fabs(y[2]), m3 = fabs(y[3]);
            const T e1 = m1 - m0, e3 = m3 - m0;
            reinterpret_cast<double2*>(rec)[0] = make_double2(m0, e1);
            reinterpret_cast<double2*>(rec)[1] = make_double2(e3, (m2 - m3) - e1);
            *reinterpret_cast<float4*>(rec + 4) = make_float4((float)y[0], (float)y[1], (float)y[2], (float)y[3]);
        } else {
#pragma unroll
            for (int c = 0; c < 4; ++c) rec[c] = y[c];
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

// GALARIO_ROWS_TMA=0 keeps the one-row-per-CTA image row pass
bool rows_tma_enabled() {
    const char* v = std::getenv("GALARIO_ROWS_TMA");
    return !(v && v[0] == '0');
}

template <typename T>
cudaError_t Launch<T>::extent(const T* u, const T* v, int nd, int N, double duv, DevState* state, cudaStream_t s,
                              T* u_out, T* v_out) {
    if ((u_out == nullptr) != (v_out == nullptr)) return cudaErrorInvalidValue;
    const int threads = u_out ? 128 : 256;
    // device arrays: as many threads as give each one iteration of the
    // four-vector loop (eight 16-byte loads in flight per thread); the
    // earlier grid of 8 CTAs per SM left most threads loading one vector at a
    // time in the tail loop
    const int per_thread = u_out ? 1 : 4 * (16 / (int)sizeof(T));
    int blocks = (int)(((long long)nd + (long long)threads * per_thread - 1) / ((long long)threads * per_thread));
    // staging from host memory: one CTA per SM keeps enough loads in flight
    // to fill the host link and leaves the SMs to the row pass beside it
    const int cap = num_sms() * (u_out ? 1 : 8);
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    // an SM changes its L1/shared split only when idle: ask for the largest
    // shared share, so that the row pass's blocks fit beside these
    cudaError_t e = cudaFuncSetAttribute(extent_kernel<T>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    extent_kernel<T><<<blocks, threads, 0, s>>>(u, v, nd, N, duv, state, u_out, v_out);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::stage3(const T* a, const T* b, const T* c, T* da, T* db, T* dc, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    int blocks = (n + 255) / 256;
    const int cap = num_sms();
    if (blocks > cap) blocks = cap;
    cudaError_t e = cudaFuncSetAttribute(stage3_kernel<T>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    stage3_kernel<T><<<blocks, 128, 0, s>>>(a, b, c, da, db, dc, n);
    return cudaGetLastError();
}

// (values per thread EE, block-size bound TT) for an FFT with `threads` threads
#define GBG_CASE_T(E_V, THR, ...)                                                          \
    {                                                                                      \
        constexpr int EE = E_V;                                                            \
        if ((THR) <= 256) { constexpr int TT = 256; __VA_ARGS__; }                         \
        else if ((THR) <= 512) { constexpr int TT = 512; __VA_ARGS__; }                    \
        else { constexpr int TT = 1024; __VA_ARGS__; }                                     \
    }
// E = 8 or 16 only (the even-sequence transforms: at least 32 threads)
#define GBG_DISPATCH_E816(E_, THR, ...)                                           \
    switch (E_) {                                                                 \
        case 8: GBG_CASE_T(8, THR, __VA_ARGS__) break;                            \
        case 16: GBG_CASE_T(16, THR, __VA_ARGS__) break;                          \
        default: return cudaErrorInvalidValue;                                    \
    }
#define GBG_DISPATCH_E(E_, THR, ...)                                              \
    switch (E_) {                                                                 \
        case 1: { constexpr int EE = 1; constexpr int TT = 256; __VA_ARGS__; } break; \
        case 2: { constexpr int EE = 2; constexpr int TT = 256; __VA_ARGS__; } break; \
        case 4: { constexpr int EE = 4; constexpr int TT = 256; __VA_ARGS__; } break; \
        case 8: GBG_CASE_T(8, THR, __VA_ARGS__) break;                             \
        case 16: GBG_CASE_T(16, THR, __VA_ARGS__) break;                           \
        default: return cudaErrorInvalidValue;                                    \
    }

template <typename T>
cudaError_t Launch<T>::rows_image(const T* image, int N, const CT* tw, const CT* stw, CT* zt, int host_K,
                                  const DevState* state, double duv, bool row_sign, cudaStream_t s) {
    if (is_pow2(N) && N <= max_fft_n_impl<T>() * 2) {
        const int M = N / 2;
        FftCfg<T> c = fft_cfg<T>(M);
        cudaError_t e = cudaSuccess;
        // FP32: the pipelined variant where its staging fits (N * 4 bytes a
        // multiple of 16, a 16-byte aligned image)
        const size_t sm_tma = 2 * sizeof(float) * (size_t)N + c.smem + 2 * sizeof(uint64_t);
        if constexpr (sizeof(T) == 4) {
            if (N >= 64 && (N % 4) == 0 && ((reinterpret_cast<uintptr_t>(image) & 15) == 0) &&
                sm_tma <= 200 * 1024 && rows_tma_enabled()) {
                GBG_DISPATCH_E(c.E, c.threads, {
                    auto kern = rows_image_tma_kernel<EE, TT>;
                    e = set_smem(kern, sm_tma);
                    int per_sm = 0;
                    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, c.threads, sm_tma);
                    if (e == cudaSuccess) {
                        const int grid = std::max(1, std::min(N, num_sms() * std::max(per_sm, 1)));
                        kern<<<grid, c.threads, sm_tma, s>>>(image, N, tw, stw, zt, host_K,
                                                             const_cast<DevState*>(state), row_sign ? 1 : 0);
                        e = cudaGetLastError();
                    }
                });
                return e;
            }
        }
        GBG_DISPATCH_E(c.E, c.threads, {
            auto kern = rows_image_kernel<T, EE, TT>;
            e = set_smem(kern, c.smem);
            if (e == cudaSuccess) {
                kern<<<N, c.threads, c.smem, s>>>(image, N, tw, stw, zt, host_K, state, duv, row_sign ? 1 : 0);
                e = cudaGetLastError();
            }
        });
        return e;
    }
    MixPlan mp;
    const C2<T>* mt = nullptr;
    if ((N % 2) == 0 && mix_plan(N / 2, &mp) && sizeof(CT) * (size_t)N <= 200 * 1024 && (mt = mix_table<T>(mp))) {
        const size_t smm = sizeof(CT) * (size_t)N;  // two buffers of N/2
        cudaError_t e = set_smem(rows_mixed_kernel<T>, smm);
        if (e != cudaSuccess) return e;
        rows_mixed_kernel<T><<<N, 256, smm, s>>>(image, N, 0, nullptr, 0, (T)0, (T)1, (T)1, (T)1, 0, (T)0, 0, tw, mp,
                                                 mt, zt, host_K, state, row_sign ? 1 : 0);
        return cudaGetLastError();
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
                                    int rmax, double central_value, int N, const CT* tw, const CT* stw, CT* zt,
                                    const DevState* state, double duv, cudaStream_t s, int kcols, const CT* stw4) {
    const int nrows = 2 * rmax;
    if (kcols > N / 2 + 1) kcols = N / 2 + 1;
    if (nrows <= 0) return cudaSuccess;
    const T inv_cos = (T)(1.0 / cos_inc);
    if constexpr (sizeof(T) == 8) {  // the FP32 passes keep the paired transforms
    if (stw4 && even_dft_ok<T>(N)) {
        FftCfg<T> c;
        c.E = even_dft_e<T>(N);
        c.threads = (N / 4) / c.E;
        const size_t sm = even_dft_smem<T>(N);
        cudaError_t e = cudaSuccess;
        GBG_DISPATCH_E816(c.E, c.threads, {
            auto kern = rows_profile_dct_kernel<T, EE, TT>;
            e = set_smem(kern, sm);
            if (e == cudaSuccess) {
                kern<<<rmax + 1, c.threads, sm, s>>>(intensity, nr, (T)Rmin, (T)dR, (T)(1.0 / dR), (T)dxy, inv_cos,
                                                     rmax, (T)central_value, N, tw, stw4, zt, state, kcols);
                e = cudaGetLastError();
            }
        });
        return e;
    }
    }
    if (is_pow2(N) && N <= max_fft_n_impl<T>() * 2) {
        const int M = N / 2;
        FftCfg<T> c = fft_cfg<T>(M);
        cudaError_t e = cudaSuccess;
        GBG_DISPATCH_E(c.E, c.threads, {
            auto kern = rows_profile_kernel<T, EE, TT>;
            e = set_smem(kern, c.smem);
            if (e == cudaSuccess) {
                kern<<<rmax + 1, c.threads, c.smem, s>>>(intensity, nr, (T)Rmin, (T)dR, (T)(1.0 / dR), (T)dxy,
                                                         inv_cos, rmax, (T)central_value, N, tw, stw, zt, state, duv,
                                                         kcols);
                e = cudaGetLastError();
            }
        });
        return e;
    }
    MixPlan mp;
    const C2<T>* mt = nullptr;
    if ((N % 2) == 0 && mix_plan(N / 2, &mp) && sizeof(CT) * (size_t)N <= 200 * 1024 && (mt = mix_table<T>(mp))) {
        const size_t smm = sizeof(CT) * (size_t)N;
        cudaError_t e = set_smem(rows_mixed_kernel<T>, smm);
        if (e != cudaSuccess) return e;
        rows_mixed_kernel<T><<<nrows, 256, smm, s>>>(nullptr, N, N / 2 - rmax, intensity, nr, (T)Rmin, (T)dR, (T)dxy,
                                                     inv_cos, rmax, (T)central_value, 1, tw, mp, mt, zt, kcols, state,
                                                     1);
        return cudaGetLastError();
    }
    const size_t sm = sizeof(T) * (size_t)N;
    cudaError_t e = set_smem(rows_direct_kernel<T>, sm);
    if (e != cudaSuccess) return e;
    rows_direct_kernel<T><<<nrows, 256, sm, s>>>(nullptr, N, N / 2 - rmax, intensity, nr, (T)Rmin, (T)dR, (T)dxy,
                                                 inv_cos, rmax, (T)central_value, 1, tw, zt, kcols, state, duv, 1);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::cols_profile(const CT* zt, int N, int band0, int band1, const CT* tw, const CT* stw, CT* out,
                                    T* amp_out, long long s_row, long long s_col, const DevState* state, double duv,
                                    cudaStream_t s, const CT* stw4) {
    if constexpr (sizeof(T) == 8) {  // the FP32 passes keep the paired transforms
    if (stw4 && amp_out && even_dft_ok<T>(N)) {
        FftCfg<T> c;
        c.E = even_dft_e<T>(N);
        c.threads = (N / 4) / c.E;
        const size_t sm = even_dft_smem<T>(N);
        const int rmax = N / 2 - band0;  // the band is [N/2 - rmax, N/2 + rmax)
        cudaError_t e = cudaSuccess;
        GBG_DISPATCH_E816(c.E, c.threads, {
            auto kern = cols_profile_dct_kernel<T, EE, TT>;
            e = set_smem(kern, sm);
            if (e == cudaSuccess) {
                kern<<<N / 2 + 1, c.threads, sm, s>>>(zt, N, rmax, tw, stw4, out, amp_out, s_row, s_col, state);
                e = cudaGetLastError();
            }
        });
        return e;
    }
    }
    if (is_pow2(N) && N <= max_fft_n_impl<T>() && amp_out) {
        const int C = N / 2 + 1;
        FftCfg<T> c = fft_cfg<T>(N);
        cudaError_t e = cudaSuccess;
        GBG_DISPATCH_E(c.E, c.threads, {
            auto kern = cols_pair_kernel<T, EE, TT>;
            e = set_smem(kern, c.smem);
            if (e == cudaSuccess) {
                kern<<<(C + 1) / 2, c.threads, c.smem, s>>>(zt, N, band0, band1, stw, out, amp_out, s_row, s_col,
                                                             state);
                e = cudaGetLastError();
            }
        });
        return e;
    }
    return cols(zt, N, band0, band1, tw, stw, out, amp_out, s_row, s_col, -1, -1, -1, state, duv, true, s);
}

template <typename T>
cudaError_t Launch<T>::cols(const CT* zt, int N, int band0, int band1, const CT* tw, const CT* stw, CT* out,
                            T* amp_out, long long s_row, long long s_col, int host_K, int host_r0, int host_W,
                            const DevState* state, double duv, bool out_sign, cudaStream_t s) {
    const int C = N / 2 + 1;
    const int grid = host_K >= 0 ? host_K : C;
    if (grid <= 0) return cudaSuccess;
    if (is_pow2(N) && N <= max_fft_n_impl<T>()) {
        FftCfg<T> c = fft_cfg<T>(N);
        cudaError_t e = cudaSuccess;
        GBG_DISPATCH_E(c.E, c.threads, {
            auto kern = cols_kernel<T, EE, TT>;
            e = set_smem(kern, c.smem);
            if (e == cudaSuccess) {
                kern<<<grid, c.threads, c.smem, s>>>(zt, N, band0, band1, stw, out, amp_out, s_row, s_col, host_K,
                                                     host_r0, host_W, state, duv, out_sign ? 1 : 0);
                e = cudaGetLastError();
            }
        });
        return e;
    }
    MixPlan mp;
    const C2<T>* mt = nullptr;
    if (mix_plan(N, &mp) && 2 * sizeof(CT) * (size_t)N <= 200 * 1024 && (mt = mix_table<T>(mp))) {
        const size_t smm = 2 * sizeof(CT) * (size_t)N;
        cudaError_t e = set_smem(cols_mixed_kernel<T>, smm);
        if (e != cudaSuccess) return e;
        cols_mixed_kernel<T><<<grid, 256, smm, s>>>(zt, N, band0, band1, mp, mt, out, amp_out, s_row, s_col, host_K,
                                                    host_r0, host_W, state, out_sign ? 1 : 0);
        return cudaGetLastError();
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
    // FP64: one wave of the profile kernel (4 blocks per SM), so that every
    // thread's share of the block reduction's FP64 additions is spread over
    // twice as many visibilities
    const int cap = num_sms() * (sizeof(T) == 8 ? 4 : 8);
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return blocks;
}

template <typename T> cudaError_t Launch<T>::vis(const VisArgs& args, cudaStream_t s, bool pdl) {
    VisArgs a = args;
    a.finalize();
    const int blocks = vis_grid(a.nd);
    const bool chi2 = a.partials != nullptr, vo = a.vis_out != nullptr;
    // real_quads: the spectrum of a swept profile, interpolated as a real spectrum
    if (!(chi2 || vo)) return cudaErrorInvalidValue;
    if (a.split < a.nd) {  // observations partly from re2/im2/w2 (chi2 only)
        if (!chi2 || vo || !a.re2 || !a.im2 || !a.w2) return cudaErrorInvalidValue;
        if (a.real_quads && a.quads) vis_kernel<T, true, false, true, true><<<blocks, 256, 0, s>>>(a);
        else vis_kernel<T, true, false, false, true><<<blocks, 256, 0, s>>>(a);
        return cudaGetLastError();
    }
    if (a.real_quads && a.quads) {
        if (chi2 && vo) return launch_on(vis_kernel<T, true, true, true>, blocks, 256, s, pdl, a);
        else if (chi2) return launch_on(vis_kernel<T, true, false, true>, blocks, 256, s, pdl, a);
        else return launch_on(vis_kernel<T, false, true, true>, blocks, 256, s, pdl, a);
    } else {
        if (chi2 && vo) vis_kernel<T, true, true, false><<<blocks, 256, 0, s>>>(a);
        else if (chi2) vis_kernel<T, true, false, false><<<blocks, 256, 0, s>>>(a);
        else vis_kernel<T, false, true, false><<<blocks, 256, 0, s>>>(a);
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::quads_real(const CT* spec, long long s_row, long long s_col, int C, const DevState* state,
                                  T* q, long long cap, cudaStream_t s, bool pdl) {
    return launch_on(quad_real_kernel<T>, num_sms() * 4, 256, s, pdl, spec, s_row, s_col, C, state, q, cap);
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
