// Device helpers shared by the galario_gb300 kernel translation units:
// complex arithmetic, the shared-memory Stockham FFT, the real-row split,
// conversion-free FP32 rounding, the profile sweep, block/grid reductions,
// double-float arithmetic and the sin/cos evaluations of the phase shift.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <vector>

#include "gb_internal.cuh"

namespace gbg {

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

// Shared-memory slot of FFT element i: one padding slot every 16 elements, so
// the power-of-two strides of the Stockham writes do not hit one bank.
__host__ __device__ __forceinline__ int sp(int i) { return i + (i >> 4); }
// shared-memory slots for an FFT of length L
__host__ __device__ __forceinline__ size_t fft_slots(int L) { return (size_t)L + (size_t)(L >> 4) + 1; }

template <typename T> struct Dft<T, 16> {
    using CT = C2<T>;
    // 16 = 4 x 4: n = 4 n1 + n2, k = k1 + 4 k2,
    // X[k1 + 4 k2] = sum_n2 W16^(n2 k1) W4^(n2 k2) sum_n1 x[4 n1 + n2] W4^(n1 k1)
    __device__ __forceinline__ static void run(CT* v) {
        const T c1 = (T)0.92387953251128675613, s1 = (T)0.38268343236508977173;
        const T h = sqrt_half<T>();
        CT a[4][4];
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) {
            CT t[4] = {v[n2], v[4 + n2], v[8 + n2], v[12 + n2]};
            Dft<T, 4>::run(t);
#pragma unroll
            for (int k1 = 0; k1 < 4; ++k1) a[n2][k1] = t[k1];
        }
        // twiddles W16^m = exp(-2 pi i m / 16)
        a[1][1] = cmul(a[1][1], CT{c1, -s1});
        a[1][2] = cmul(a[1][2], CT{h, -h});
        a[1][3] = cmul(a[1][3], CT{s1, -c1});
        a[2][1] = cmul(a[2][1], CT{h, -h});
        a[2][2] = cmul_mi(a[2][2]);
        a[2][3] = cmul(a[2][3], CT{-h, -h});
        a[3][1] = cmul(a[3][1], CT{s1, -c1});
        a[3][2] = cmul(a[3][2], CT{-h, -h});
        a[3][3] = cmul(a[3][3], CT{-c1, s1});
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            CT t[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
            Dft<T, 4>::run(t);
#pragma unroll
            for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
        }
    }
};

// One Stockham stage of radix R on buf[0, M) (in place, two barriers).
// Every thread owns E/R butterflies.  stw holds this stage's twiddles
// W^(r k) = exp(-2 pi i r k / (Ns R)) at stw[(r - 1) * Ns + k], r in [1, R),
// k in [0, Ns): consecutive threads read consecutive entries.
template <typename T, int E, int R>
__device__ __forceinline__ void stockham_stage(C2<T>* buf, int M, int Ns, const C2<T>* __restrict__ stw) {
    using CT = C2<T>;
    constexpr int B = E / R;
    const int nt = blockDim.x, tid = threadIdx.x;
    const int stride = M / R;
    CT v[E];
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = tid + b * nt;
#pragma unroll
        for (int r = 0; r < R; ++r) v[b * R + r] = buf[sp(j + r * stride)];
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = tid + b * nt;
        const int k = j & (Ns - 1);
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) v[b * R + r] = cmul(v[b * R + r], __ldg(&stw[(r - 1) * Ns + k]));
        }
        Dft<T, R>::run(&v[b * R]);
        const int d = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) buf[sp(d + r * Ns)] = v[b * R + r];
    }
    __syncthreads();
}

template <typename T> struct Dft<T, 1> {
    __device__ __forceinline__ static void run(C2<T>*) {}
};

// radix of the next stage for E values per thread and `bits` = log2 of the
// remaining length; the host builds the stage twiddles with the same rule
__host__ __device__ __forceinline__ int stage_radix(int E, int bits) {
    if (E >= 16 && bits >= 4) return 16;
    if (E >= 8 && bits >= 3) return 8;
    if (E >= 4 && bits >= 2) return 4;
    return 2;
}

// Forward complex FFT of length M = E * blockDim.x (power of two) on shared
// memory (padded slots, sp()), natural order in and out.  stw: the stage
// twiddles of (M, E), stage after stage.
template <typename T, int E>
__device__ void block_fft(C2<T>* buf, int M, int log2M, const C2<T>* __restrict__ stw) {
    int Ns = 1, bits = log2M;
    while (bits > 0) {
        if constexpr (E >= 16) {
            if (bits >= 4) {
                stockham_stage<T, E, 16>(buf, M, Ns, stw);
                stw += 15 * Ns;
                Ns <<= 4;
                bits -= 4;
                continue;
            }
        }
        if constexpr (E >= 8) {
            if (bits >= 3) {
                stockham_stage<T, E, 8>(buf, M, Ns, stw);
                stw += 7 * Ns;
                Ns <<= 3;
                bits -= 3;
                continue;
            }
        }
        if constexpr (E >= 4) {
            if (bits >= 2) {
                stockham_stage<T, E, 4>(buf, M, Ns, stw);
                stw += 3 * Ns;
                Ns <<= 2;
                bits -= 2;
                continue;
            }
        }
        if constexpr (E >= 2) {
            stockham_stage<T, E, 2>(buf, M, Ns, stw);
            stw += Ns;
            Ns <<= 1;
            bits -= 1;
        } else {
            bits = 0;  // E == 1 means M == 1: nothing to do
        }
    }
}

// The same FFT with the length a compile-time constant: every stride, mask
// and thread count below is a constant, so the padded shared-memory offsets
// of a butterfly's R values fold into immediates (a stride that is a multiple
// of 16 moves sp() by a constant) instead of being recomputed per value.
// blockDim.x must be M / E.
template <typename T, int E, int R, int M, int NS>
__device__ __forceinline__ void stockham_stage_ct(C2<T>* buf, const C2<T>* __restrict__ stw) {
    using CT = C2<T>;
    constexpr int B = E / R, NT = M / E, STRIDE = M / R;
    const int tid = threadIdx.x;
    CT v[E];
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = tid + b * NT;
#pragma unroll
        for (int r = 0; r < R; ++r) v[b * R + r] = buf[sp(j + r * STRIDE)];
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = tid + b * NT;
        const int k = j & (NS - 1);
        if constexpr (NS > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) v[b * R + r] = cmul(v[b * R + r], __ldg(&stw[(r - 1) * NS + k]));
        }
        Dft<T, R>::run(&v[b * R]);
        const int d = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) buf[sp(d + r * NS)] = v[b * R + r];
    }
    __syncthreads();
}

template <typename T, int E, int M, int NS, int BITS>
__device__ __forceinline__ void block_fft_ct_rec(C2<T>* buf, const C2<T>* __restrict__ stw) {
    if constexpr (BITS > 0) {
        constexpr int R = (E >= 16 && BITS >= 4) ? 16 : (E >= 8 && BITS >= 3) ? 8 : (E >= 4 && BITS >= 2) ? 4 : 2;
        constexpr int RB = R == 16 ? 4 : R == 8 ? 3 : R == 4 ? 2 : 1;
        stockham_stage_ct<T, E, R, M, NS>(buf, stw);
        block_fft_ct_rec<T, E, M, NS * R, BITS - RB>(buf, stw + (R - 1) * NS);
    }
}

// LG > 0: the compile-time FFT of length 2^LG (L must equal it); LG == 0:
// the run-time one
template <typename T, int E, int LG>
__device__ __forceinline__ void block_fft_sel(C2<T>* buf, int L, const C2<T>* __restrict__ stw) {
    if constexpr (LG > 0) {
        block_fft_ct_rec<T, E, (1 << LG), 1, LG>(buf, stw);
    } else {
        block_fft<T, E>(buf, L, 31 - __clz(L), stw);
    }
}

// Stage twiddles of a length-L FFT with E values per thread (host side):
// for each stage (radix R, span Ns), W^(r k) for r in [1, R), k in [0, Ns),
// evaluated in long double.
template <typename T> inline std::vector<C2<T>> stage_twiddles(int L, int E) {
    std::vector<C2<T>> out;
    int bits = 0;
    while ((1 << bits) < L) ++bits;
    int Ns = 1;
    const long double two_pi = 6.283185307179586476925286766559005768L;
    while (bits > 0) {
        const int R = stage_radix(E, bits);
        int rb = 0;
        while ((1 << rb) < R) ++rb;
        for (int r = 1; r < R; ++r)
            for (int k = 0; k < Ns; ++k) {
                const long double a = -two_pi * (long double)r * (long double)k / ((long double)Ns * R);
                C2<T> w;
                w.x = (T)cosl(a);
                w.y = (T)sinl(a);
                out.push_back(w);
            }
        Ns *= R;
        bits -= rb;
    }
    if (out.empty()) out.push_back(C2<T>{(T)1, (T)0});
    return out;
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
    const CT za = Z[sp(k == M ? 0 : k)];
    const CT zb = Z[sp(k == 0 ? 0 : M - k)];
    // Ek = (za + conj(zb))/2 ; Ok = (za - conj(zb))/(2i)
    const T h = (T)0.5;
    const CT e = CT{h * (za.x + zb.x), h * (za.y - zb.y)};
    const T pr = za.x - zb.x, pi = za.y + zb.y;
    const CT o = CT{h * pi, -h * pr};
    const CT w = __ldg(&tw[k]);  // exp(-2 pi i k / N), N = 2M
    return cadd(e, cmul(o, w));
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


// ---------------------------------------------------------------------------
// Mixed-radix Stockham FFT (radices 2, 3, 4, 5, 7) for lengths that are not
// powers of two: the same autosort scheme as block_fft (Govindaraju et al.,
// SC 2008), one radix-R stage after the other with Ns = the product of the
// previous radices: for j < L/R, k = j mod Ns, the R values
// in[j + m L/R] times exp(-2 pi i m k / (Ns R)) go through an R-point DFT and
// land at out[(j / Ns) Ns R + k + m Ns].  Stages alternate between two
// shared-memory buffers.  Twiddles and the R-th roots of unity come from a
// table built on the host in long double (MixPlan offsets).
// ---------------------------------------------------------------------------
constexpr int kMixMaxStages = 24;
struct MixPlan {
    int L, nst;
    int R[kMixMaxStages], Ns[kMixMaxStages], off[kMixMaxStages];
    int root_off[8];  // offset of exp(-2 pi i j / R), j < R, for R = 3, 5, 7
};

template <typename T, int R>
__device__ __forceinline__ void mix_dft(C2<T>* x, const C2<T>* __restrict__ root) {
    using CT = C2<T>;
    if constexpr (R == 2) {
        const CT a = x[0], b = x[1];
        x[0] = cadd(a, b);
        x[1] = CT{a.x - b.x, a.y - b.y};
    } else if constexpr (R == 4) {
        const CT t0 = cadd(x[0], x[2]), t1 = CT{x[0].x - x[2].x, x[0].y - x[2].y};
        const CT t2 = cadd(x[1], x[3]), d = CT{x[1].x - x[3].x, x[1].y - x[3].y};
        const CT t3 = CT{d.y, -d.x};  // -i (x1 - x3)
        x[0] = cadd(t0, t2);
        x[2] = CT{t0.x - t2.x, t0.y - t2.y};
        x[1] = cadd(t1, t3);
        x[3] = CT{t1.x - t3.x, t1.y - t3.y};
    } else {
        CT w[R];
#pragma unroll
        for (int j = 0; j < R; ++j) w[j] = __ldg(&root[j]);
        CT y[R];
#pragma unroll
        for (int q = 0; q < R; ++q) {
            CT acc = x[0];
#pragma unroll
            for (int m = 1; m < R; ++m) acc = cadd(acc, cmul(x[m], w[(m * q) % R]));
            y[q] = acc;
        }
#pragma unroll
        for (int q = 0; q < R; ++q) x[q] = y[q];
    }
}

template <typename T, int R>
__device__ __forceinline__ void mix_stage(const C2<T>* in, C2<T>* out, int L, int Ns, const C2<T>* __restrict__ tw,
                                          const C2<T>* __restrict__ root) {
    using CT = C2<T>;
    const int nb = L / R;
    for (int j = threadIdx.x; j < nb; j += blockDim.x) {
        const int k = j % Ns;
        CT x[R];
#pragma unroll
        for (int m = 0; m < R; ++m) x[m] = in[j + m * nb];
        if (Ns > 1) {
#pragma unroll
            for (int m = 1; m < R; ++m) x[m] = cmul(x[m], __ldg(&tw[(m - 1) * Ns + k]));
        }
        mix_dft<T, R>(x, root);
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int m = 0; m < R; ++m) out[base + m * Ns] = x[m];
    }
}

// the transform of the L values in a (b: scratch of L values); returns the
// buffer that holds the result, in natural order
template <typename T>
__device__ C2<T>* block_fft_mixed(C2<T>* a, C2<T>* b, const MixPlan& p, const C2<T>* __restrict__ tab) {
    C2<T>* in = a;
    C2<T>* out = b;
    for (int s = 0; s < p.nst; ++s) {
        const int R = p.R[s], Ns = p.Ns[s];
        const C2<T>* tw = tab + p.off[s];
        switch (R) {
            case 2: mix_stage<T, 2>(in, out, p.L, Ns, tw, nullptr); break;
            case 4: mix_stage<T, 4>(in, out, p.L, Ns, tw, nullptr); break;
            case 3: mix_stage<T, 3>(in, out, p.L, Ns, tw, tab + p.root_off[3]); break;
            case 5: mix_stage<T, 5>(in, out, p.L, Ns, tw, tab + p.root_off[5]); break;
            default: mix_stage<T, 7>(in, out, p.L, Ns, tw, tab + p.root_off[7]); break;
        }
        __syncthreads();
        C2<T>* t = in;
        in = out;
        out = t;
    }
    return in;
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

// ---------------------------------------------------------------------------
// Transform of a real sequence even about index 0 (a DCT-I): with period
// N = 2n, s[0] = x_0, s[+-j] = x_j (0 < j < n), s[n] = x_n,
//   C_k = sum_J s[J] exp(-2 pi i J k / N)
//       = x_0 + (-1)^k x_n + 2 sum_{j=1}^{n-1} x_j cos(pi j k / n),  k in [0, kmax],
// from one complex FFT of length n/2 (a quarter of N).  With
//   y_0 = (x_0 + x_n)/2,  y_j = (x_j + x_{n-j})/2 - sin(pi j/n) (x_j - x_{n-j}),
// and Y = DFT_n(y): the part of y odd about n/2 drops out of Re Y_k and the
// part even about n/2 out of Im Y_k, and the product-to-sum identity
// 2 sin(a) sin(2ka) = cos((2k-1)a) - cos((2k+1)a) gives
//   C_{2k} = 2 Re Y_k,   C_{2k+1} = C_{2k-1} - 2 Im Y_k,
//   C_1 = (x_0 - x_n) + 2 sum_{j=1}^{n-1} x_j cos(pi j/n),
// so the odd outputs are C_1 minus twice a prefix sum of Im Y (the cosine
// transform algorithm of Numerical Recipes' cosft1, derived here with the
// forward sign of this code).  Y comes from the length-n/2 complex FFT of
// y_{2m} + i y_{2m+1} and the even/odd split.  Block-wide: blockDim.x =
// n / (2E) threads, at least 32.
//   xs   x_0 .. x_{nnz-1} in shared memory (x_j = 0 for nnz <= j < n); xn = x_n
//   twN  exp(-2 pi i j / N), j < N;  stw: stage twiddles of the length-n/2 FFT
//   buf  fft_slots(n/2) complex;  im: n/2 + 1 reals;  out: kmax + 1 reals
//        (may alias xs: xs is read only before the transform)
// Sums are in FP64 in a fixed order (reproducible).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ C2<T> real_split_stride2(const C2<T>* Z, int M, int k, const C2<T>* __restrict__ twN) {
    using CT = C2<T>;
    const CT za = Z[sp(k == M ? 0 : k)];
    const CT zb = Z[sp(k == 0 ? 0 : M - k)];
    const T h = (T)0.5;
    const CT e = CT{h * (za.x + zb.x), h * (za.y - zb.y)};
    const T pr = za.x - zb.x, pi = za.y + zb.y;
    const CT o = CT{h * pi, -h * pr};
    const CT w = __ldg(&twN[2 * k]);  // exp(-2 pi i k / n), n = 2M
    return cadd(e, cmul(o, w));
}

template <typename T, int E>
__device__ void even_dft_block(const T* xs, int nnz, T xn, int n, const C2<T>* __restrict__ twN,
                               const C2<T>* __restrict__ stw, C2<T>* buf, T* im, T* out, int kmax) {
    using CT = C2<T>;
    __shared__ double sh[32];
    __shared__ double c1_sh;
    const int t = threadIdx.x, bd = blockDim.x;
    const int M = n / 2;
    // C_1
    double acc = 0.0;
    for (int j = 1 + t; j < nnz; j += bd) acc += (double)xs[j] * (double)__ldg(&twN[j]).x;
    const double s = block_sum(acc, sh);
    if (t == 0) c1_sh = ((nnz > 0 ? (double)xs[0] : 0.0) - (double)xn) + 2.0 * s;
    // y packed as z_m = y_{2m} + i y_{2m+1}
    for (int m = t; m < M; m += bd) {
        T y[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int j = 2 * m + h;
            if (j == 0) {
                y[h] = (T)0.5 * ((nnz > 0 ? xs[0] : (T)0) + xn);
            } else {
                const T xj = j < nnz ? xs[j] : (T)0;
                const T xm = (n - j) < nnz ? xs[n - j] : (T)0;
                const T sj = -__ldg(&twN[j]).y;  // sin(pi j / n)
                y[h] = (T)0.5 * (xj + xm) - sj * (xj - xm);
            }
        }
        buf[sp(m)] = CT{y[0], y[1]};
    }
    __syncthreads();
    block_fft<T, E>(buf, M, 31 - __clz(M), stw);
    __syncthreads();
    const int kh = kmax / 2;  // Y_k for k <= kh gives C_0 .. C_kmax
    for (int k = t; k <= kh; k += bd) {
        const CT Y = real_split_stride2<T>(buf, M, k, twN);
        out[2 * k] = (T)2 * Y.x;
        im[k] = Y.y;
    }
    __syncthreads();
    // odd outputs: C_{2k+1} = C_1 - 2 sum_{i=1}^{k} Im Y_i (warp 0: contiguous
    // segments per lane, a shuffle scan of the segment sums, then the segments)
    if (t < 32) {
        const int L = (kmax - 1) / 2;  // odd outputs 3, 5, .., need prefixes up to L
        const int seg = (L + 31) / 32;
        const int b0 = 1 + t * seg, b1 = min(b0 + seg, L + 1);
        double loc = 0.0;
        for (int i = b0; i < b1; ++i) loc += (double)im[i];
        double incl = loc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double v = __shfl_up_sync(0xffffffffu, incl, o);
            if (t >= o) incl += v;
        }
        double run = __shfl_up_sync(0xffffffffu, incl, 1);
        if (t == 0) run = 0.0;
        const double c1 = c1_sh;
        if (t == 0 && kmax >= 1) out[1] = (T)c1;
        for (int i = b0; i < b1; ++i) {
            run += (double)im[i];
            out[2 * i + 1] = (T)(c1 - 2.0 * run);
        }
    }
    __syncthreads();
}

// Deterministic grid reduction: each block writes its partial, the last block
// to arrive sums the partials with all its threads: thread i takes partials
// i, i + blockDim, ... in order, then a fixed-shape tree (block_sum).  The
// summation order depends only on the grid size, so results are reproducible.
// A reduction split over several launches (chunks of the visibilities, which
// may run concurrently on two streams): the launch whose blocks are numbered
// from `off` writes partials[off + b], every block of every launch takes a
// ticket, and the block that takes ticket nparts - 1 (nparts = all launches'
// blocks) sums partials[0, nparts) in the fixed order.
__device__ __forceinline__ void grid_finish(double block_total, double* partials, DevState* st,
                                            double* extra_out = nullptr, int off = 0, int nparts_all = 0) {
    __shared__ bool last;
    __shared__ double sh2[32];
    const unsigned nparts = nparts_all > 0 ? (unsigned)nparts_all : gridDim.x;
    if (threadIdx.x == 0) {
        partials[off + blockIdx.x] = block_total;
        __threadfence();
        const unsigned t = atomicAdd(&st->ticket, 1u);
        last = (t == nparts - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s = 0.0;
    const volatile double* p = partials;
    for (unsigned b = threadIdx.x; b < nparts; b += blockDim.x) s += p[b];
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
// Block sum of FP32 values: double-float warp sums (FP32 instructions only;
// GB300's FP64 pipe runs at a 64th of the FP32 rate), the warp totals added in
// FP64 by thread 0.  Valid in thread 0.
__device__ __forceinline__ double block_sum_df(float x, double* sh) {
    DF s{x, 0.f};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h = __shfl_xor_sync(0xffffffffu, s.hi, o);
        const float l = __shfl_xor_sync(0xffffffffu, s.lo, o);
        s = df_add(s, DF{h, l});
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = (double)s.hi + (double)s.lo;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < nw; ++q) t += sh[q];
    return t;  // valid in thread 0
}
// floor of x = hi + lo (|hi| < 2^22, |lo| at most a few ulps of hi) as an
// integer and the fraction in [0, 1]: n = rint(hi) by the magic-number
// method, hi - n is exact (Sterbenz), f = (hi - n) + lo lies in
// [-1/2 - tiny, 1/2 + tiny], and a negative f moves to the integer below.
__device__ __forceinline__ void df_floor(DF x, int* fl, float* frac) {
    const float r = __fadd_rn(x.hi, kMagic);
    float f = __fadd_rn(__fsub_rn(x.hi, __fsub_rn(r, kMagic)), x.lo);
    int n = __float_as_int(r) - kMagicBits;
    if (f < 0.f) {
        n -= 1;
        f = __fadd_rn(f, 1.f);
    }
    *fl = n;
    *frac = f;
}

// sin/cos(2 pi (j/4 + d)) for |d| <= 1/8 + tiny: x = 2 pi d, |x| <= pi/4,
// Taylor series to x^9 (sin) and x^8 (cos), truncation error below 3e-8, then
// the rotation by i^j as a swap and two sign-bit flips.
__device__ __forceinline__ void sincos2pi_quadrant(float d, unsigned j, float* s, float* c) {
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
    // i^j: (s, c) = (sx, cx), (cx, -sx), (-sx, -cx), (-cx, sx) for j = 0..3 (mod 4)
    const bool odd = j & 1u;
    const float so = odd ? cx : sx, co = odd ? sx : cx;
    *s = __int_as_float(__float_as_int(so) ^ (int)((j & 2u) << 30));
    *c = __int_as_float(__float_as_int(co) ^ (int)(((j + 1u) & 2u) << 30));
}

// sin/cos(2 pi (hi + lo)) for a double-float argument in turns (|hi| < 2^41,
// |lo| at most a few ulps of hi), all in FP32: exact reductions by a whole
// multiple of 2^20 turns (|h| <= 2^19 afterwards) and by quarter turns, each
// with one magic-number rounding and one Sterbenz subtraction, then
// d = (h - j/4) + lo and sincos2pi_quadrant.
__device__ __forceinline__ void sincos2pi_df(DF ph, float* s, float* c) {
    const float kb = __fsub_rn(__fmaf_rn(ph.hi, 0x1p-20f, kMagic), kMagic);
    const float h = __fmaf_rn(kb, -0x1p20f, ph.hi);
    const float r = __fmaf_rn(h, 4.f, kMagic);
    const float d = __fadd_rn(__fmaf_rn(__fsub_rn(r, kMagic), -0.25f, h), ph.lo);
    sincos2pi_quadrant(d, (unsigned)(__float_as_int(r) - kMagicBits), s, c);
}


// sin/cos(2 pi a), a in cycles, FP64, table-driven (Tang's method): a = m/T
// + d with m = rint(a T) and |d| <= 1/(2T), T = 2^20.  a T + 1.5 * 2^52
// (exact product, one rounding for |a T| < 2^51) holds m in its low mantissa
// bits, so the table index m mod T comes from the bit pattern without a
// conversion; d = a - m/T is exact (Sterbenz), x = 2 pi d with |x| <= pi/T =
// 3.0e-6, so cos x = 1 - x^2/2 and sin x = x leave out at most x^3/6 < 4.5e-18
// in absolute terms.  exp(2 pi i a) = E (1 - h + i x) with h = x^2/2:
// cos = E.x - E.x h - E.y x, sin = E.y + E.x x - E.y h in fused multiply-adds.
// The table E[j] = exp(2 pi i j / T) is built on the host (1 ulp).
__device__ __forceinline__ void sincos2pi_tab(double a, const double2* __restrict__ tab, double* s, double* c) {
    constexpr double kMagic52 = 6755399441055744.0;  // 1.5 * 2^52
    const double r = fma(a, (double)PHASE_T, kMagic52);
    const int j = __double2loint(r) & (PHASE_T - 1);
    const double d = fma(r - kMagic52, -1.0 / (double)PHASE_T, a);
    const double x = d * 6.283185307179586476925286766559;
    const double h = (0.5 * x) * x;
    const double2 e = __ldg(&tab[j]);
    *c = fma(-e.x, h, fma(-e.y, x, e.x));
    *s = fma(-e.y, h, fma(e.x, x, e.y));
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


template <typename T> int max_fft_n_impl() { return sizeof(T) == 8 ? 8192 : 16384; }

// dispatch helper: launch a shared-memory FFT kernel with E elements per thread
template <typename T> struct FftCfg {
    int E, threads;
    size_t smem;
};
template <typename T> FftCfg<T> fft_cfg(int M) {
    FftCfg<T> c;
    // FP32: radix-16 stages once there are 32+ threads; FP64 keeps 8 values per
    // thread (16 double2 per thread costs too many registers)
    if (M >= 16384 || (sizeof(T) == 4 && M >= 512)) c.E = 16;
    else if (M >= 8) c.E = 8;
    else c.E = M < 1 ? 1 : M;
    c.threads = M / c.E < 1 ? 1 : M / c.E;
    c.smem = sizeof(C2<T>) * fft_slots(M < 1 ? 1 : M);
    return c;
}

// values per thread of the shared-memory FFT of length M in precision T
template <typename T> inline int fft_e(int M) { return fft_cfg<T>(M).E; }

// shared memory of the even-sequence transform kernels of length N: the
// length-N/4 FFT buffer, the N/2 + 1 half sequence and N/4 + 1 scratch reals
template <typename T> inline size_t even_dft_smem(int N) {
    return sizeof(C2<T>) * fft_slots(N / 4) + sizeof(T) * ((size_t)N / 2 + 1) + sizeof(T) * ((size_t)N / 4 + 1);
}
// values per thread of the even-sequence transforms' length-N/4 FFT (those
// of the plain FFT; 4 per thread, with twice the warps, measured slower)
template <typename T> inline int even_dft_e(int N) { return fft_cfg<T>(N / 4).E; }
// the even-sequence transforms need a power-of-two N, a length-N/4 FFT with
// at least one warp of threads, and shared memory within a block's limit
template <typename T> inline bool even_dft_ok(int N) {
    if (!is_pow2(N) || N < 16 || N / 4 > max_fft_n_impl<T>()) return false;
    const int threads = (N / 4) / even_dft_e<T>(N);
    return threads >= 32 && threads <= 1024 && even_dft_smem<T>(N) <= 200 * 1024;
}

template <typename K> cudaError_t set_smem(K kernel, size_t smem) {
    if (smem > 48 * 1024) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return cudaSuccess;
}

// Reals per record of a real spectrum: FP32, the 4 corners; FP64, the 4
// coefficients of the bilinear modulus and the 4 corners as FP32 (4 floats in
// the space of 2 doubles; 48-byte records).
template <typename T> __host__ __device__ constexpr int real_rec() { return sizeof(T) == 8 ? 6 : 4; }

}  // namespace gbg
