// Batched FP32 chi2 of B models (radial profiles or images) against one
// device-resident dataset, with the gradient of every chi2 with respect to
// the model (profile samples or pixels), the inclination, the position angle
// and the offsets.
//
// Forward (per model b, all models in the same launches):
//   model_setup   per-model constants (rotation, offsets, 1/cos inc, central pixel)
//   rows          sweep fused into the shared-memory real FFT of each non-zero
//                 image row (or the rows of a given image)
//   cols          column FFT of the K needed columns -> window elements
//                 (re, im, modulus) as one float4 each
//   vis           for every visibility, all B models: double-float index and
//                 phase, the four corners of its cell gathered from the
//                 window, bilinear amp/phase interpolation, residual, chi2
// Adjoint (reverse mode; the spectrum is recomputed by the forward launches
// of the same call, not stored between calls):
//   vis           dchi2/dV = 2 w (V - obs) -> through the phase shift (dRA,
//                 dDec), the modulus/argument interpolation (cell-corner
//                 gradients, summed over runs of equal cells and added with
//                 float4 atomics into per-cell records) and the
//                 interpolation position (PA)
//   quadT         per-cell records -> gradient of every window element,
//                 plus the modulus part times S/|S|, times the output sign
//   colsT         inverse column FFT (the adjoint of the forward column FFT)
//   rowsT         inverse real FFT of each image row with Hermitian weights
//                 (the adjoint of the R2C row transform), times the row sign,
//                 fused with the adjoint of the sweep (profile samples, inc)
//   central       adjoint of the central-pixel average
// Reference semantics followed: sweep_core src/galario.cpp:1048-1071, central
// pixel :1136-1153, interpolate_core :749-815, apply_phase_sampled_core
// :877-884, uv_rotate_core :955-960, reduce_chi2 :1504-1538.
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/galario_gb300.h"
#include "gb_device.cuh"
#include "gb_internal.cuh"
#include "gb_tc.cuh"
#include "gb_tune.h"

namespace gbg {
void set_error_message(const std::string& msg);  // gb_api.cu

namespace {

constexpr int kVisThreads = 256;
// threads of a vis block with PTS visibilities per thread: spans of 512 or
// 1024 visibilities, so that no block straddles two sets (kSetAlign)
constexpr int vis_threads(int pts) { return pts >= 8 ? 1024 / pts : kVisThreads; }
constexpr int kRowsPerCta = 16;  // folded image rows (up to two box rows each) per CTA in the row adjoint
constexpr int kGRec = 12;       // floats per gradient cell record
constexpr int kTmaCols = 100;   // column-pass shape code: E + kTmaCols selects the TMA-fed variant

struct ModelConst {
    DF cu, sv;            // cos(PA) / duv, sin(PA) / duv: (u, v) -> rotated grid coordinates
    DF dra, ddec;         // offsets (radians); the phase u'dRA' + v'dDec' = u dRA + v dDec
    float inv_cos_inc;    // 1 / cos(inc)
    float tan_inc;        // tan(inc)
    float central;        // central pixel value (Jy/pixel)
    int phase;
    float pad[4];
};

struct Geo {  // geometry shared by all models of a batch
    int N, M, C, K, r0, W, rmax, band0, R, nr, iIN;
    float Rmin, dR, inv_dR, dxy, sr_to_px;
    float inv_duv_hi, inv_duv_lo, half_nrow;
    float vo;  // v_origin: profiles use origin 'upper' (+1)
};

// ---------------------------------------------------------------------------
// forward kernels
// ---------------------------------------------------------------------------
// params per model: (inc, PA, dRA, dDec) for profiles (pstride 4), (PA, dRA,
// dDec) for images (pstride 3, no inclination)
__global__ void model_setup_kernel(int B, const float* __restrict__ params, int pstride,
                                   const float* __restrict__ intensity, int nr,
                                   const double* __restrict__ central_coef, int ncoef, double inv_duv,
                                   ModelConst* mc) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float* pb = params + (size_t)pstride * b + (pstride - 3);
    const double inc = pstride == 4 ? params[(size_t)4 * b] : 0.0;
    const double PA = pb[0], dRA = pb[1], dDec = pb[2];
    ModelConst m;
    auto split = [](double x) {
        DF r;
        r.hi = (float)x;
        r.lo = (float)(x - (double)r.hi);
        return r;
    };
    const double c = (PA != 0.0) ? cos(PA) : 1.0, s = (PA != 0.0) ? sin(PA) : 0.0;
    m.cu = split(c * inv_duv);
    m.sv = split(s * inv_duv);
    m.dra = split(dRA);
    m.ddec = split(dDec);
    m.phase = !(dRA == 0.0 && dDec == 0.0);
    const double ci = cos(inc);
    m.inv_cos_inc = (float)(1.0 / ci);
    m.tan_inc = (float)tan(inc);
    double cen = 0.0;
    const float* I = intensity + (size_t)b * nr;
    for (int i = 0; i < ncoef; ++i) cen += central_coef[i] * (double)I[i];
    m.central = (float)cen;
    m.pad[0] = m.pad[1] = m.pad[2] = m.pad[3] = 0.f;
    mc[b] = m;
}

// The swept image depends on (|x|, |y|) only: pixel (i, j) of the 2 rmax box
// has the value of the folded pixel (a, c) = (|rmax - i|, |rmax - j|).  A CTA
// takes F consecutive folded rows a0..a0+F-1; for each it evaluates the
// rmax + 1 folded pixels once and transforms the box rows rmax - a and
// rmax + a (one row for a = 0 and for a = rmax, whose mirror rmax + a = 2 rmax
// lies outside the box).  The 2F transformed rows are two runs of
// consecutive box rows, staged in shared memory and written column by column
// as contiguous runs of the row-major-transposed layout zt[b][k][row].
// e = k * n + j with 0 <= j < n, for e < 2^22, without the integer divider
// (whose float conversions run on the slow conversion pipe)
__device__ __forceinline__ void split_index(int e, int n, float inv_n, int* k, int* j) {
    float fl;
    int q = floor_i((i2f_small(e) + 0.5f) * inv_n, &fl);
    int r = e - q * n;
    if (r < 0) { --q; r += n; }
    if (r >= n) { ++q; r -= n; }
    *k = q;
    *j = r;
}

__device__ __forceinline__ int fold_rows(const Geo& g, int a0, int F, int* lo0, int* lo1, int* n1) {
    const int n0 = min(F, g.rmax + 1 - a0);  // folded rows of this CTA
    *lo0 = g.rmax - (a0 + n0 - 1);           // side 0: box rows rmax - a, a in [a0, a0 + n0)
    const int s1 = max(a0, 1);               // side 1: box rows rmax + a, 1 <= a <= rmax - 1
    const int e1 = min(a0 + n0, g.rmax);
    *lo1 = g.rmax + s1;
    *n1 = max(0, e1 - s1);
    return n0;
}

template <int E, int MAXT, int LG>
__global__ void __launch_bounds__(MAXT) rows_batch_kernel(Geo g, int F, const float* __restrict__ intensity,
                                                          const ModelConst* __restrict__ mc,
                                                          const float2* __restrict__ tw,
                                                          const float2* __restrict__ stw, void* __restrict__ zt_any,
                                                          int real_out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* buf = reinterpret_cast<float2*>(smem_raw);
    const int S = 2 * F + 1;                                  // staging row stride (odd: no bank conflicts)
    float2* stg = buf + fft_slots(g.M);                       // [K][S] staged outputs
    float* val = reinterpret_cast<float*>(stg + (size_t)g.K * S);  // rmax + 1 folded pixels
    const int b = blockIdx.y;
    const int a0 = blockIdx.x * F;
    int lo0, lo1, n1;
    const int n0 = fold_rows(g, a0, F, &lo0, &lo1, &n1);
    const int off = g.N / 2 - g.rmax;
    const float* Ib = intensity + (size_t)b * g.nr;
    const ModelConst m = mc[b];
    for (int aa = 0; aa < n0; ++aa) {
        const int a = a0 + aa;
        __syncthreads();  // val and buf free
        for (int c = threadIdx.x; c <= g.rmax; c += blockDim.x)
            val[c] = sweep_pixel<float>(off + g.rmax - a, off + g.rmax - c, Ib, g.nr, g.Rmin, g.dR, g.inv_dR, g.dxy,
                                        m.inv_cos_inc, g.rmax, off, g.sr_to_px);
        // the mirror rows rmax - a and rmax + a hold the same pixels and have
        // the same row-sign parity: one transform serves both
        const int I = off + g.rmax - a;
        const int slot0 = (g.rmax - a) - lo0;
        const bool mirror = a > 0 && a < g.rmax;
        const int slot1 = mirror ? F + (g.rmax + a - lo1) : -1;
        __syncthreads();  // val ready; buf free
        for (int mm = threadIdx.x; mm < g.M; mm += blockDim.x) {
            const int j0 = 2 * mm - off, j1 = j0 + 1;
            float x0 = 0.f, x1 = 0.f;
            if (j0 >= 0 && j0 < 2 * g.rmax) x0 = val[abs(g.rmax - j0)];
            if (j1 >= 0 && j1 < 2 * g.rmax) x1 = val[abs(g.rmax - j1)];
            if (I == g.N / 2) {
                if (2 * mm == g.N / 2) x0 = m.central;
                if (2 * mm + 1 == g.N / 2) x1 = m.central;
            }
            buf[sp(mm)] = make_float2(x0, x1);
        }
        __syncthreads();
        block_fft_sel<float, E, LG>(buf, g.M, stw);
        const float sgn = (I & 1) ? -1.f : 1.f;
        for (int k = threadIdx.x; k < g.K; k += blockDim.x) {
            const float2 x = real_split<float>(buf, g.M, k, tw);
            const float2 y = make_float2(sgn * x.x, sgn * x.y);
            stg[k * S + slot0] = y;
            if (mirror) stg[k * S + slot1] = y;
        }
    }
    __syncthreads();
    // real_out: the swept image is even in x, so the row transforms are real
    // (up to rounding); only the real parts are kept, as floats
    const int nrun = n0 + n1;
    const float inv_nrun = 1.f / i2f_small(nrun);
    float2* out = static_cast<float2*>(zt_any) + (size_t)b * g.K * g.R;
    float* outr = static_cast<float*>(zt_any) + (size_t)b * g.K * g.R;
    for (int e = threadIdx.x; e < g.K * nrun; e += blockDim.x) {
        int k, j;
        split_index(e, nrun, inv_nrun, &k, &j);
        const int row = j < n0 ? lo0 + j : lo1 + (j - n0);
        const int slot = j < n0 ? j : F + (j - n0);
        if (real_out) outr[(size_t)k * g.R + row] = stg[k * S + slot].x;
        else out[(size_t)k * g.R + row] = stg[k * S + slot];
    }
}

// Column pass of real, even columns (swept profiles): columns k1 = 2p and
// k2 = 2p + 1 are the real and the imaginary part of one complex transform,
// whose real and imaginary outputs are their (real) transforms.  Writes one
// float per window element (output sign applied).
template <int E, int MAXT, int LG>
__global__ void __launch_bounds__(MAXT) cols_pair_batch_kernel(Geo g, const float* __restrict__ ztr,
                                                               const float2* __restrict__ stw,
                                                               float* __restrict__ wr) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* buf = reinterpret_cast<float2*>(smem_raw);
    const int b = blockIdx.y, k1 = 2 * blockIdx.x, k2 = k1 + 1;
    const bool two = k2 < g.K;
    const float* c1 = ztr + ((size_t)b * g.K + k1) * g.R;
    const float* c2 = c1 + g.R;
    for (int i = threadIdx.x; i < g.N; i += blockDim.x) {
        const int q = i - g.band0;
        const bool in = q >= 0 && q < g.R;
        buf[sp(i)] = make_float2(in ? __ldg(&c1[q]) : 0.f, (in && two) ? __ldg(&c2[q]) : 0.f);
    }
    __syncthreads();
    block_fft_sel<float, E, LG>(buf, g.N, stw);
    const int par1 = (k1 + g.N / 2) & 1;
    float* w1 = wr + ((size_t)b * g.K + k1) * g.W;
    float* w2 = w1 + g.W;
    for (int q = threadIdx.x; q < g.W; q += blockDim.x) {
        const int r = g.r0 + q;
        const float2 x = buf[sp(r)];
        const bool flip1 = ((r & 1) ^ par1) != 0;  // k2 has the opposite output-sign parity
        w1[q] = flip1 ? -x.x : x.x;
        if (two) w2[q] = flip1 ? x.y : -x.y;
    }
}

// Cell gradients of a real window -> gradient of every element: the sum of
// the corner sums of the (up to) four cells that have it as a corner, times
// sign(y) (dchi2/dA -> dchi2/dy through |y|), times the output sign.  Grid (K, B).
__global__ void quadT_real_kernel(Geo g, const float* __restrict__ cgrad4, const float* __restrict__ wr,
                                  float* __restrict__ gwr) {
    const long long ncell = (long long)g.K * g.W;
    const int k = blockIdx.x, b = blockIdx.y;
    const float* cg = cgrad4 + (size_t)b * ncell * 4;
    for (int q = threadIdx.x; q < g.W; q += blockDim.x) {
        float ga = 0.f;
        auto take = [&](int kc, int qc, int c) {
            if (kc < 0 || qc < 0 || kc >= g.K || qc >= g.W) return;
            ga += cg[((long long)kc * g.W + qc) * 4 + c];
        };
        take(k, q, 0);
        take(k, q - 1, 1);
        take(k - 1, q - 1, 2);
        take(k - 1, q, 3);
        const size_t el = (size_t)b * ncell + (size_t)k * g.W + q;
        const float y = wr[el];
        ga *= 2.f;  // the vis pass records halves of dchi2/dA
        float gy = y < 0.f ? -ga : (y > 0.f ? ga : 0.f);
        const int row = g.r0 + q;
        if (((row + k + g.N / 2) & 1)) gy = -gy;
        gwr[el] = gy;
    }
}

// Adjoint of cols_pair_batch_kernel.  The forward keeps the real part of the
// transform of a real column, whose adjoint is Re(FFT(g)); only its part even
// about row N/2 matters (the row adjoint adds mirror rows), and that is the
// transform of the even part of g, which is real: so two columns again share
// one complex transform.  Writes (value, 0) per band row, the row adjoint's
// complex layout.
template <int E, int MAXT, int LG>
__global__ void __launch_bounds__(MAXT) colsT_pair_batch_kernel(Geo g, const float* __restrict__ gwr,
                                                                const float2* __restrict__ stw,
                                                                float2* __restrict__ zbar) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* buf = reinterpret_cast<float2*>(smem_raw);
    const int b = blockIdx.y, k1 = 2 * blockIdx.x, k2 = k1 + 1;
    const bool two = k2 < g.K;
    const float* c1 = gwr + ((size_t)b * g.K + k1) * g.W;
    const float* c2 = c1 + g.W;
    auto at = [&](const float* c, int r) {  // element of window row r (0 outside the window)
        const int q = r - g.r0;
        return (q >= 0 && q < g.W) ? __ldg(&c[q]) : 0.f;
    };
    for (int i = threadIdx.x; i < g.N; i += blockDim.x) {
        const int m = (g.N - i) & (g.N - 1);
        const float e1 = 0.5f * (at(c1, i) + at(c1, m));
        const float e2 = two ? 0.5f * (at(c2, i) + at(c2, m)) : 0.f;
        buf[sp(i)] = make_float2(e1, e2);
    }
    __syncthreads();
    block_fft_sel<float, E, LG>(buf, g.N, stw);
    float2* o1 = zbar + ((size_t)b * g.K + k1) * g.R;
    float2* o2 = o1 + g.R;
    for (int q = threadIdx.x; q < g.R; q += blockDim.x) {
        const float2 x = buf[sp(g.band0 + q)];
        o1[q] = make_float2(x.x, 0.f);
        if (two) o2[q] = make_float2(x.y, 0.f);
    }
}

template <int E, int MAXT, int LG>
__global__ void __launch_bounds__(MAXT) cols_batch_kernel(Geo g, const float2* __restrict__ zt,
                                                          const float2* __restrict__ stw, float4* __restrict__ wel) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* buf = reinterpret_cast<float2*>(smem_raw);
    const int b = blockIdx.y, k = blockIdx.x;
    const float2* col = zt + ((size_t)b * g.K + k) * g.R;
    for (int i = threadIdx.x; i < g.N; i += blockDim.x) {
        const int q = i - g.band0;
        buf[sp(i)] = (q >= 0 && q < g.R) ? __ldg(&col[q]) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    block_fft_sel<float, E, LG>(buf, g.N, stw);
    const int par = (k + g.N / 2) & 1;
    float4* wcol = wel + ((size_t)b * g.K + k) * g.W;
    for (int q = threadIdx.x; q < g.W; q += blockDim.x) {
        const int r = g.r0 + q;
        float2 x = buf[sp(r)];
        if ((r & 1) ^ par) x = make_float2(-x.x, -x.y);
        wcol[q] = make_float4(x.x, x.y, sqrtf(fmaf(x.x, x.x, x.y * x.y)), 0.f);
    }
}

// ---------------------------------------------------------------------------
// TMA-fed column pass: persistent CTAs, each looping over columns
// c = blockIdx.x, blockIdx.x + gridDim.x, ...; the R non-zero entries of the
// next column are fetched by a 1D bulk copy (cp.async.bulk, completion counted
// on an mbarrier) into one of two staging buffers while the current column is
// transformed.  Requires R*8 bytes to be a multiple of 16 (R even), which also
// keeps every column start 16-byte aligned.  Waits are bounded: a wait that
// gives up sets ERR_SPIN, waits (bounded) for the copies it issued and ends
// the CTA.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst_smem, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst_smem)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// true once the barrier's phase with this parity has completed; false when
// the bounded number of polls ran out
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    const unsigned a = smem_u32(bar);
    for (int it = 0; it < (1 << 22); ++it) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

template <int E, int MAXT, int LG>
__global__ void __launch_bounds__(MAXT) cols_batch_tma_kernel(Geo g, int total, const float2* __restrict__ zt,
                                                              const float2* __restrict__ stw,
                                                              float4* __restrict__ wel,
                                                              DevState* st) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* stg = reinterpret_cast<float2*>(smem_raw);  // [2][R], 16-byte aligned
    float2* buf = stg + 2 * (size_t)g.R;
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(buf + fft_slots(g.N));
    const unsigned bytes = (unsigned)g.R * 8u;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int c = blockIdx.x;
    if (threadIdx.x == 0 && c < total) bulk_load(stg, zt + (size_t)c * g.R, bytes, &bar[0]);
    int issued = (c < total) ? 1 : 0, consumed = 0;
    for (int i = 0; c < total; ++i, c += gridDim.x) {
        const int cur = i & 1;
        const int nxt = c + gridDim.x;
        if (threadIdx.x == 0 && nxt < total) {
            // the other buffer was read by all threads before the barriers of the previous column
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            bulk_load(stg + (size_t)(cur ^ 1) * g.R, zt + (size_t)nxt * g.R, bytes, &bar[cur ^ 1]);
            ++issued;
        }
        const bool ok = mbar_wait(&bar[cur], (unsigned)((i >> 1) & 1));
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0) {
                atomicOr(&st->err, ERR_SPIN);
                for (int j = consumed; j < issued; ++j) (void)mbar_wait(&bar[j & 1], (unsigned)((j >> 1) & 1));
            }
            __syncthreads();
            return;
        }
        ++consumed;
        const float2* col = stg + (size_t)cur * g.R;
        for (int r = threadIdx.x; r < g.N; r += blockDim.x) {
            const int q = r - g.band0;
            buf[sp(r)] = (q >= 0 && q < g.R) ? col[q] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        block_fft_sel<float, E, LG>(buf, g.N, stw);
        const int b = c / g.K, k = c - b * g.K;
        const int par = (k + g.N / 2) & 1;
        float4* wcol = wel + ((size_t)b * g.K + k) * g.W;
        for (int q = threadIdx.x; q < g.W; q += blockDim.x) {
            const int r = g.r0 + q;
            float2 x = buf[sp(r)];
            if ((r & 1) ^ par) x = make_float2(-x.x, -x.y);
            wcol[q] = make_float4(x.x, x.y, sqrtf(fmaf(x.x, x.x, x.y * x.y)), 0.f);
        }
        __syncthreads();  // buf and this staging buffer are free again
    }
}

// One (visibility, model) evaluation with the intermediates the adjoint needs.
struct PointEval {
    float2 V;              // model visibility
    float2 y[4];           // cell corners
    float am[4];           // corner moduli
    float t, q, su;        // fractions along v and u, sign of u'
    float A, zr, zi, rn;   // interpolated modulus, complex bilinear, 1/|z|
    float pc, ps;          // phase factor
    float ur, vr;          // rotated u, v (float)
    int cell;              // cell index in the model's window
    unsigned err;
};

// a*x + b*y for exact floats x, y and double-float a, b, as an unnormalised
// pair (s, e): s + e equals the product sum to ~2^-44 relative; |e| is a few
// ulps of s, which is all df_floor needs.
__device__ __forceinline__ DF df_dot2(float x, DF a, float y, DF b) {
    const float p1 = __fmul_rn(x, a.hi);
    const float e1 = __fmaf_rn(x, a.lo, __fmaf_rn(x, a.hi, -p1));
    const float p2 = __fmul_rn(y, b.hi);
    const float e2 = __fmaf_rn(y, b.lo, __fmaf_rn(y, b.hi, -p2));
    const DF s = df_two_sum(p1, p2);
    return DF{s.hi, __fadd_rn(s.lo, __fadd_rn(e1, e2))};
}

// Every visibility of a dataset lies inside the spectrum window: the host
// checks max|uv| against the image's uv range before the launch and the
// window is derived from the same maximum (with a rounding margin), and the
// dataset holds only finite (u, v).  The cell indices are still clamped to
// the window, so that no access can leave it; a clamp that changes an index
// raises ERR_WINDOW.
// rotation, cell index and fractions of one (visibility, model); returns the
// clamped cell (c0, q0) of the column-major window
__device__ __forceinline__ void locate_point(const Geo& g, const ModelConst& m, float u, float v, PointEval& p,
                                             int* c0, int* q0) {
    p.err = 0u;
    // rotated coordinates in grid units: a = u'/duv, c = v'/duv
    const DF a = df_dot2(u, m.cu, -v, m.sv);
    const DF cv = df_dot2(u, m.sv, v, m.cu);
    p.ur = a.hi;
    p.vr = cv.hi;
    // the sign of u' from the pair's rounded sum: df_dot2's pair is not
    // normalised (|lo| reaches a few ulps of the products, ~1e-5 cells), so
    // within that distance of u' = 0 the high part alone can have the wrong
    // sign and the floor below would give -1
    const float a_sum = __fadd_rn(a.hi, a.lo);
    const bool neg = a_sum < 0.f || (a_sum == 0.f && a.hi < 0.f);
    const float su = neg ? -1.f : 1.f;
    p.su = su;
    const DF indu = neg ? df_neg(a) : a;
    // N/2 + vo su c with |c| < N/2: Fast2Sum
    const bool flip = g.vo * su < 0.f;
    const float cs = flip ? -cv.hi : cv.hi, cl = flip ? -cv.lo : cv.lo;
    const float vh = __fadd_rn(g.half_nrow, cs);
    const DF indv{vh, __fadd_rn(__fsub_rn(cs, __fsub_rn(vh, g.half_nrow)), cl)};
    int fu, fv;
    df_floor(indu, &fu, &p.q);
    df_floor(indv, &fv, &p.t);
    const int qq = fv - g.r0;
    const int c0c = min(max(fu, 0), g.K - 2), qqc = min(max(qq, 0), g.W - 2);
    if (c0c != fu || qqc != qq) p.err = ERR_WINDOW;
    p.cell = c0c * g.W + qqc;
    *c0 = c0c;
    *q0 = qqc;
}

// V = U exp(2 pi i (u dRA + v dDec)) (the rotation-invariant form of the phase)
__device__ __forceinline__ void apply_phase_point(const ModelConst& m, float u, float v, float2 U, PointEval& p) {
    p.pc = 1.f;
    p.ps = 0.f;
    if (m.phase) {
        // u'dRA' + v'dDec' = u dRA + v dDec (both pairs rotated by PA)
        sincos2pi_df(df_dot2(u, m.dra, v, m.ddec), &p.ps, &p.pc);
        U = make_float2(U.x * p.pc - U.y * p.ps, U.x * p.ps + U.y * p.pc);
    }
    p.V = U;
}

__device__ __forceinline__ void eval_point(const Geo& g, const ModelConst& m, const float4* __restrict__ wel_b,
                                           float u, float v, PointEval& p) {
    int c0c, qqc;
    locate_point(g, m, u, v, p, &c0c, &qqc);
    const float su = p.su;
    // corners of cell (k, q): (k, q), (k, q+1), (k+1, q+1), (k+1, q) of the
    // column-major window (no wrap: K < N/2 + 1 by the host's uv-range check)
    const float4* e0 = wel_b + (size_t)c0c * g.W + qqc;
    const float4 c0v = __ldg(e0), c1v = __ldg(e0 + 1), c2v = __ldg(e0 + g.W + 1), c3v = __ldg(e0 + g.W);
    p.y[0] = make_float2(c0v.x, c0v.y);
    p.y[1] = make_float2(c1v.x, c1v.y);
    p.y[2] = make_float2(c2v.x, c2v.y);
    p.y[3] = make_float2(c3v.x, c3v.y);
    p.am[0] = c0v.z;
    p.am[1] = c1v.z;
    p.am[2] = c2v.z;
    p.am[3] = c3v.z;
    const float t = p.t, q = p.q;
    const float d1r = (p.y[0].x + p.y[2].x) - (p.y[1].x + p.y[3].x);
    const float d1i = (p.y[0].y + p.y[2].y) - (p.y[1].y + p.y[3].y);
    p.zr = t * (q * d1r) + (t * (p.y[1].x - p.y[0].x) + q * (p.y[3].x - p.y[0].x)) + p.y[0].x;
    p.zi = t * (q * d1i) + (t * (p.y[1].y - p.y[0].y) + q * (p.y[3].y - p.y[0].y)) + p.y[0].y;
    float A = p.am[0];
    A += (p.am[3] - p.am[0]) * q;
    A += (p.am[1] - p.am[0]) * t;
    A += (p.am[0] - p.am[1] + p.am[2] - p.am[3]) * t * q;
    p.A = A;
    float cph = 1.f, sph = 0.f;
    p.rn = 0.f;
    if (p.zr != 0.f || p.zi != 0.f) {
        p.rn = rsqrtf(fmaf(p.zr, p.zr, p.zi * p.zi));
        cph = p.zr * p.rn;
        sph = su * p.zi * p.rn;
    }
    apply_phase_point(m, u, v, make_float2(A * cph, A * sph), p);
}

// Accumulators per model and block: chi2, dPA, dRA, dDec
constexpr int kAcc = 4;

// One (visibility, model) of a real window (swept profiles, origin 'upper',
// every term evaluated, no branch: padding points have w = 0 and (u, v) = 0,
// so they add zero everywhere).  V = A sign(z) exp(2 pi i (u dRA + v dDec))
// with A the bilinear modulus and z the bilinear signed value of the cell's
// corners.  Returns the chi2 term.  With GRAD: hA = (dchi2/dA) / 2 for the
// cell's corner moments, and acc[1..3] += halves of dchi2/dPA and of
// dchi2/d(dRA, dDec) / (2 pi); kReal_scale restores the factors once per model.
struct RealPoint {
    float hA, t, q;
    int cell;
};
template <bool GRAD>
__device__ __forceinline__ float real_point(const Geo& g, const ModelConst& m, const float* __restrict__ wr_b,
                                            float u, float v, float re, float im, float w, float* acc,
                                            RealPoint& e, unsigned& err) {
    // rotated coordinates in grid units: a = u'/duv, c = v'/duv
    const DF a = df_dot2(u, m.cu, -v, m.sv);
    const DF cv = df_dot2(u, m.sv, v, m.cu);
    // u' < 0 reads the Hermitian point (-u', -v'); a real spectrum is unchanged
    // by it.  The sign comes from the pair's rounded sum (see locate_point).
    const float a_sum = __fadd_rn(a.hi, a.lo);
    const bool neg = a_sum < 0.f || (a_sum == 0.f && a.hi < 0.f);
    const DF indu = neg ? df_neg(a) : a;
    const float cs = neg ? -cv.hi : cv.hi, cl = neg ? -cv.lo : cv.lo;
    const float vh = __fadd_rn(g.half_nrow, cs);  // N/2 + c: Fast2Sum (|c| < N/2)
    const DF indv{vh, __fadd_rn(__fsub_rn(cs, __fsub_rn(vh, g.half_nrow)), cl)};
    int fu, fv;
    float q, t;
    df_floor(indu, &fu, &q);
    df_floor(indv, &fv, &t);
    const int qq = fv - g.r0;
    const int c0 = min(max(fu, 0), g.K - 2), q0 = min(max(qq, 0), g.W - 2);
    if (c0 != fu || q0 != qq) err |= ERR_WINDOW;
    e.cell = c0 * g.W + q0;
    e.t = t;
    e.q = q;
    // corners (k, q), (k, q+1), (k+1, q+1), (k+1, q) of the column-major window
    const float* e0 = wr_b + e.cell;
    const float y0 = __ldg(e0), y1 = __ldg(e0 + 1), y2 = __ldg(e0 + g.W + 1), y3 = __ldg(e0 + g.W);
    const float a0 = fabsf(y0), a1 = fabsf(y1), a2 = fabsf(y2), a3 = fabsf(y3);
    const float D = (a0 - a1) + (a2 - a3);
    const float dAq = fmaf(t, D, a3 - a0);  // dA/dq
    const float A = fmaf(q, dAq, fmaf(t, a1 - a0, a0));
    const float z = fmaf(q, fmaf(t, (y0 - y1) + (y2 - y3), y3 - y0), fmaf(t, y1 - y0, y0));
    const float As = z < 0.f ? -A : A;
    float ps = 0.f, pc = 1.f;
    // the model is the same for the whole warp: no divergence
    if (m.phase) sincos2pi_df(df_dot2(u, m.dra, v, m.ddec), &ps, &pc);
    const float vx = As * pc, vy = As * ps;
    const float dr = vx - re, di = vy - im;
    const float hx = w * dr, hy = w * di;  // (dchi2/dV) / 2
    if constexpr (GRAD) {
        const float gAs = fmaf(hx, pc, hy * ps);
        e.hA = z < 0.f ? -gAs : gAs;
        // phase 2 pi (u dRA + v dDec): (dchi2/dphi) / 2 = Im(conj(V) h)
        const float dphi = fmaf(hy, vx, -hx * vy);
        acc[2] = fmaf(dphi, u, acc[2]);
        acc[3] = fmaf(dphi, v, acc[3]);
        // position: q = |a|, t = N/2 + sign(a) c; da/dPA = -c, dc/dPA = a
        const float dAt = fmaf(q, D, a1 - a0);  // dA/dt
        acc[1] = fmaf(e.hA, fmaf(dAt, indu.hi, -dAq * cs), acc[1]);
    }
    return fmaf(dr, hx, di * hy);
}

// lane l of a warp ends with the warp's sum of a[(l >> 3) & 3]: one exchange
// of two values, one of one value, then three single-value halvings
__device__ __forceinline__ float warp_sum4(const float* a, int lane) {
    const unsigned full = 0xffffffffu;
    const bool h16 = lane & 16, h8 = lane & 8;
    float k0 = h16 ? a[2] : a[0], k1 = h16 ? a[3] : a[1];
    const float s0 = h16 ? a[0] : a[2], s1 = h16 ? a[1] : a[3];
    k0 += __shfl_xor_sync(full, s0, 16);
    k1 += __shfl_xor_sync(full, s1, 16);
    float k = h8 ? k1 : k0;
    k += __shfl_xor_sync(full, h8 ? k0 : k1, 8);
    k += __shfl_xor_sync(full, k, 4);
    k += __shfl_xor_sync(full, k, 2);
    k += __shfl_xor_sync(full, k, 1);
    return k;
}

// PTS consecutive entries of a float array, one vector load when aligned and in range
template <int PTS>
__device__ __forceinline__ void load_pts(const float* __restrict__ a, long long i0, long long n, float* out) {
    if (i0 + PTS <= n) {
        if constexpr (PTS == 4) {
            const float4 x = __ldg(reinterpret_cast<const float4*>(a + i0));
            out[0] = x.x; out[1] = x.y; out[2] = x.z; out[3] = x.w;
            return;
        } else if constexpr (PTS == 2) {
            const float2 x = __ldg(reinterpret_cast<const float2*>(a + i0));
            out[0] = x.x; out[1] = x.y;
            return;
        }
    }
#pragma unroll
    for (int j = 0; j < PTS; ++j) out[j] = (i0 + j < n) ? __ldg(&a[i0 + j]) : 0.f;
}

// A run of visibilities in one cell is summed as the moments of its corner
// gradients g = (dchi2/dRe z, dchi2/dIm z, dchi2/dA): M = (sum g, sum g t,
// sum g q, sum g t q), 12 floats [moment][component].  The cell's corner
// weights are (1-t)(1-q), t(1-q), tq, (1-t)q, so the corner sums follow from
// the moments; they are added to the model's 12-float cell record
// (re/im of corners 0..3, then the moduli of corners 0..3) with three 16-byte
// atomics.
__device__ __forceinline__ void emit_cell(float* __restrict__ cg, int cell, const float* M) {
    float r[12];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float m1 = M[i], mt = M[3 + i], mq = M[6 + i], mtq = M[9 + i];
        const float c[4] = {(m1 - mt) - (mq - mtq), mt - mtq, mtq, mq - mtq};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (i < 2) r[2 * k + i] = c[k];
            else r[8 + k] = c[k];
        }
    }
    float4* dst = reinterpret_cast<float4*>(cg + (size_t)cell * kGRec);
    atomicAdd(dst, make_float4(r[0], r[1], r[2], r[3]));
    atomicAdd(dst + 1, make_float4(r[4], r[5], r[6], r[7]));
    atomicAdd(dst + 2, make_float4(r[8], r[9], r[10], r[11]));
}
constexpr int kFirstStride = 13;  // shared-memory slot of a thread's first run (odd: no bank conflicts)

// real windows: the moments of dchi2/dA give the 4 corner sums of the cell,
// added to its 4-float record with one 16-byte atomic
__device__ __forceinline__ void emit_cell_real(float* __restrict__ cg, int cell, const float* M) {
    const float m1 = M[0], mt = M[1], mq = M[2], mtq = M[3];
    atomicAdd(reinterpret_cast<float4*>(cg + (size_t)cell * 4),
              make_float4((m1 - mt) - (mq - mtq), mt - mtq, mtq, mq - mtq));
}
template <bool REAL> __device__ __forceinline__ void emit_run(float* __restrict__ cg, int cell, const float* M) {
    if constexpr (REAL) emit_cell_real(cg, cell, M);
    else emit_cell(cg, cell, M);
}

// Grid: x = blocks of NT * PTS visibilities, y = groups of Bg models.  The
// hardware issues the x blocks of one group before the next, so the windows
// (and gradient records) of about Bg models are live in L2 at a time.
//
// Thread t of a block owns the PTS consecutive visibilities t*PTS .. t*PTS+PTS-1
// of the block's span (vector loads; consecutive in the Morton order, so they
// often share a uv cell).  With the gradient, each thread first sums the cell
// records of its own runs of equal cells in registers; runs that begin and
// end inside the thread are added to the cell gradient directly; the thread's
// first run, when it continues the previous lane's last run, is handed to that
// lane; the last runs then go through one warp-segmented reduction (shuffles)
// and one lane per run of equal cells adds it.
// REAL: the window is real (swept profiles): one float per element, one
// gradient component (dchi2/dA) per corner, 4-float cell records, and the
// point evaluation of real_point (halved gradients, restored per model).
constexpr double kTwoPi = 6.283185307179586476925286766559;

template <bool GRAD, int PTS, bool REAL, int NT>
__global__ void __launch_bounds__(NT) vis_batch_kernel(Geo g, int B, int Bg, int nd, const float* __restrict__ u,
                                                       const float* __restrict__ v, const float* __restrict__ re,
                                                       const float* __restrict__ im, const float* __restrict__ w,
                                                       const ModelConst* __restrict__ mc,
                                                       const void* __restrict__ wel_any, float* __restrict__ cgrad,
                                                       double* __restrict__ partials, DevState* st) {
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b0 = blockIdx.y * Bg;
    const int nb = min(Bg, B - b0);
    ModelConst* smc = reinterpret_cast<ModelConst*>(smem_raw);
    // per-warp sums [Bg][kAcc][warps]: every slot is written once, no zeroing
    // and no barrier between models
    float* wacc = reinterpret_cast<float*>(smc + Bg);
    // each thread's first run of equal cells (moments), read by the previous lane
    float* fst_all = wacc + Bg * kAcc * NW;
    constexpr int NR = REAL ? 4 : 12;              // floats of a run's moments
    constexpr int FS = REAL ? 5 : kFirstStride;   // odd slot stride: no bank conflicts
    float* fst = fst_all + threadIdx.x * FS;
    const float4* wel = static_cast<const float4*>(wel_any);
    const float* welr = static_cast<const float*>(wel_any);
    constexpr int kRecF = REAL ? 4 : kGRec;       // floats per gradient cell record
    for (int i = threadIdx.x; i < nb; i += blockDim.x) smc[i] = mc[b0 + i];
    // this thread's points
    float pu[PTS], pv[PTS], pre[PTS], pim[PTS], pw[PTS];
    const long long i0 = ((long long)blockIdx.x * NT + threadIdx.x) * PTS;
    load_pts<PTS>(u, i0, nd, pu);
    load_pts<PTS>(v, i0, nd, pv);
    load_pts<PTS>(re, i0, nd, pre);
    load_pts<PTS>(im, i0, nd, pim);
    load_pts<PTS>(w, i0, nd, pw);  // w = 0 marks the padding points
    __syncthreads();
    const long long ncell = (long long)g.K * g.W;
    unsigned err = 0u;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int bl = 0; bl < nb; ++bl) {
        const int b = b0 + bl;
        const ModelConst m = smc[bl];
        float* cg = cgrad + (size_t)b * ncell * kRecF;
        float acc[kAcc] = {0.f, 0.f, 0.f, 0.f};
        float run[NR];  // moments of the open run of equal cells
        int cur = -1, fcell = -1;
#pragma unroll
        for (int cc = 0; cc < NR; ++cc) run[cc] = 0.f;
#pragma unroll
        for (int j = 0; j < PTS; ++j) {
            if constexpr (REAL) {
                RealPoint e;
                acc[0] += real_point<GRAD>(g, m, welr + (size_t)b * ncell, pu[j], pv[j], pre[j], pim[j], pw[j], acc,
                                           e, err);
                if constexpr (GRAD) {
                    const float mom[4] = {1.f, e.t, e.q, e.t * e.q};
                    const bool same = e.cell == cur;
                    if (!same) {
                        if (cur >= 0) {
                            if (fcell < 0) {
                                fcell = cur;
#pragma unroll
                                for (int cc = 0; cc < NR; ++cc) fst[cc] = run[cc];
                            } else {
                                emit_run<REAL>(cg, cur, run);  // begins and ends inside this thread
                            }
                        }
                        cur = e.cell;
                    }
#pragma unroll
                    for (int mm = 0; mm < 4; ++mm) run[mm] = fmaf(e.hA, mom[mm], same ? run[mm] : 0.f);
                }
                continue;
            } else {
            const bool live = pw[j] != 0.f;  // w = 0: padding (or a zero-weight visibility)
            PointEval p;
            p.cell = -1;
            p.V = make_float2(0.f, 0.f);
            if (live) {
                eval_point(g, m, wel + (size_t)b * ncell, pu[j], pv[j], p);
                err |= p.err;
            }
            const float dr = p.V.x - pre[j], di = p.V.y - pim[j];
            if (live) acc[0] += pw[j] * (dr * dr + di * di);
            if (GRAD && live) {
                // dchi2/dV
                const float gx = 2.f * pw[j] * dr, gy = 2.f * pw[j] * di;
                // phase shift V = U P: dchi2/dphi = -Im(conj(G) V); phi = 2 pi (u dRA + v dDec)
                const float dphi = -(gx * p.V.y - gy * p.V.x);
                acc[2] += dphi * 6.28318530717958647692f * pu[j];
                acc[3] += dphi * 6.28318530717958647692f * pv[j];
                const float t = p.t, q = p.q;
                float gv[NR];
                // G_U = G conj(P)
                const float gux = gx * p.pc + gy * p.ps, guy = -gx * p.ps + gy * p.pc;
                // U = A * (zr, su zi) / |z|
                const float ex = p.zr * p.rn, ey = p.zi * p.rn;  // e = z/|z|
                const float gA = gux * ex + guy * (p.su * ey);
                // gradient w.r.t. e (undo the conjugation for u < 0)
                const float gex = p.A * gux, gey = p.su * p.A * guy;
                const float dot = ex * gex + ey * gey;
                const float gzx = (gex - ex * dot) * p.rn, gzy = (gey - ey * dot) * p.rn;
                // position: q = |a|, t = N/2 + vo su c with a = u'/duv, c = v'/duv;
                // da/dPA = -c, dc/dPA = a
                const float dzqx = (p.y[3].x - p.y[0].x) + t * ((p.y[0].x - p.y[1].x) + (p.y[2].x - p.y[3].x));
                const float dzqy = (p.y[3].y - p.y[0].y) + t * ((p.y[0].y - p.y[1].y) + (p.y[2].y - p.y[3].y));
                const float dztx = (p.y[1].x - p.y[0].x) + q * ((p.y[0].x - p.y[1].x) + (p.y[2].x - p.y[3].x));
                const float dzty = (p.y[1].y - p.y[0].y) + q * ((p.y[0].y - p.y[1].y) + (p.y[2].y - p.y[3].y));
                const float dAq = (p.am[3] - p.am[0]) + t * ((p.am[0] - p.am[1]) + (p.am[2] - p.am[3]));
                const float dAt = (p.am[1] - p.am[0]) + q * ((p.am[0] - p.am[1]) + (p.am[2] - p.am[3]));
                const float gq = gzx * dzqx + gzy * dzqy + gA * dAq;
                const float gt = gzx * dztx + gzy * dzty + gA * dAt;
                gv[0] = gzx;
                gv[1] = gzy;
                gv[2] = gA;
                acc[1] += gq * (p.su * (-p.vr)) + gt * (g.vo * p.su * p.ur);
                // runs of equal cells within the thread, summed as moments in registers
                const float mom[4] = {1.f, t, q, t * q};
                if (p.cell == cur) {
#pragma unroll
                    for (int mm = 0; mm < 4; ++mm)
#pragma unroll
                        for (int i = 0; i < 3; ++i) run[3 * mm + i] = fmaf(gv[i], mom[mm], run[3 * mm + i]);
                } else {
                    if (cur >= 0) {
                        if (fcell < 0) {
                            fcell = cur;
#pragma unroll
                            for (int cc = 0; cc < NR; ++cc) fst[cc] = run[cc];
                        } else {
                            emit_run<REAL>(cg, cur, run);  // begins and ends inside this thread
                        }
                    }
                    cur = p.cell;
#pragma unroll
                    for (int mm = 0; mm < 4; ++mm)
#pragma unroll
                        for (int i = 0; i < 3; ++i) run[3 * mm + i] = gv[i] * mom[mm];
                }
            }
            }
        }
        if (GRAD) {
            const unsigned full = 0xffffffffu;
            const int klast = cur >= 0 ? cur : -1 - lane;  // empty lanes get keys no cell matches
            const int kprev = __shfl_up_sync(full, klast, 1);
            // the first run continues the previous lane's last run: hand it over
            const bool pass = fcell >= 0 && lane > 0 && fcell == kprev;
            __syncwarp();
            const bool take = __shfl_down_sync(full, (int)pass, 1) && lane < 31;
            if (take) {
                const float* nf = fst + FS;  // the next lane's slot
#pragma unroll
                for (int cc = 0; cc < NR; ++cc) run[cc] += nf[cc];
            }
            if (fcell >= 0 && !pass) emit_run<REAL>(cg, fcell, fst);
            // last runs: lanes with equal keys are consecutive; reduce each
            // segment with shuffles, then its first lane adds it
            const unsigned heads = __ballot_sync(full, lane == 0 || klast != kprev);
            if (heads != full) {
                const int seg = __popc(heads & ((2u << lane) - 1u));
                // only as many halving steps as the longest segment needs
                const unsigned later = heads & ~((2u << lane) - 1u);
                const int len = ((heads >> lane) & 1u) ? (later ? __ffs(later) - 1 : 32) - lane : 0;
                const int maxlen = __reduce_max_sync(full, len);
                for (int d = 1; d < maxlen; d <<= 1) {
                    const int seg_d = __shfl_down_sync(full, seg, d);
#pragma unroll
                    for (int cc = 0; cc < NR; ++cc) {
                        const float o = __shfl_down_sync(full, run[cc], d);
                        if (lane + d < 32 && seg_d == seg) run[cc] += o;
                    }
                }
            }
            if (cur >= 0 && ((heads >> lane) & 1u)) emit_run<REAL>(cg, cur, run);
            __syncwarp();  // the slots are rewritten for the next model
            // warp sums of the four accumulators: lanes 0, 8, 16, 24 hold them
            const float x = warp_sum4(acc, lane);
            if ((lane & 7) == 0) wacc[(bl * kAcc + (lane >> 3)) * NW + wid] = x;
        } else {
            float x = acc[0];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) wacc[(bl * kAcc) * NW + wid] = x;
        }
    }
    if (err) atomicOr(&st->err, err);
    __syncthreads();
    // real_point accumulates halves of dchi2/dPA and of dchi2/d(dRA, dDec) / (2 pi)
    double* dst = partials + ((size_t)blockIdx.x * B + b0) * kAcc;
    for (int i = threadIdx.x; i < nb * kAcc; i += blockDim.x) {
        const int a = i % kAcc;
        double s = 0.0;
        if (GRAD || a == 0) {
            for (int q = 0; q < NW; ++q) s += (double)wacc[i * NW + q];
        }
        if (REAL && a > 0) s *= (a == 1 ? 2.0 : 2.0 * kTwoPi);
        dst[i] = s;
    }
}

// partials [blocks][B][kAcc] -> chi2 per set and in total, gradient sums
// (fixed summation order).  Set k owns the blocks [pad[k], pad[k+1]) / bpts.
__global__ void batch_finalize_kernel(int B, int nsets, const long long* __restrict__ pad, int bpts,
                                      const double* __restrict__ partials, double* __restrict__ chi2,
                                      double* __restrict__ chi2_sets, double* __restrict__ gsum) {
    __shared__ double sh[32];
    const int b = blockIdx.x, a = blockIdx.y;
    if (a == 0) {
        double tot = 0.0;
        for (int k = 0; k < nsets; ++k) {
            const long long q0 = pad[k] / bpts, q1 = pad[k + 1] / bpts;
            double s = 0.0;
            for (long long q = q0 + threadIdx.x; q < q1; q += blockDim.x) s += partials[((size_t)q * B + b) * kAcc];
            s = block_sum(s, sh);
            if (threadIdx.x == 0 && chi2_sets) chi2_sets[(size_t)b * nsets + k] = s;
            tot += s;
        }
        if (threadIdx.x == 0) chi2[b] = tot;
    } else {
        const long long nblocks = pad[nsets] / bpts;
        double s = 0.0;
        for (long long q = threadIdx.x; q < nblocks; q += blockDim.x) s += partials[((size_t)q * B + b) * kAcc + a];
        s = block_sum(s, sh);
        if (threadIdx.x == 0) gsum[b * kAcc + a] = s;
    }
}

// ---------------------------------------------------------------------------
// adjoint kernels
// ---------------------------------------------------------------------------
// gradient of every window element from the cell records; S/|S| for the
// modulus part; times the forward output sign
// Grid (K, B): the block of column k of model b walks the window rows q.
__global__ void quadT_batch_kernel(Geo g, const float* __restrict__ cgrad, const float4* __restrict__ wel,
                                   float2* __restrict__ gwin) {
    const long long ncell = (long long)g.K * g.W;
    const int k = blockIdx.x, b = blockIdx.y;
    const float* cg = cgrad + (size_t)b * ncell * kGRec;
    for (int q = threadIdx.x; q < g.W; q += blockDim.x) {
        float gx = 0.f, gy = 0.f, ga = 0.f;
        // the element (k, q) is corner c of cell (kc, qc)
        auto take = [&](int kc, int qc, int c) {
            if (kc < 0 || qc < 0 || kc >= g.K || qc >= g.W) return;
            const float* rec = cg + ((long long)kc * g.W + qc) * kGRec;
            gx += rec[2 * c];
            gy += rec[2 * c + 1];
            ga += rec[8 + c];
        };
        take(k, q, 0);
        take(k, q - 1, 1);
        take(k - 1, q - 1, 2);
        take(k - 1, q, 3);
        const size_t el = (size_t)b * ncell + (size_t)k * g.W + q;
        const float4 sv = wel[el];
        if (sv.z > 0.f) {
            const float r = 1.f / sv.z;
            gx += ga * sv.x * r;
            gy += ga * sv.y * r;
        }
        const int row = g.r0 + q;
        if (((row + k + g.N / 2) & 1)) {
            gx = -gx;
            gy = -gy;
        }
        gwin[el] = make_float2(gx, gy);
    }
}

// adjoint of the column pass: inverse column FFT of the window gradient, kept
// on the band rows.  IFFT(x) = conj(FFT(conj(x))): the forward transform runs
// on the conjugated column.
template <int E, int MAXT, int LG>
__global__ void __launch_bounds__(MAXT) colsT_batch_kernel(Geo g, const float2* __restrict__ gwin,
                                                           const float2* __restrict__ stw,
                                                           float2* __restrict__ zbar) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* buf = reinterpret_cast<float2*>(smem_raw);
    const int b = blockIdx.y, k = blockIdx.x;
    const float2* col = gwin + ((size_t)b * g.K + k) * g.W;
    for (int i = threadIdx.x; i < g.N; i += blockDim.x) {
        const int q = i - g.r0;
        const float2 x = (q >= 0 && q < g.W) ? col[q] : make_float2(0.f, 0.f);
        buf[sp(i)] = make_float2(x.x, -x.y);
    }
    __syncthreads();
    block_fft_sel<float, E, LG>(buf, g.N, stw);
    float2* out = zbar + ((size_t)b * g.K + k) * g.R;
    for (int q = threadIdx.x; q < g.R; q += blockDim.x) {
        const float2 x = buf[sp(g.band0 + q)];
        out[q] = make_float2(x.x, -x.y);
    }
}

// adjoint of the row pass + sweep: for each image row, x_bar[j] =
// (-1)^I Re(sum_{k<K} zbar[k] e^{+2 pi i j k/N}) via the half-length inverse
// complex FFT (Hermitian weights), then the sweep adjoint into the profile
// and the inclination.
template <int E, int MAXT, int LG>
__global__ void __launch_bounds__(MAXT, (MAXT <= 256 ? 3 : 1)) rowsT_batch_kernel(Geo g, int F, int G, const float* __restrict__ intensity,
                                                           const ModelConst* __restrict__ mc,
                                                           const float2* __restrict__ stw,
                                                           const float2* __restrict__ twc,
                                                           const float2* __restrict__ zbar,
                                                           float* __restrict__ gI, double* __restrict__ ginc,
                                                           float* __restrict__ gcentral) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* buf = reinterpret_cast<float2*>(smem_raw);               // M complex
    const int S = 2 * F + 1;                                         // staging row stride (odd: no bank conflicts)
    float2* stg = buf + fft_slots(g.M);                              // [K][S] staged input rows
    float* gIs = reinterpret_cast<float*>(stg + (size_t)g.K * S);    // nr floats
    float* fold = gIs + g.nr;                                        // rmax + 1 floats
    __shared__ double sinc;
    __shared__ int lo_bin, hi_bin;
    const int b = blockIdx.y;
    const ModelConst m = mc[b];
    const float* Ib = intensity + (size_t)b * g.nr;
    const float2* zb = zbar + (size_t)b * g.K * g.R;
    for (int i = threadIdx.x; i < g.nr; i += blockDim.x) gIs[i] = 0.f;
    if (threadIdx.x == 0) {
        lo_bin = g.nr;
        hi_bin = -1;
        sinc = 0.0;
    }
    float ginc_acc = 0.f;
    int my_lo = g.nr, my_hi = -1;  // bins this thread touched
    const int off = g.N / 2 - g.rmax;
    const int M = g.M;
    // G groups of F folded rows per CTA: the profile flush below is paid once
    // per G * F folded rows, the staging holds one group
    for (int grp = 0; grp < G; ++grp) {
    const int a0 = (blockIdx.x * G + grp) * F;
    if (a0 > g.rmax) break;  // uniform
    int lo0, lo1, n1;
    const int n0 = fold_rows(g, a0, F, &lo0, &lo1, &n1);
    __syncthreads();  // the previous group's rows are consumed
    {
        // the group's 2F rows of every column k: two contiguous runs each
        const int nrun = n0 + n1;
        const float inv_nrun = 1.f / i2f_small(nrun);
        for (int e = threadIdx.x; e < g.K * nrun; e += blockDim.x) {
            int k, j;
            split_index(e, nrun, inv_nrun, &k, &j);
            const int row = j < n0 ? lo0 + j : lo1 + (j - n0);
            const int slot = j < n0 ? j : F + (j - n0);
            stg[k * S + slot] = zb[(size_t)k * g.R + row];
        }
    }
    for (int ff = 0; ff < n0; ++ff) {
        const int a = a0 + ff;  // folded row
        // sum of the pixel adjoints over the (up to) four mirror images
        // (+-x, +-y) of every folded pixel of this folded row.  The mirror
        // rows rmax - a and rmax + a have the same row sign, so their spectra
        // are added first and one inverse transform serves both.
        const int I = off + g.rmax - a;
        const int slot0 = (g.rmax - a) - lo0;
        const bool mirror = a > 0 && a < g.rmax;
        const int slot1 = mirror ? F + (g.rmax + a - lo1) : slot0;
        const float wm = mirror ? 1.f : 0.f;
        __syncthreads();
        // Hermitian weights: Y~0 = Re Y0, Y~k = Yk/2 (0<k<M), Y~M = Re YM; zero for k >= K
        for (int k = threadIdx.x; k < M; k += blockDim.x) {
            if (k >= g.K && M - k >= g.K) {  // both partners outside the K computed columns
                buf[sp(k)] = make_float2(0.f, 0.f);
                continue;
            }
            auto yk = [&](int kk) -> float2 {
                if (kk >= g.K) return make_float2(0.f, 0.f);
                const float2 y0 = stg[kk * S + slot0], y1 = stg[kk * S + slot1];
                const float2 y = make_float2(fmaf(wm, y1.x, y0.x), fmaf(wm, y1.y, y0.y));
                if (kk == 0 || kk == M) return make_float2(y.x, 0.f);
                return make_float2(0.5f * y.x, 0.5f * y.y);
            };
            const float2 ya = yk(k), yc = yk(M - k);
            // E' = a + conj(c), O' = (a - conj(c)) e^{+2 pi i k/N}, Z = E' + i O'
            const float2 Ep = make_float2(ya.x + yc.x, ya.y - yc.y);
            const float2 d = make_float2(ya.x - yc.x, ya.y + yc.y);
            const float2 w = twc[k];  // e^{+2 pi i k / N}
            const float2 Op = make_float2(d.x * w.x - d.y * w.y, d.x * w.y + d.y * w.x);
            // Z = E' + i O', stored conjugated: the inverse FFT is conj(FFT(conj(Z)))
            buf[sp(k)] = make_float2(Ep.x - Op.y, -(Ep.y + Op.x));
        }
        __syncthreads();
        block_fft_sel<float, E, LG>(buf, M, stw);
        const float sgn = (I & 1) ? -1.f : 1.f;
        // x_bar of box pixel j: conj(z) in buf, x[2m] = Re z, x[2m+1] = Im z = -buf.y
        auto xbar = [&](int j) {
            const int J = j + off;
            const float2 zz = buf[sp(J >> 1)];
            return sgn * ((J & 1) ? -zz.y : zz.x);
        };
        for (int c = threadIdx.x; c <= g.rmax; c += blockDim.x) {  // each c stays with one thread
            float acc = xbar(g.rmax - c);
            if (c > 0 && c < g.rmax) acc += xbar(g.rmax + c);
            fold[c] = acc;
        }
        __syncthreads();
        // sweep adjoint of the folded row; (a, c) = (0, 0) is the central pixel alone
        const float y = i2f_small(a) * g.dxy;
        for (int c = threadIdx.x; c <= g.rmax; c += blockDim.x) {
            const float xb = fold[c];
            if (a == 0 && c == 0) {
                gcentral[b] = xb;
                continue;
            }
            const float x = i2f_small(c) * g.dxy;
            const float xs = x * m.inv_cos_inc;
            const float r = sqrtf(xs * xs + y * y);  // bit-identical to the forward sweep's radius
            const float tR = (r - g.Rmin) * g.inv_dR;
            if (!(tR < (float)(g.nr - 1))) continue;
            int iR = 0;
            if (tR > 0.f) {
                float fl;
                iR = floor_i(tR, &fl);
            }
            const float frac = (r - i2f_small(iR) * g.dR - g.Rmin) * g.inv_dR;
            const float gxs = xb * g.sr_to_px;
            const float I0 = __ldg(&Ib[iR]), I1 = __ldg(&Ib[iR + 1]);  // issued before the atomics
            atomicAdd(&gIs[iR], gxs * (1.f - frac));
            atomicAdd(&gIs[iR + 1], gxs * frac);
            my_lo = min(my_lo, iR);
            my_hi = max(my_hi, iR + 1);
            // dr/dinc = xs^2 tan(inc) / r (r = 0 only at the central pixel, handled above)
            const float rinv = r > 0.f ? __fdividef(1.f, r) : 0.f;
            ginc_acc += gxs * ((I1 - I0) * g.inv_dR) * (xs * xs * m.tan_inc) * rinv;
        }
    }
    }  // groups
    // once per thread (the block may be narrower than a warp for small images)
    atomicMin(&lo_bin, my_lo);
    atomicMax(&hi_bin, my_hi);
    atomicAdd(&sinc, (double)ginc_acc);
    __syncthreads();
    float* gIb = gI + (size_t)b * g.nr;
    for (int i = lo_bin + threadIdx.x; i <= hi_bin; i += blockDim.x)
        if (gIs[i] != 0.f) atomicAdd(&gIb[i], gIs[i]);
    if (threadIdx.x == 0) atomicAdd(&ginc[b], sinc);
}

// ---------------------------------------------------------------------------
// Spectrum passes of swept profiles as products with fixed cosine matrices,
// on the tensor cores (gb_tc.cuh).  The swept image is even in x and y about
// the centre pixel, so with F[a][c] its folded quadrant (a = |y|, c = |x| in
// pixels, 0 <= a, c <= rmax; F[0][0] the central pixel) the shifted spectrum
// is real and
//     S[r][k] = sum_a Cv[r][a] sum_c Ck[k][c] F[a][c],
//     Ck[k][c] = w_c cos(2 pi c k / N),  Cv[q][a] = w_a cos(2 pi a |r0 + q - N/2| / N)
// (w_j = 1 for j = 0 and j = N/2, 2 otherwise: the number of mirror pixels),
// the reference's fftshift_axis0(rfft2(fftshift(image))) without any sign
// folding.  For B models the cosine matrices are shared, so the row and the
// column pass are two batched products per direction:
//     forward   D1_b = Ck F_b^T        (K x (rmax+1))
//               S_b  = D1_b Cv^T       (K x W, the window, column-major by k)
//     adjoint   G1_b = Cv^T G_b^T      ((rmax+1) x K, G_b the window gradient)
//               GF_b = G1_b Ck         ((rmax+1) x (rmax+1) = dchi2/dF)
// each FP32 operand as a TF32 hi/lo pair (3xTF32).
// ---------------------------------------------------------------------------
// the folded quadrant of every model as a TF32 pair; grid (ceil((rmax+1)^2 / 256), B)
__global__ void sweep_fold_kernel(Geo g, const float* __restrict__ intensity, const ModelConst* __restrict__ mc,
                                  float* __restrict__ fhi, float* __restrict__ flo, int ldF) {
    const int b = blockIdx.y;
    const int n = g.rmax + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * n) return;
    const int a = e / n, c = e - a * n;
    const ModelConst& m = mc[b];
    const int off = g.N / 2 - g.rmax;
    float x;
    if (a == 0 && c == 0) {
        x = m.central;
    } else {
        x = sweep_pixel<float>(off + g.rmax - a, off + g.rmax - c, intensity + (size_t)b * g.nr, g.nr, g.Rmin, g.dR,
                               g.inv_dR, g.dxy, m.inv_cos_inc, g.rmax, off, g.sr_to_px);
    }
    const float hi = tc::tf32_rna(x);
    const size_t o = ((size_t)b * n + a) * ldF + c;
    fhi[o] = hi;
    flo[o] = tc::tf32_rna(x - hi);
}

// Cell gradients of a real window -> the window gradient, folded over the
// mirror rows: G'[k][t] = G[k][h0 - t] + G[k][h0 + t] (h0 = N/2 - r0, the
// terms inside the window), t < T1, as a TF32 pair (the tensor-core path's
// spectrum carries no sign folding); grid (K, B).  The spectrum is even
// about row N/2, so its adjoint needs only the folded gradient.
__global__ void quadT_real_tc_kernel(Geo g, const float* __restrict__ cgrad4, const float* __restrict__ wr,
                                     float* __restrict__ ghi, float* __restrict__ glo, int T1, int ldT) {
    const long long ncell = (long long)g.K * g.W;
    const int k = blockIdx.x, b = blockIdx.y;
    const int h0 = g.N / 2 - g.r0;
    const float* cg = cgrad4 + (size_t)b * ncell * 4;
    auto grad_at = [&](int q) {  // dchi2 / dS[k][q]
        float ga = 0.f;
        auto take = [&](int kc, int qc, int c) {
            if (kc < 0 || qc < 0 || kc >= g.K || qc >= g.W) return;
            ga += cg[((long long)kc * g.W + qc) * 4 + c];
        };
        take(k, q, 0);
        take(k, q - 1, 1);
        take(k - 1, q - 1, 2);
        take(k - 1, q, 3);
        const float y = wr[(size_t)b * ncell + (size_t)k * g.W + q];
        ga *= 2.f;  // the vis pass records halves of dchi2/dA
        return y < 0.f ? -ga : (y > 0.f ? ga : 0.f);
    };
    for (int t = threadIdx.x; t < T1; t += blockDim.x) {
        const int q1 = h0 - t, q2 = h0 + t;
        float gy = (q1 >= 0 && q1 < g.W) ? grad_at(q1) : 0.f;
        if (t > 0 && q2 >= 0 && q2 < g.W) gy += grad_at(q2);
        const float hi = tc::tf32_rna(gy);
        const size_t o = ((size_t)b * g.K + k) * ldT + t;
        ghi[o] = hi;
        glo[o] = tc::tf32_rna(gy - hi);
    }
}

// Adjoint of the sweep from dchi2/dF: the profile samples (linear
// interpolation weights, binned in shared memory), the inclination
// (dr/dinc = xs^2 tan(inc) / r) and the central pixel.  A CTA takes
// kRowsPerCta folded rows of one model and writes its nr bins and its
// inclination sum as one partial (no global atomics);
// sweep_adjoint_reduce_kernel adds the partials in a fixed order.
// Grid (nchunk = ceil((rmax+1)/kRowsPerCta), B).
__global__ void sweep_adjoint_kernel(Geo g, const float* __restrict__ intensity, const ModelConst* __restrict__ mc,
                                     const float* __restrict__ gF, int ldF, float* __restrict__ part,
                                     double* __restrict__ part_inc, float* __restrict__ gcentral) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* gIs = reinterpret_cast<float*>(smem_raw);  // nr bins
    __shared__ double sh[32];
    const int b = blockIdx.y;
    const ModelConst m = mc[b];
    const float* Ib = intensity + (size_t)b * g.nr;
    const int n = g.rmax + 1;
    for (int i = threadIdx.x; i < g.nr; i += blockDim.x) gIs[i] = 0.f;
    __syncthreads();
    float ginc_acc = 0.f;
    const int a0 = blockIdx.x * kRowsPerCta;
    const int a1 = min(n, a0 + kRowsPerCta);
    for (int e = threadIdx.x; e < (a1 - a0) * n; e += blockDim.x) {
        const int a = a0 + e / n, c = e % n;
        const float xb = gF[((size_t)b * n + a) * ldF + c];
        if (a == 0 && c == 0) {
            gcentral[b] = xb;
            continue;
        }
        const float y = i2f_small(a) * g.dxy;
        const float x = i2f_small(c) * g.dxy;
        const float xs = x * m.inv_cos_inc;
        const float r = sqrtf(xs * xs + y * y);  // bit-identical to the forward sweep's radius
        const float tR = (r - g.Rmin) * g.inv_dR;
        if (!(tR < (float)(g.nr - 1))) continue;
        int iR = 0;
        if (tR > 0.f) {
            float fl;
            iR = floor_i(tR, &fl);
        }
        const float frac = (r - i2f_small(iR) * g.dR - g.Rmin) * g.inv_dR;
        const float gxs = xb * g.sr_to_px;
        const float I0 = __ldg(&Ib[iR]), I1 = __ldg(&Ib[iR + 1]);
        atomicAdd(&gIs[iR], gxs * (1.f - frac));
        atomicAdd(&gIs[iR + 1], gxs * frac);
        const float rinv = r > 0.f ? __fdividef(1.f, r) : 0.f;
        ginc_acc += gxs * ((I1 - I0) * g.inv_dR) * (xs * xs * m.tan_inc) * rinv;
    }
    const double tot = block_sum_df(ginc_acc, sh);  // FP32 instructions only
    __syncthreads();
    float* pb = part + ((size_t)b * gridDim.x + blockIdx.x) * g.nr;
    for (int i = threadIdx.x; i < g.nr; i += blockDim.x) pb[i] = gIs[i];
    if (threadIdx.x == 0) part_inc[(size_t)b * gridDim.x + blockIdx.x] = tot;
}

// gI[b][i] = sum of the nchunk partial bins of model b (fixed order),
// ginc[b] = sum of the partial inclination sums.  Grid (ceil(nr/256), B).
__global__ void sweep_adjoint_reduce_kernel(int nr, int nchunk, const float* __restrict__ part,
                                            const double* __restrict__ part_inc, float* __restrict__ gI,
                                            double* __restrict__ ginc) {
    const int b = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nr) {
        const float* pb = part + (size_t)b * nchunk * nr + i;
        float s = 0.f;
        for (int q = 0; q < nchunk; ++q) s += pb[(size_t)q * nr];
        gI[(size_t)b * nr + i] = s;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < nchunk; ++q) t += part_inc[(size_t)b * nchunk + q];
        ginc[b] = t;
    }
}

// adjoint of the central pixel: I_bar += coef * x_bar(center)
__global__ void central_adjoint_kernel(int B, int nr, const double* __restrict__ coef, int ncoef,
                                       const float* __restrict__ gcentral, float* __restrict__ gI) {
    const int b = blockIdx.x;
    for (int i = threadIdx.x; i < ncoef; i += blockDim.x) gI[(size_t)b * nr + i] += (float)(coef[i] * gcentral[b]);
}

__global__ void write_grad_params_kernel(int B, int pstride, const double* __restrict__ gsum,
                                         const double* __restrict__ ginc, float* __restrict__ gp) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    float* o = gp + (size_t)pstride * b;
    if (pstride == 4) *o++ = (float)ginc[b];
    o[0] = (float)gsum[b * kAcc + 1];
    o[1] = (float)gsum[b * kAcc + 2];
    o[2] = (float)gsum[b * kAcc + 3];
}

// ---------------------------------------------------------------------------
// image models: B images of N x N pixels [Jy/pixel], all N rows transformed
// (band0 = 0, R = N).  A CTA takes F consecutive rows and stages their K
// spectrum columns in shared memory (row stride S = F + 1) so that the
// transposed layout zt[b][k][row] is written, and read back by the adjoint,
// in contiguous runs of F rows.
// ---------------------------------------------------------------------------
template <int E, int MAXT, int LG>
__global__ void __launch_bounds__(MAXT) rows_image_batch_kernel(Geo g, int F, const float* __restrict__ images,
                                                                const float2* __restrict__ tw,
                                                                const float2* __restrict__ stw,
                                                                float2* __restrict__ zt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* buf = reinterpret_cast<float2*>(smem_raw);
    const int S = F + 1;
    float2* stg = buf + fft_slots(g.M);  // [K][S]
    const int b = blockIdx.y;
    const int i0 = blockIdx.x * F;
    const int nrow = min(F, g.N - i0);
    const float* img = images + (size_t)b * g.N * g.N;
    for (int rr = 0; rr < nrow; ++rr) {
        const int i = i0 + rr;
        const float2* row = reinterpret_cast<const float2*>(img + (size_t)i * g.N);
        __syncthreads();  // buf free
        for (int mm = threadIdx.x; mm < g.M; mm += blockDim.x) buf[sp(mm)] = __ldg(&row[mm]);
        __syncthreads();
        block_fft_sel<float, E, LG>(buf, g.M, stw);
        const float sgn = (i & 1) ? -1.f : 1.f;  // the image fftshift, folded into the rows
        for (int k = threadIdx.x; k < g.K; k += blockDim.x) {
            const float2 x = real_split<float>(buf, g.M, k, tw);
            stg[k * S + rr] = make_float2(sgn * x.x, sgn * x.y);
        }
    }
    __syncthreads();
    float2* out = zt + (size_t)b * g.K * g.R;
    const float inv_n = 1.f / i2f_small(nrow);
    for (int e = threadIdx.x; e < g.K * nrow; e += blockDim.x) {
        int k, j;
        split_index(e, nrow, inv_n, &k, &j);
        out[(size_t)k * g.R + i0 + j] = stg[k * S + j];
    }
}

// adjoint of rows_image_batch_kernel: dchi2/d(pixel) of every image row
template <int E, int MAXT, int LG>
__global__ void __launch_bounds__(MAXT) rowsT_image_batch_kernel(Geo g, int F, const float2* __restrict__ stw,
                                                                 const float2* __restrict__ twc,
                                                                 const float2* __restrict__ zbar,
                                                                 float* __restrict__ gimg) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* buf = reinterpret_cast<float2*>(smem_raw);
    const int S = F + 1;
    float2* stg = buf + fft_slots(g.M);  // [K][S]
    const int b = blockIdx.y;
    const int i0 = blockIdx.x * F;
    const int nrow = min(F, g.N - i0);
    const int M = g.M;
    const float2* zb = zbar + (size_t)b * g.K * g.R;
    {
        const float inv_n = 1.f / i2f_small(nrow);
        for (int e = threadIdx.x; e < g.K * nrow; e += blockDim.x) {
            int k, j;
            split_index(e, nrow, inv_n, &k, &j);
            stg[k * S + j] = zb[(size_t)k * g.R + i0 + j];
        }
    }
    for (int rr = 0; rr < nrow; ++rr) {
        const int i = i0 + rr;
        __syncthreads();
        // Hermitian weights: Y~0 = Re Y0, Y~k = Yk/2 (0<k<M), Y~M = Re YM; zero for k >= K
        for (int k = threadIdx.x; k < M; k += blockDim.x) {
            if (k >= g.K && M - k >= g.K) {  // both partners outside the K computed columns
                buf[sp(k)] = make_float2(0.f, 0.f);
                continue;
            }
            auto yk = [&](int kk) -> float2 {
                if (kk >= g.K) return make_float2(0.f, 0.f);
                const float2 y = stg[kk * S + rr];
                if (kk == 0 || kk == M) return make_float2(y.x, 0.f);
                return make_float2(0.5f * y.x, 0.5f * y.y);
            };
            const float2 ya = yk(k), yc = yk(M - k);
            const float2 Ep = make_float2(ya.x + yc.x, ya.y - yc.y);
            const float2 d = make_float2(ya.x - yc.x, ya.y + yc.y);
            const float2 w = twc[k];  // e^{+2 pi i k / N}
            const float2 Op = make_float2(d.x * w.x - d.y * w.y, d.x * w.y + d.y * w.x);
            buf[sp(k)] = make_float2(Ep.x - Op.y, -(Ep.y + Op.x));  // conjugated: inverse FFT by a forward one
        }
        __syncthreads();
        block_fft_sel<float, E, LG>(buf, M, stw);
        const float sgn = (i & 1) ? -1.f : 1.f;
        float2* grow = reinterpret_cast<float2*>(gimg + ((size_t)b * g.N + i) * g.N);
        for (int mm = threadIdx.x; mm < M; mm += blockDim.x) {
            const float2 zz = buf[sp(mm)];  // conj(z): x[2m] = Re z, x[2m+1] = Im z
            grow[mm] = make_float2(sgn * zz.x, -sgn * zz.y);
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// launch-shape autotuner: per geometry, each pass's candidate shapes (complex
// values per thread of the FFT passes, visibilities per thread of the vis pass)
// are timed once with CUDA events on the caller's stream and the fastest is
// kept, in memory and in the cache file of gb_tune.h (keyed by GPU name,
// geometry, batch size and visibility-count bucket), so a later process on
// the same kind of GPU skips the timing.  GALARIO_AUTOTUNE=0 keeps the
// default shapes.
// ---------------------------------------------------------------------------
using Shape = tune::Shape;
struct TuneKey {
    int N, K, W, R, B, nd, grad, nr, image, tc;
    bool operator<(const TuneKey& o) const {
        return std::memcmp(this, &o, sizeof(TuneKey)) < 0;
    }
};
std::vector<int> fft_candidates(int L) {
    std::vector<int> c;
    for (int e : {8, 16})
        if (L / e >= 1 && L / e <= 1024 && L % e == 0) c.push_back(e);
    return c;
}
Shape default_shape(const Geo& g) {
    Shape sh;
    sh.e_rows = g.M >= 16384 ? 16 : 8;
    sh.e_cols = g.N >= 16384 ? 16 : 8;
    sh.e_colsT = sh.e_cols;
    sh.e_rowsT = sh.e_rows;
    sh.pts = 4;
    return sh;
}
// a cached shape is used only if every field is one of the current candidates
// (the tensor-core passes use only the visibility pass's field)
bool shape_valid(const Geo& g, const Shape& sh, bool real, bool tma_ok, bool tc) {
    auto in = [](int x, const std::vector<int>& c) {
        for (int y : c)
            if (y == x) return true;
        return false;
    };
    const std::vector<int> pts = real ? std::vector<int>{2, 4, 8} : std::vector<int>{2, 4};
    if (tc) return in(sh.pts, pts);
    const std::vector<int> rows = fft_candidates(g.M), cols = fft_candidates(g.N);
    const bool col_ok = in(sh.e_cols, cols) || (tma_ok && sh.e_cols >= kTmaCols && in(sh.e_cols - kTmaCols, cols));
    return in(sh.e_rows, rows) && col_ok && in(sh.e_colsT, cols) && in(sh.e_rowsT, rows) && in(sh.pts, pts);
}
bool graphs_enabled() {
    const char* v = std::getenv("GALARIO_GRAPHS");
    return !(v && v[0] == '0');
}
bool autotune_enabled() {
    const char* v = std::getenv("GALARIO_AUTOTUNE");
    return !(v && v[0] == '0');
}
struct Tuner {
    cudaStream_t s;
    cudaEvent_t a = nullptr, b = nullptr;
    explicit Tuner(cudaStream_t st) : s(st) {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    ~Tuner() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    // every candidate: one warm-up launch, then the fastest of three timed
    // launches (tune::best_of), timed with CUDA events on the caller's stream
    template <class F> int best(const std::vector<int>& cand, F&& run) {
        return tune::best_of(cand, run, [&](int c) -> double {
            cudaEventRecord(a, s);
            run(c);
            cudaEventRecord(b, s);
            if (cudaEventSynchronize(b) != cudaSuccess) return -1.0;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            return ms;
        });
    }
};

// the tuning cache file, shared by every device of the process
tune::Cache& tune_file() {
    static tune::Cache c(tune::default_path());
    return c;
}
tune::Key tune_file_key(int N, int K, int W, int R, int B, long long nd_pad, int grad, int nr, int image) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    const char* name = cudaGetDeviceProperties(&prop, dev) == cudaSuccess ? prop.name : "unknown";
    return tune::Key{tune::gpu_token(name), N, K, W, R, B, tune::nvis_bucket(nd_pad), grad, nr, image};
}

struct Err {
    int status;
    std::string msg;
};

// bumped whenever a workspace buffer moves: captured graphs older than it are stale
std::atomic<unsigned long long> g_buf_gen{1};
// set while a batched call is being captured into a CUDA graph
thread_local bool t_capturing = false;

struct Buf {
    void* p = nullptr;
    size_t cap = 0;
    template <typename T> T* get(size_t n) {
        size_t bytes = sizeof(T) * (n ? n : 1);
        if (bytes > cap) {
            if (t_capturing) throw Err{GALARIO_ERUNTIME, "Error in batch: workspace grew during graph capture"};
            g_buf_gen.fetch_add(1);
            if (p) cudaFree(p);
            p = nullptr;
            cap = 0;
            cudaError_t e = cudaMalloc(&p, bytes);
            if (e != cudaSuccess) throw e;
            cap = bytes;
        }
        return static_cast<T*>(p);
    }
};

// One captured batched call: the launch sequence of a (geometry, dataset,
// batch size, outputs) combination, reading its inputs from and writing its
// outputs to the workspace's staging buffers.
struct GraphKey {
    TuneKey tk;
    unsigned long long dataset;  // Dataset::serial
    float Rmin, dR, dxy, vo;
    int per_set;
    bool operator<(const GraphKey& o) const {
        return std::tie(tk, dataset, Rmin, dR, dxy, vo, per_set) <
               std::tie(o.tk, o.dataset, o.Rmin, o.dR, o.dxy, o.vo, o.per_set);
    }
};
struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    unsigned long long gen = 0;
    int calls = 0;
};
constexpr size_t kMaxGraphs = 32;

// cosine matrices of the tensor-core spectrum passes (one geometry) as TF32
// pairs in device memory; row-major with the leading dimensions below
struct CosMats {
    int ldF = 0, ldT = 0, ldK = 0;
    int T1 = 0;                                  // distinct |r - N/2| over the window rows: 0 .. T1 - 1
    float *ck_hi = nullptr, *ck_lo = nullptr;    // Ck   [K][ldF]
    float *cv_hi = nullptr, *cv_lo = nullptr;    // Cv   [T1][ldF]: row t = w_a cos(2 pi a t / N)
    float *cvt_hi = nullptr, *cvt_lo = nullptr;  // Cv^T [rmax+1][ldT]
    float *ckt_hi = nullptr, *ckt_lo = nullptr;  // Ck^T [rmax+1][ldK]
};
inline int round4(int x) { return (x + 3) / 4 * 4; }
// round to the nearest TF32 value, ties away from zero (cvt.rna.tf32.f32 on the host)
inline float tf32_rna_host(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    b += 0x1000u;
    b &= ~0x1FFFu;
    float r;
    std::memcpy(&r, &b, 4);
    return r;
}

struct BatchWs {
    std::mutex mu;
    Buf mc, coef, zt, win, partials, gsum, cgrad, gwin, zbar, ginc, gcentral, gI_tmp, state;
    Buf tcF, tcD1, tcG, tcG1, tcGF;  // tensor-core passes: F, D1, window gradient, G1 (TF32 pairs), dchi2/dF
    Buf tcPart, tcPinc;               // sweep adjoint: per-CTA partial profile bins and inclination sums
    std::map<std::tuple<int, int, int, int, int>, CosMats> cos;
    // Ck, Cv and their transposes for geometry g, built on the host in long double
    const CosMats& cos_mats(int N, int K, int r0, int W, int rmax) {
        const auto key = std::make_tuple(N, K, r0, W, rmax);
        auto it = cos.find(key);
        if (it != cos.end()) return it->second;
        const int n = rmax + 1;
        CosMats m;
        m.ldF = round4(n);
        m.T1 = std::max(N / 2 - r0, r0 + W - 1 - N / 2) + 1;
        m.ldT = round4(m.T1);
        m.ldK = round4(K);
        const long double two_pi = 6.283185307179586476925286766559005768L;
        auto wgt = [&](int j) { return (j == 0 || 2 * j == N) ? 1.0L : 2.0L; };
        auto cosn = [&](long long p) { return cosl(two_pi * (long double)(p % N) / (long double)N); };
        std::vector<float> ckh((size_t)K * m.ldF, 0.f), ckl(ckh.size(), 0.f);
        std::vector<float> cvh((size_t)m.T1 * m.ldF, 0.f), cvl(cvh.size(), 0.f);
        std::vector<float> cvth((size_t)n * m.ldT, 0.f), cvtl(cvth.size(), 0.f);
        std::vector<float> ckth((size_t)n * m.ldK, 0.f), cktl(ckth.size(), 0.f);
        auto put = [](std::vector<float>& h, std::vector<float>& l, size_t i, long double x) {
            const float f = (float)x;
            h[i] = tf32_rna_host(f);
            l[i] = tf32_rna_host((float)(x - (long double)h[i]));
        };
        for (int k = 0; k < K; ++k)
            for (int c = 0; c < n; ++c) {
                const long double x = wgt(c) * cosn((long long)c * k);
                put(ckh, ckl, (size_t)k * m.ldF + c, x);
                put(ckth, cktl, (size_t)c * m.ldK + k, x);
            }
        for (int t = 0; t < m.T1; ++t) {  // the spectrum is even about row N/2: one row per |r - N/2|
            for (int a = 0; a < n; ++a) {
                const long double x = wgt(a) * cosn((long long)a * t);
                put(cvh, cvl, (size_t)t * m.ldF + a, x);
                put(cvth, cvtl, (size_t)a * m.ldT + t, x);
            }
        }
        auto up = [](const std::vector<float>& h) {
            float* d = nullptr;
            cudaError_t e = cudaMalloc(&d, sizeof(float) * h.size());
            if (e == cudaSuccess) e = cudaMemcpy(d, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) throw e;
            return d;
        };
        m.ck_hi = up(ckh);
        m.ck_lo = up(ckl);
        m.cv_hi = up(cvh);
        m.cv_lo = up(cvl);
        m.cvt_hi = up(cvth);
        m.cvt_lo = up(cvtl);
        m.ckt_hi = up(ckth);
        m.ckt_lo = up(cktl);
        return cos.emplace(key, m).first->second;
    }
    Buf in_I, in_p, out_chi2, out_sets, out_gI, out_gp;  // staging of graph launches
    std::map<GraphKey, GraphEntry> graphs;
    cudaStream_t cap = nullptr;  // capture stream (captures cannot use the legacy default stream)
    void drop_graphs() {
        for (auto& kv : graphs)
            if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        graphs.clear();
    }
    std::map<TuneKey, Shape> shapes;
    std::map<std::pair<int, int>, float2*> stw;  // (L, E) -> stage twiddles
    const float2* stage_tw(int L, int E) {
        auto key = std::make_pair(L, E);
        auto it = stw.find(key);
        if (it != stw.end()) return it->second;
        std::vector<float2> h = stage_twiddles<float>(L, E);
        float2* d = nullptr;
        cudaError_t e = cudaMalloc(&d, sizeof(float2) * h.size());
        if (e == cudaSuccess) e = cudaMemcpy(d, h.data(), sizeof(float2) * h.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) throw e;
        stw[key] = d;
        return d;
    }
    std::map<int, std::pair<float2*, float2*>> tw;  // N -> (forward, conjugate)
    std::pair<float2*, float2*> twiddles(int N) {
        auto it = tw.find(N);
        if (it != tw.end()) return it->second;
        std::vector<float2> f((size_t)N), c((size_t)N);
        const long double two_pi = 6.283185307179586476925286766559005768L;
        for (int m = 0; m < N; ++m) {
            const long double a = -two_pi * (long double)m / (long double)N;
            f[(size_t)m] = make_float2((float)cosl(a), (float)sinl(a));
            c[(size_t)m] = make_float2((float)cosl(a), (float)-sinl(a));
        }
        float2 *df = nullptr, *dc = nullptr;
        cudaError_t e = cudaMalloc(&df, sizeof(float2) * N);
        if (e == cudaSuccess) e = cudaMalloc(&dc, sizeof(float2) * N);
        if (e == cudaSuccess) e = cudaMemcpy(df, f.data(), sizeof(float2) * N, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(dc, c.data(), sizeof(float2) * N, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) throw e;
        tw[N] = std::make_pair(df, dc);
        return tw[N];
    }
};

std::mutex g_bws_mu;
std::map<int, BatchWs*> g_bws;
BatchWs& batch_ws() {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_bws_mu);
    auto it = g_bws.find(dev);
    if (it != g_bws.end()) return *it->second;
    BatchWs* w = new BatchWs();
    g_bws[dev] = w;
    return *w;
}

// Visibility sets stored one after the other, each padded with zero-weight
// entries to a multiple of kSetAlign so that no block of the vis pass straddles
// two sets; within a set the visibilities are in Morton order.
constexpr int kSetAlign = kVisThreads * 4;
std::atomic<unsigned long long> g_dataset_serial{1};
struct Dataset {
    unsigned long long serial = g_dataset_serial.fetch_add(1);
    int device = 0;
    int nd = 0;       // visibilities given
    int nd_pad = 0;   // stored entries, padding included
    int nsets = 1;
    std::vector<long long> set_pad;  // nsets + 1 offsets into the padded arrays
    std::vector<int> set_nd;         // visibilities of each set
    long long* set_pad_d = nullptr;
    float *u = nullptr, *v = nullptr, *re = nullptr, *im = nullptr, *w = nullptr;
    double rmax2 = 0.0;
};

int smem_attr(const void* kern, size_t smem) {
    if (t_capturing) return 0;  // set by the eager run that precedes every capture
    if (smem > 48 * 1024)
        return (int)cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return 0;
}

#define BCK(x)                                                                                           \
    do {                                                                                                 \
        cudaError_t e_ = (x);                                                                            \
        if (e_ != cudaSuccess) {                                                                         \
            if (e_ == cudaErrorMemoryAllocation) throw Err{GALARIO_ENOMEM, "cuda out of memory"};         \
            throw Err{GALARIO_ERUNTIME, std::string("Error in cuda (" #x "): ") + cudaGetErrorString(e_)}; \
        }                                                                                                \
    } while (0)

template <class F> int bguard(F&& f) {
    try {
        f();
        return GALARIO_OK;
    } catch (const Err& e) {
        set_error_message(e.msg);
        return e.status;
    } catch (cudaError_t e) {
        set_error_message(std::string("Error in cuda: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? GALARIO_ENOMEM : GALARIO_ERUNTIME;
    } catch (const std::exception& e) {
        set_error_message(e.what());
        return GALARIO_ERUNTIME;
    }
}

// the tensor-core spectrum passes: GALARIO_TC=0 keeps the FFT passes
bool tc_enabled() {
    const char* v = std::getenv("GALARIO_TC");
    return !(v && v[0] == '0');
}

// One batched product C[z] = A[z] B[z]^T on the tensor cores (gb_tc.cuh), the
// N tile chosen to waste the fewest columns (ties: the wider tile).
template <int BN>
void tc_launch_bn(const tc::Operand& A, const tc::Operand& Bo, const tc::Params& p, int batch, cudaStream_t s) {
    CUtensorMap ah, al, bh, bl;
    if (!tc::make_map(&ah, A.hi, A, tc::BM) || !tc::make_map(&al, A.lo, A, tc::BM) ||
        !tc::make_map(&bh, Bo.hi, Bo, BN) || !tc::make_map(&bl, Bo.lo, Bo, BN))
        throw Err{GALARIO_ERUNTIME, "Error in batch: cannot encode a tensor map"};
    BCK((cudaError_t)smem_attr((const void*)tc::gemm_3xtf32_kernel<BN>, tc::Cfg<BN>::kSmem));
    const dim3 grid((p.M + tc::BM - 1) / tc::BM, (p.N + BN - 1) / BN, batch);
    tc::gemm_3xtf32_kernel<BN><<<grid, tc::kThreads, tc::Cfg<BN>::kSmem, s>>>(ah, al, bh, bl, p);
    BCK(cudaGetLastError());
}
void tc_gemm(const tc::Operand& A, const tc::Operand& Bo, const tc::Params& p, int batch, cudaStream_t s) {
    const int cand[2] = {128, 64};
    int best = 128;
    long long waste = 1LL << 60;
    for (int bn : cand) {
        const long long w = (long long)((p.N + bn - 1) / bn) * bn - p.N;
        if (w < waste) {
            waste = w;
            best = bn;
        }
    }
    if (best == 128) tc_launch_bn<128>(A, Bo, p, batch, s);
    else tc_launch_bn<64>(A, Bo, p, batch, s);
}

__global__ void extent_f32_kernel(const float* __restrict__ u, const float* __restrict__ v, int nd,
                                  double* __restrict__ out) {
    float m = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += gridDim.x * blockDim.x) {
        const float r = u[i] * u[i] + v[i] * v[i];
        m = (r == r) ? fmaxf(m, r) : __int_as_float(0x7f800000);  // NaN -> +inf: flagged as non-finite
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.f)
        atomicMax(reinterpret_cast<unsigned long long*>(out), (unsigned long long)__double_as_longlong((double)m));
}

// Morton (Z-order) key of (u, v) on a 2^15 x 2^15 grid over [-rmax, rmax]^2:
// visibilities close in the uv plane get close keys, for every rotation.
__device__ __forceinline__ unsigned spread15(unsigned x) {
    x &= 0x7fffu;
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}
__global__ void morton_kernel(const float* __restrict__ u, const float* __restrict__ v, int nd, float inv_span,
                              unsigned* __restrict__ key, int* __restrict__ idx) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += gridDim.x * blockDim.x) {
        float fu = (u[i] * inv_span + 0.5f) * 32767.f, fv = (v[i] * inv_span + 0.5f) * 32767.f;
        fu = fminf(fmaxf(fu, 0.f), 32767.f);
        fv = fminf(fmaxf(fv, 0.f), 32767.f);
        key[i] = (spread15((unsigned)fu) << 1) | spread15((unsigned)fv);
        idx[i] = i;
    }
}
// padded entry p of set k <- raw entry idx[raw[k] + (p - pad[k])], or a
// zero-weight padding entry past the set's own visibilities
__global__ void gather_sets_kernel(int nsets, const long long* __restrict__ pad, const long long* __restrict__ raw,
                                   const int* __restrict__ idx, long long nd_pad, const float* __restrict__ a0,
                                   const float* __restrict__ a1, const float* __restrict__ a2,
                                   const float* __restrict__ a3, const float* __restrict__ a4,
                                   float* __restrict__ b0, float* __restrict__ b1, float* __restrict__ b2,
                                   float* __restrict__ b3, float* __restrict__ b4) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nd_pad;
         p += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = nsets;  // largest k with pad[k] <= p
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (pad[mid] <= p) lo = mid;
            else hi = mid;
        }
        const long long jj = p - pad[lo];
        if (jj < raw[lo + 1] - raw[lo]) {
            const int j = idx[raw[lo] + jj];
            b0[p] = a0[j];
            b1[p] = a1[j];
            b2[p] = a2[j];
            b3[p] = a3[j];
            b4[p] = a4[j];
        } else {
            b0[p] = 0.f;
            b1[p] = 0.f;
            b2[p] = 0.f;
            b3[p] = 0.f;
            b4[p] = 0.f;
        }
    }
}
__global__ void iota_kernel(int* __restrict__ idx, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) idx[i] = i;
}

// (values per thread EE, block-size bound TT, compile-time log2 length LG)
// for an FFT of length L_ with E_ values per thread: lengths 2^9..2^13 get the
// compile-time FFT, others the run-time one (LG = 0)
#define GBB_CASE_T(E_V, THR, ...)                                                          \
    {                                                                                      \
        constexpr int EE = E_V;                                                            \
        constexpr int LG = 0;                                                              \
        if ((THR) <= 256) { constexpr int TT = 256; __VA_ARGS__; }                         \
        else if ((THR) <= 512) { constexpr int TT = 512; __VA_ARGS__; }                    \
        else { constexpr int TT = 1024; __VA_ARGS__; }                                     \
    }
#define GBB_CASE_LG(E_V, LG_V, ...)                                                        \
    {                                                                                      \
        constexpr int EE = E_V;                                                            \
        constexpr int LG = LG_V;                                                           \
        constexpr int TT = ((1 << LG_V) / E_V) <= 256 ? 256 : ((1 << LG_V) / E_V);          \
        __VA_ARGS__;                                                                       \
    }
#define GBB_CASE_EL(E_V, L_, ...)                                                          \
    switch (L_) {                                                                          \
        case 512: GBB_CASE_LG(E_V, 9, __VA_ARGS__) break;                                  \
        case 1024: GBB_CASE_LG(E_V, 10, __VA_ARGS__) break;                                \
        case 2048: GBB_CASE_LG(E_V, 11, __VA_ARGS__) break;                                \
        case 4096: GBB_CASE_LG(E_V, 12, __VA_ARGS__) break;                                \
        case 8192: GBB_CASE_LG(E_V, 13, __VA_ARGS__) break;                                \
        default: GBB_CASE_T(E_V, (L_) / (E_V), __VA_ARGS__) break;                         \
    }
#define GBB_DISPATCH_E(E_, L_, ...)                                       \
    switch (E_) {                                                         \
        case 8: GBB_CASE_EL(8, L_, __VA_ARGS__) break;                    \
        case 16: GBB_CASE_EL(16, L_, __VA_ARGS__) break;                  \
        default: throw Err{GALARIO_EINVAL, "unsupported FFT length"};     \
    }

}  // namespace
}  // namespace gbg

using namespace gbg;

#define API extern "C" __attribute__((visibility("default")))

API int galario_dataset_create_f(int nd, const float* u, const float* v, const float* re, const float* im,
                                 const float* w, int nsets, const int* set_offsets, int on_device, void** handle) {
    return bguard([&] {
        if (nd <= 0) throw Err{GALARIO_EINVAL, "Error in dataset: nd must be positive"};
        if (!handle) throw Err{GALARIO_EINVAL, "Error in dataset: handle is NULL"};
        if (nsets < 1) throw Err{GALARIO_EINVAL, "Error in dataset: nsets must be positive"};
        if (!set_offsets && nsets != 1) throw Err{GALARIO_EINVAL, "Error in dataset: set_offsets is NULL"};
        std::vector<long long> raw((size_t)nsets + 1);
        for (int k = 0; k <= nsets; ++k) raw[k] = set_offsets ? set_offsets[k] : (k ? nd : 0);
        if (raw[0] != 0 || raw[nsets] != nd)
            throw Err{GALARIO_EINVAL, "Error in dataset: set_offsets must start at 0 and end at nd"};
        std::unique_ptr<Dataset> d(new Dataset());
        d->nsets = nsets;
        d->set_pad.assign((size_t)nsets + 1, 0);
        d->set_nd.assign((size_t)nsets, 0);
        for (int k = 0; k < nsets; ++k) {
            const long long n = raw[k + 1] - raw[k];
            if (n < 0) throw Err{GALARIO_EINVAL, "Error in dataset: set_offsets must not decrease"};
            d->set_nd[k] = (int)n;
            d->set_pad[k + 1] = d->set_pad[k] + (n + kSetAlign - 1) / kSetAlign * kSetAlign;
        }
        if (d->set_pad[nsets] > (long long)INT_MAX - kSetAlign)
            throw Err{GALARIO_EINVAL, "Error in dataset: too many visibilities"};
        const long long nd_pad = d->set_pad[nsets];
        BCK(cudaGetDevice(&d->device));
        d->nd = nd;
        d->nd_pad = (int)nd_pad;
        const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        const float* src[5] = {u, v, re, im, w};
        float* raw_d[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
        float** dst[5] = {&d->u, &d->v, &d->re, &d->im, &d->w};
        unsigned *k0 = nullptr, *k1 = nullptr;
        int *i0 = nullptr, *i1 = nullptr;
        long long* raw_off_d = nullptr;
        double* r2 = nullptr;
        void* cub_tmp = nullptr;
        auto cleanup = [&] {
            for (float* t : raw_d) cudaFree(t);
            cudaFree(k0); cudaFree(k1); cudaFree(i0); cudaFree(i1);
            cudaFree(raw_off_d); cudaFree(r2); cudaFree(cub_tmp);
        };
        try {
            for (int i = 0; i < 5; ++i) {
                BCK(cudaMalloc(&raw_d[i], sizeof(float) * (size_t)nd));
                BCK(cudaMemcpy(raw_d[i], src[i], sizeof(float) * (size_t)nd, kind));
            }
            BCK(cudaMalloc(&r2, sizeof(double)));
            BCK(cudaMemset(r2, 0, sizeof(double)));
            extent_f32_kernel<<<num_sms() * 4, 256>>>(raw_d[0], raw_d[1], nd, r2);
            BCK(cudaGetLastError());
            BCK(cudaMemcpy(&d->rmax2, r2, sizeof(double), cudaMemcpyDeviceToHost));
            if (!std::isfinite(d->rmax2)) throw Err{GALARIO_EINVAL, "Error in dataset: u and v must be finite"};
            BCK(cudaMalloc(&i0, sizeof(int) * (size_t)nd));
            BCK(cudaMalloc(&i1, sizeof(int) * (size_t)nd));
            const int* order = i0;
            if (d->rmax2 > 0.0 && std::isfinite(d->rmax2)) {
                // spatial order within each set (chi2 is a sum: the order changes only the rounding)
                BCK(cudaMalloc(&k0, sizeof(unsigned) * (size_t)nd));
                BCK(cudaMalloc(&k1, sizeof(unsigned) * (size_t)nd));
                const float inv_span = (float)(0.5 / (std::sqrt(d->rmax2) * 1.0000001));
                morton_kernel<<<num_sms() * 4, 256>>>(raw_d[0], raw_d[1], nd, inv_span, k0, i0);
                BCK(cudaGetLastError());
                size_t cub_bytes = 0;
                for (int k = 0; k < nsets; ++k) {
                    size_t b = 0;
                    if (d->set_nd[k] == 0) continue;
                    BCK(cub::DeviceRadixSort::SortPairs(nullptr, b, k0, k1, i0, i1, d->set_nd[k], 0, 30));
                    cub_bytes = std::max(cub_bytes, b);
                }
                BCK(cudaMalloc(&cub_tmp, cub_bytes ? cub_bytes : 16));
                for (int k = 0; k < nsets; ++k) {
                    if (d->set_nd[k] == 0) continue;
                    size_t b = cub_bytes;
                    BCK(cub::DeviceRadixSort::SortPairs(cub_tmp, b, k0 + raw[k], k1 + raw[k], i0 + raw[k],
                                                        i1 + raw[k], d->set_nd[k], 0, 30));
                }
                order = i1;
            } else {
                iota_kernel<<<num_sms() * 4, 256>>>(i0, nd);
                BCK(cudaGetLastError());
            }
            BCK(cudaMalloc(&raw_off_d, sizeof(long long) * raw.size()));
            BCK(cudaMemcpy(raw_off_d, raw.data(), sizeof(long long) * raw.size(), cudaMemcpyHostToDevice));
            BCK(cudaMalloc(&d->set_pad_d, sizeof(long long) * d->set_pad.size()));
            BCK(cudaMemcpy(d->set_pad_d, d->set_pad.data(), sizeof(long long) * d->set_pad.size(),
                           cudaMemcpyHostToDevice));
            for (int i = 0; i < 5; ++i) BCK(cudaMalloc(dst[i], sizeof(float) * (size_t)nd_pad));
            gather_sets_kernel<<<num_sms() * 4, 256>>>(nsets, d->set_pad_d, raw_off_d, order, nd_pad, raw_d[0],
                                                      raw_d[1], raw_d[2], raw_d[3], raw_d[4], d->u, d->v, d->re,
                                                      d->im, d->w);
            BCK(cudaGetLastError());
            BCK(cudaDeviceSynchronize());
        } catch (...) {
            cleanup();
            for (int i = 0; i < 5; ++i)
                if (*dst[i]) cudaFree(*dst[i]);
            cudaFree(d->set_pad_d);
            throw;
        }
        cleanup();
        *handle = d.release();
    });
}

API int galario_dataset_free(void* handle) {
    return bguard([&] {
        Dataset* d = static_cast<Dataset*>(handle);
        if (!d) return;
        cudaDeviceSynchronize();
        float* p[5] = {d->u, d->v, d->re, d->im, d->w};
        for (float* x : p) cudaFree(x);
        cudaFree(d->set_pad_d);
        delete d;
    });
}

API int galario_dataset_nvis(void* handle, int* nd) {
    return bguard([&] {
        if (!handle) throw Err{GALARIO_EINVAL, "Error in dataset: handle is NULL"};
        *nd = static_cast<Dataset*>(handle)->nd;
    });
}

API int galario_batch_status(unsigned int* err_bits) {
    return bguard([&] {
        if (!err_bits) throw Err{GALARIO_EINVAL, "Error in batch: err_bits is NULL"};
        BatchWs& ws = batch_ws();
        std::lock_guard<std::mutex> lk(ws.mu);
        BCK(cudaDeviceSynchronize());
        DevState* st = ws.state.get<DevState>(1);
        unsigned int e = 0;
        BCK(cudaMemcpy(&e, &st->err, sizeof(unsigned int), cudaMemcpyDeviceToHost));
        *err_bits = e;
    });
}

API int galario_dataset_nsets(void* handle, int* nsets) {
    return bguard([&] {
        if (!handle) throw Err{GALARIO_EINVAL, "Error in dataset: handle is NULL"};
        *nsets = static_cast<Dataset*>(handle)->nsets;
    });
}

// One batched call: B models (radial profiles or images) against a dataset.
struct BatchCall {
    gbg::Dataset* d = nullptr;
    int B = 0;
    bool image = false;
    int nr = 0;                        // profiles: samples per profile
    const float* input = nullptr;      // profiles (B x nr) or images (B x nxy x nxy)
    float Rmin = 0.f, dR = 0.f;        // profiles
    float dxy = 0.f, vo = 1.f;
    int nxy = 0;
    const float* params = nullptr;     // B x pstride
    int pstride = 4;
    double* chi2 = nullptr;
    double* chi2_sets = nullptr;
    float* grad_input = nullptr;
    float* grad_params = nullptr;
    void* stream = nullptr;
};

static void batch_run(const BatchCall& call) {
        Dataset* d = call.d;
        const int B = call.B;
        const bool image = call.image;
        const int nr = image ? 0 : call.nr;
        const float* intensity = call.input;  // the model input: profiles or images
        const float Rmin = call.Rmin, dR = call.dR, dxy = call.dxy;
        const int nxy = call.nxy;
        const float* params = call.params;
        const int pstride = call.pstride;
        double* chi2 = call.chi2;
        double* chi2_sets = call.chi2_sets;
        float* grad_intensity = call.grad_input;
        float* grad_params = call.grad_params;
        void* stream = call.stream;
        if (!d) throw Err{GALARIO_EINVAL, "Error in batch: dataset is NULL"};
        if (B <= 0) throw Err{GALARIO_EINVAL, "Error in batch: B must be positive"};
        if (nxy < 2 || (nxy & 1))
            throw Err{GALARIO_EINVAL, "Error in check input image: x dimension = " + std::to_string(nxy) +
                                          (nxy < 2 ? " is less than 2" : " is odd")};
        if (nxy < 16 || nxy > 16384) throw Err{GALARIO_EINVAL, "Error in batch: nxy must lie in [16, 16384]"};
        if (!image) {
            const double ratio = ((double)dxy / 2. - (double)Rmin) / (double)dR;
            if (ratio < 5)
                throw Err{GALARIO_EINVAL,
                          "Error in create image: Expect (dxy/2-Rmin)/dR > 5, i.e. dR small enough to ensure reliable "
                          "interpolation the inside central pixel but got (dxy/2-Rmin)/dR = " +
                              std::to_string(ratio) + ". Try reducing dR."};
        }
        const bool grad = grad_intensity || grad_params;
        if (grad && !(grad_intensity && grad_params))
            throw Err{GALARIO_EINVAL, "Error in batch: pass both gradient outputs or neither"};
        cudaStream_t s = static_cast<cudaStream_t>(stream);  // the launchers below enqueue on `s`
        const cudaStream_t s_user = s;
        BatchWs& ws = batch_ws();
        std::lock_guard<std::mutex> lk(ws.mu);

        // ---- geometry (host) ----
        Geo g;
        g.N = nxy;
        g.M = nxy / 2;
        g.C = nxy / 2 + 1;
        const double duv = (double)(float)(1.0 / ((double)dxy * nxy));  // as the FP32 module passes it
        {
            const double ext = std::sqrt(d->rmax2) / duv;
            if (!(ext * (1.0 + 2e-6) + 1e-6 + 2.0 < (double)(nxy / 2)))
                throw Err{GALARIO_EINVAL, "Error in batch: the visibilities reach max|uv|/duv = " +
                                              std::to_string(ext) + ", beyond the image's uv range (nxy/2 - 2 = " +
                                              std::to_string(nxy / 2 - 2) + "); increase nxy or reduce dxy"};
        }
        const Window w = window_from_extent(d->rmax2, duv, nxy);
        g.K = w.K;
        g.r0 = w.r0;
        g.W = w.W;
        if (image) {  // every row of the image is transformed
            g.rmax = nxy / 2;
            g.band0 = 0;
            g.R = nxy;
        } else {
            long long rm = (long long)std::ceil(((double)Rmin + nr * (double)dR) / (double)dxy);
            g.rmax = (int)(rm < nxy / 2 ? rm : nxy / 2);
            g.band0 = nxy / 2 - g.rmax;
            g.R = 2 * g.rmax;
        }
        g.nr = nr;
        g.Rmin = Rmin;
        g.dR = dR;
        g.inv_dR = image ? 0.f : (float)(1.0 / (double)dR);
        g.dxy = dxy;
        g.sr_to_px = dxy * dxy;
        const double inv_duv = 1.0 / duv;
        g.inv_duv_hi = (float)inv_duv;
        g.inv_duv_lo = (float)(inv_duv - (double)g.inv_duv_hi);
        g.half_nrow = (float)(nxy / 2);
        g.vo = call.vo;
        if (g.R <= 0) throw Err{GALARIO_EINVAL, "Error in batch: empty profile support"};
        if (!image && (nr < 2 || nr >= (1 << 22))) throw Err{GALARIO_EINVAL, "Error in batch: nr out of range"};
        // central-pixel coefficients of profiles: central = sum_i coef_i I_i (reference :1136-1153)
        const int iIN = image ? 0 : (int)std::floor(((double)dxy / 2 - (double)Rmin) / (double)dR);
        if (!image && (iIN < 0 || iIN + 1 >= nr))
            throw Err{GALARIO_EINVAL, "Error in create image: profile too short"};
        g.iIN = iIN;
        std::vector<double> coef(image ? 0 : (size_t)iIN + 2, 0.0);
        if (!image) {
            const double Rm = Rmin, dr = dR, h = (double)dxy / 2.;
            for (int i = 1; i < iIN; ++i) coef[i] += 2. * dr * (Rm + dr * i);
            coef[0] += dr * Rm;
            coef[iIN] += dr * (Rm + iIN * dr);
            const double span = h - (Rm + iIN * dr);
            // ((Rm + iIN dr) I_iIN + h I_interp) * span, I_interp = (I_{iIN+1} - I_iIN)/dr * span + I_iIN
            coef[iIN] += (Rm + iIN * dr) * span;
            coef[iIN] += h * span * (1. - span / dr);
            coef[iIN + 1] += h * span * (span / dr);
            const double area = h * h - Rm * Rm;
            const double sr = (double)dxy * (double)dxy;
            for (auto& c : coef) c *= sr / area;
        }
        const int ncoef = image ? 0 : iIN + 2;

        // ---- buffers ----
        const long long ncell = (long long)g.K * g.W;
        ModelConst* mc = ws.mc.get<ModelConst>((size_t)B);
        double* coef_d = ws.coef.get<double>((size_t)ncoef);
        float2* zt = ws.zt.get<float2>((size_t)B * g.K * g.R);
        float4* wel = ws.win.get<float4>((size_t)B * ncell);  // window elements (re, im, |.|, 0)
        const int max_vblocks = (int)((d->nd_pad + (long long)kVisThreads * 2 - 1) / ((long long)kVisThreads * 2));
        double* partials = ws.partials.get<double>((size_t)max_vblocks * B * kAcc);
        double* gsum = ws.gsum.get<double>((size_t)B * kAcc);
        auto tws = ws.twiddles(nxy);
        if (ncoef) BCK(cudaMemcpyAsync(coef_d, coef.data(), sizeof(double) * ncoef, cudaMemcpyHostToDevice, s));
        DevState* st = ws.state.get<DevState>(1);
        BCK(cudaMemsetAsync(st, 0, sizeof(DevState), s));
        // swept profiles have a real spectrum: real window, 4-float gradient records
        const bool real = !image;
        const int recf = real ? 4 : kGRec;
        float* cgrad = grad ? ws.cgrad.get<float>((size_t)B * ncell * recf) : nullptr;
        float2* gwin = grad ? ws.gwin.get<float2>((size_t)B * ncell) : nullptr;
        float2* zbar = grad ? ws.zbar.get<float2>((size_t)B * g.K * g.R) : nullptr;
        double* ginc_d = grad ? ws.gI_tmp.get<double>((size_t)B) : nullptr;
        float* gcentral = grad ? ws.gcentral.get<float>((size_t)B) : nullptr;
        // models per group of the vis pass: the group's windows and gradient records within ~64 MiB of L2
        const double rec_bytes = (double)ncell * ((real ? sizeof(float) : sizeof(float4)) + (grad ? recf * sizeof(float) : 0));
        int Bg = (int)std::floor(64.0 * 1024 * 1024 / rec_bytes);
        if (Bg < 1) Bg = 1;
        if (Bg > B) Bg = B;
        const int ngroups = (B + Bg - 1) / Bg;

        // tensor-core spectrum passes for swept profiles (products with the
        // cosine matrices) where the folded quadrant, the window and the
        // profile bins fit; the FFT passes otherwise
        const int nF = g.rmax + 1;
        const bool use_tc = real && tc_enabled() && tc::encode_fn() != nullptr && nF <= 2048 && g.K <= 2048 &&
                            g.W <= 4096 && (size_t)nr * sizeof(float) <= 160 * 1024;
        // the FFT passes need a power of two; the cosine-matrix products take any even nxy
        if (!use_tc && !is_pow2(nxy))
            throw Err{GALARIO_EINVAL, std::string("Error in batch: nxy must be a power of two in [16, 16384]") +
                                          (image ? "" : " (profiles on the tensor-core passes take any even nxy)")};
        const CosMats* cm = use_tc ? &ws.cos_mats(g.N, g.K, g.r0, g.W, g.rmax) : nullptr;
        float *tF = nullptr, *tD1 = nullptr, *tG = nullptr, *tG1 = nullptr, *tGF = nullptr, *tPart = nullptr;
        double* tPinc = nullptr;
        if (use_tc) {
            tF = ws.tcF.get<float>((size_t)2 * B * nF * cm->ldF);
            tD1 = ws.tcD1.get<float>((size_t)2 * B * g.K * cm->ldF);
            if (grad) {
                tG = ws.tcG.get<float>((size_t)2 * B * g.K * cm->ldT);
                tG1 = ws.tcG1.get<float>((size_t)2 * B * nF * cm->ldK);
                tGF = ws.tcGF.get<float>((size_t)B * nF * cm->ldF);
                const size_t nchunk = (size_t)(nF + kRowsPerCta - 1) / kRowsPerCta;
                tPart = ws.tcPart.get<float>((size_t)B * nchunk * nr);
                tPinc = ws.tcPinc.get<double>((size_t)B * nchunk);
            }
        }

        // folded rows per staging group of the row passes: 2F rows x K columns
        // within 20 KiB; the adjoint runs G groups per CTA to amortise its flush
        const int Fcap = std::max(1, (int)((20 * 1024) / (sizeof(float2) * 2 * (size_t)g.K) - 1));
        const int Frows = std::min(4, Fcap);
        const int GrowsT = std::max(1, kRowsPerCta / Frows);
        // ---- launchers, one per pass, parameterised by the tuned shape ----
        auto fft_threads = [](int L, int E) { return L / E; };
        auto check_smem = [](size_t sm) {
            if (sm > 227 * 1024)
                throw Err{GALARIO_EINVAL, "Error in batch: nxy and the uv coverage need " + std::to_string(sm) +
                                              " bytes of shared memory per block (at most 232448)"};
        };
        const int Fimg = 2 * Frows;  // image rows per CTA of the image row passes
        auto rows = [&](int E) {
            if (image) {
                const size_t sm = sizeof(float2) * (fft_slots(g.M) + (size_t)g.K * (Fimg + 1));
                check_smem(sm);
                GBB_DISPATCH_E(E, g.M, {
                    BCK((cudaError_t)smem_attr((const void*)rows_image_batch_kernel<EE, TT, LG>, sm));
                    rows_image_batch_kernel<EE, TT, LG><<<dim3((g.N + Fimg - 1) / Fimg, B), fft_threads(g.M, EE), sm, s>>>(
                        g, Fimg, intensity, tws.first, ws.stage_tw(g.M, EE), zt);
                });
                BCK(cudaGetLastError());
                return;
            }
            const size_t sm = sizeof(float2) * (fft_slots(g.M) + (size_t)g.K * (2 * Frows + 1)) +
                              sizeof(float) * (g.rmax + 1);
            check_smem(sm);
            GBB_DISPATCH_E(E, g.M, {
                BCK((cudaError_t)smem_attr((const void*)rows_batch_kernel<EE, TT, LG>, sm));
                rows_batch_kernel<EE, TT, LG><<<dim3((g.rmax + Frows) / Frows, B), fft_threads(g.M, EE), sm, s>>>(
                    g, Frows, intensity, mc, tws.first, ws.stage_tw(g.M, EE), (void*)zt, real ? 1 : 0);
            });
            BCK(cudaGetLastError());
        };
        // column pass shape: E values per thread, + kTmaCols for the TMA-fed persistent variant
        const bool tma_ok = !real && (g.R % 2 == 0) &&
                            sizeof(float2) * (2 * (size_t)g.R + fft_slots(g.N)) + 16 <= 200 * 1024;
        auto cols = [&](int shape) {
            const int E = shape % kTmaCols;
            if (shape >= kTmaCols) {
                const size_t sm = sizeof(float2) * (2 * (size_t)g.R + fft_slots(g.N)) + 2 * sizeof(unsigned long long);
                const int total = g.K * B;
                GBB_DISPATCH_E(E, g.N, {
                    const void* fn = (const void*)cols_batch_tma_kernel<EE, TT, LG>;
                    BCK((cudaError_t)smem_attr(fn, sm));
                    int per_sm = 0;
                    BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cols_batch_tma_kernel<EE, TT, LG>,
                                                                      fft_threads(g.N, EE), sm));
                    const int grid = std::max(1, std::min(total, num_sms() * std::max(per_sm, 1)));
                    cols_batch_tma_kernel<EE, TT, LG><<<grid, fft_threads(g.N, EE), sm, s>>>(
                        g, total, zt, ws.stage_tw(g.N, EE), wel, st);
                });
                BCK(cudaGetLastError());
                return;
            }
            const size_t sm = sizeof(float2) * fft_slots(g.N);
            if (real) {
                GBB_DISPATCH_E(E, g.N, {
                    BCK((cudaError_t)smem_attr((const void*)cols_pair_batch_kernel<EE, TT, LG>, sm));
                    cols_pair_batch_kernel<EE, TT, LG><<<dim3((g.K + 1) / 2, B), fft_threads(g.N, EE), sm, s>>>(
                        g, reinterpret_cast<const float*>(zt), ws.stage_tw(g.N, EE), reinterpret_cast<float*>(wel));
                });
                BCK(cudaGetLastError());
                return;
            }
            GBB_DISPATCH_E(E, g.N, {
                BCK((cudaError_t)smem_attr((const void*)cols_batch_kernel<EE, TT, LG>, sm));
                cols_batch_kernel<EE, TT, LG><<<dim3(g.K, B), fft_threads(g.N, EE), sm, s>>>(
                    g, zt, ws.stage_tw(g.N, EE), wel);
            });
            BCK(cudaGetLastError());
        };
        auto vis = [&](int pts) {
            const int nt = vis_threads(pts);
            const int vb = (int)((d->nd_pad + (long long)nt * pts - 1) / ((long long)nt * pts));
            const size_t vsm = sizeof(ModelConst) * Bg + sizeof(float) * Bg * kAcc * (nt / 32) +
                               (grad ? sizeof(float) * nt * (real ? 5 : kFirstStride) : 0);
            const dim3 grid(vb, ngroups);
#define GBB_VIS(G_, P_, R_)                                                                                    \
    do {                                                                                                       \
        constexpr int NT_ = vis_threads(P_);                                                                   \
        BCK((cudaError_t)smem_attr((const void*)vis_batch_kernel<G_, P_, R_, NT_>, vsm));                      \
        vis_batch_kernel<G_, P_, R_, NT_><<<grid, NT_, vsm, s>>>(g, B, Bg, d->nd_pad, d->u, d->v, d->re,      \
                                                                d->im, d->w, mc, (const void*)wel, cgrad,     \
                                                                partials, st);                                \
    } while (0)
            if (real) {
                if (grad) {
                    if (pts == 2) GBB_VIS(true, 2, true);
                    else if (pts == 8) GBB_VIS(true, 8, true);
                    else GBB_VIS(true, 4, true);
                } else {
                    if (pts == 2) GBB_VIS(false, 2, true);
                    else if (pts == 8) GBB_VIS(false, 8, true);
                    else GBB_VIS(false, 4, true);
                }
            } else {
                if (grad) {
                    if (pts == 2) GBB_VIS(true, 2, false);
                    else GBB_VIS(true, 4, false);
                } else {
                    if (pts == 2) GBB_VIS(false, 2, false);
                    else GBB_VIS(false, 4, false);
                }
            }
#undef GBB_VIS
            BCK(cudaGetLastError());
            return vb;
        };
        auto colsT = [&](int E) {
            const size_t sm = sizeof(float2) * fft_slots(g.N);
            if (real) {
                GBB_DISPATCH_E(E, g.N, {
                    BCK((cudaError_t)smem_attr((const void*)colsT_pair_batch_kernel<EE, TT, LG>, sm));
                    colsT_pair_batch_kernel<EE, TT, LG><<<dim3((g.K + 1) / 2, B), fft_threads(g.N, EE), sm, s>>>(
                        g, reinterpret_cast<const float*>(gwin), ws.stage_tw(g.N, EE), zbar);
                });
                BCK(cudaGetLastError());
                return;
            }
            GBB_DISPATCH_E(E, g.N, {
                BCK((cudaError_t)smem_attr((const void*)colsT_batch_kernel<EE, TT, LG>, sm));
                colsT_batch_kernel<EE, TT, LG><<<dim3(g.K, B), fft_threads(g.N, EE), sm, s>>>(
                    g, gwin, ws.stage_tw(g.N, EE), zbar);
            });
            BCK(cudaGetLastError());
        };
        auto rowsT = [&](int E) {
            if (image) {
                const size_t smi = sizeof(float2) * (fft_slots(g.M) + (size_t)g.K * (Fimg + 1));
                check_smem(smi);
                GBB_DISPATCH_E(E, g.M, {
                    BCK((cudaError_t)smem_attr((const void*)rowsT_image_batch_kernel<EE, TT, LG>, smi));
                    rowsT_image_batch_kernel<EE, TT, LG><<<dim3((g.N + Fimg - 1) / Fimg, B), fft_threads(g.M, EE), smi, s>>>(
                        g, Fimg, ws.stage_tw(g.M, EE), tws.second, zbar, grad_intensity);
                });
                BCK(cudaGetLastError());
                return;
            }
            const size_t sm = sizeof(float2) * (fft_slots(g.M) + (size_t)g.K * (2 * Frows + 1)) +
                              sizeof(float) * (nr + g.rmax + 1);
            check_smem(sm);
            GBB_DISPATCH_E(E, g.M, {
                BCK((cudaError_t)smem_attr((const void*)rowsT_batch_kernel<EE, TT, LG>, sm));
                rowsT_batch_kernel<EE, TT, LG><<<dim3((g.rmax + Frows * GrowsT) / (Frows * GrowsT), B), fft_threads(g.M, EE), sm, s>>>(
                    g, Frows, GrowsT, intensity, mc, ws.stage_tw(g.M, EE), tws.second, zbar, grad_intensity, ginc_d, gcentral);
            });
            BCK(cudaGetLastError());
        };
        // forward spectrum passes on the tensor cores: F -> D1 = Ck F^T -> S' = D1 Cv^T,
        // S' over the distinct |r - N/2| and written to both mirror rows of the window
        auto tc_forward = [&] {
            const size_t sF = (size_t)nF * cm->ldF, sD = (size_t)g.K * cm->ldF;
            sweep_fold_kernel<<<dim3((nF * nF + 255) / 256, B), 256, 0, s>>>(g, intensity, mc, tF, tF + B * sF,
                                                                             cm->ldF);
            BCK(cudaGetLastError());
            const tc::Operand a1{cm->ck_hi, cm->ck_lo, g.K, nF, cm->ldF, 0, 1};
            const tc::Operand b1{tF, tF + B * sF, nF, nF, cm->ldF, (long long)sF, B};
            const tc::Params p1{g.K, nF, nF, tD1, tD1 + B * sD, (long long)sD, cm->ldF, tc::kStoreTf32, 0, 1, &st->err};
            tc_gemm(a1, b1, p1, B, s);
            const tc::Operand a2{tD1, tD1 + B * sD, g.K, nF, cm->ldF, (long long)sD, B};
            const tc::Operand b2{cm->cv_hi, cm->cv_lo, cm->T1, nF, cm->ldF, 0, 1};
            tc::Params p2{g.K, cm->T1, nF, reinterpret_cast<float*>(wel), nullptr, (long long)ncell, g.W,
                          tc::kStoreMirror, 1, 0, &st->err};
            p2.mirror_h0 = g.N / 2 - g.r0;
            tc_gemm(a2, b2, p2, B, s);
        };
        // adjoint on the tensor cores: window gradient G -> G1 = Cv^T G^T -> dchi2/dF = G1 Ck -> sweep adjoint
        auto tc_adjoint = [&] {
            const size_t sG = (size_t)g.K * cm->ldT, sG1 = (size_t)nF * cm->ldK, sF = (size_t)nF * cm->ldF;
            quadT_real_tc_kernel<<<dim3(g.K, B), 256, 0, s>>>(g, cgrad, reinterpret_cast<const float*>(wel), tG,
                                                              tG + B * sG, cm->T1, cm->ldT);
            BCK(cudaGetLastError());
            const tc::Operand a1{cm->cvt_hi, cm->cvt_lo, nF, cm->T1, cm->ldT, 0, 1};
            const tc::Operand b1{tG, tG + B * sG, g.K, cm->T1, cm->ldT, (long long)sG, B};
            const tc::Params p1{nF, g.K, cm->T1, tG1, tG1 + B * sG1, (long long)sG1, cm->ldK, tc::kStoreTf32, 0, 1,
                                &st->err};
            tc_gemm(a1, b1, p1, B, s);
            const tc::Operand a2{tG1, tG1 + B * sG1, nF, g.K, cm->ldK, (long long)sG1, B};
            const tc::Operand b2{cm->ckt_hi, cm->ckt_lo, nF, g.K, cm->ldK, 0, 1};
            const tc::Params p2{nF, nF, g.K, tGF, nullptr, (long long)sF, cm->ldF, tc::kStore, 1, 0, &st->err};
            tc_gemm(a2, b2, p2, B, s);
            const size_t smA = sizeof(float) * nr;
            const int nchunk = (nF + kRowsPerCta - 1) / kRowsPerCta;
            BCK((cudaError_t)smem_attr((const void*)sweep_adjoint_kernel, smA));
            sweep_adjoint_kernel<<<dim3(nchunk, B), 256, smA, s>>>(g, intensity, mc, tGF, cm->ldF, tPart, tPinc,
                                                                   gcentral);
            BCK(cudaGetLastError());
            sweep_adjoint_reduce_kernel<<<dim3((nr + 255) / 256, B), 256, 0, s>>>(nr, nchunk, tPart, tPinc,
                                                                                 grad_intensity, ginc_d);
            BCK(cudaGetLastError());
        };
        auto zero_grads = [&] {
            BCK(cudaMemsetAsync(cgrad, 0, sizeof(float) * (size_t)B * ncell * recf, s));
            BCK(cudaMemsetAsync(ginc_d, 0, sizeof(double) * B, s));
            BCK(cudaMemsetAsync(gcentral, 0, sizeof(float) * B, s));
            if (!image) BCK(cudaMemsetAsync(grad_intensity, 0, sizeof(float) * (size_t)B * nr, s));
        };

        // ---- the launch sequence of one call, for the launch shapes in `sh` ----
        Shape sh = default_shape(g);
        auto run_all = [&] {
            BCK(cudaMemsetAsync(st, 0, sizeof(DevState), s));
            model_setup_kernel<<<(B + 31) / 32, 32, 0, s>>>(B, params, pstride, intensity, nr, coef_d, ncoef, inv_duv,
                                                             mc);
            BCK(cudaGetLastError());
            if (use_tc) {
                tc_forward();
            } else {
                rows(sh.e_rows);
                cols(sh.e_cols);
            }
            if (grad) zero_grads();
            vis(sh.pts);
            batch_finalize_kernel<<<dim3(B, grad ? kAcc : 1), 256, 0, s>>>(
                B, d->nsets, d->set_pad_d, vis_threads(sh.pts) * sh.pts, partials, chi2, chi2_sets, gsum);
            BCK(cudaGetLastError());
            if (!grad) return;
            // ---- adjoint ----
            if (use_tc) {
                tc_adjoint();
            } else {
                if (real)
                    quadT_real_kernel<<<dim3(g.K, B), 256, 0, s>>>(g, cgrad, reinterpret_cast<const float*>(wel),
                                                                   reinterpret_cast<float*>(gwin));
                else
                    quadT_batch_kernel<<<dim3(g.K, B), 256, 0, s>>>(g, cgrad, wel, gwin);
                BCK(cudaGetLastError());
                colsT(sh.e_colsT);
                rowsT(sh.e_rowsT);
            }
            if (!image) {
                central_adjoint_kernel<<<B, 64, 0, s>>>(B, nr, coef_d, ncoef, gcentral, grad_intensity);
                BCK(cudaGetLastError());
            }
            write_grad_params_kernel<<<(B + 127) / 128, 128, 0, s>>>(B, pstride, gsum, ginc_d, grad_params);
            BCK(cudaGetLastError());
        };

        // ---- launch shapes: tuned once per geometry ----
        // Coordinate descent over the passes, every candidate timed inside a
        // complete call (so that each pass sees the cache state it has in
        // production), best of three interleaved timings.
        const TuneKey key{g.N, g.K, g.W, g.R, B, d->nd_pad, grad ? 1 : 0, nr, image ? 1 : 0, use_tc ? 1 : 0};
        auto it = ws.shapes.find(key);
        const bool tuned = it != ws.shapes.end();
        tune::Key fkey;
        Shape fsh;
        const bool from_file = !tuned && autotune_enabled() &&
                               (fkey = tune_file_key(g.N, g.K, g.W, g.R, B, d->nd_pad, grad ? 1 : 0, nr,
                                                      image ? 1 : (use_tc ? 2 : 0)),
                                tune_file().lookup(fkey, &fsh)) &&
                               shape_valid(g, fsh, real, tma_ok, use_tc);
        if (tuned) {
            sh = it->second;
        } else if (from_file) {
            sh = fsh;
            ws.shapes[key] = sh;
        } else if (autotune_enabled()) {
            Tuner tu(s);
            std::vector<int> col_shapes = fft_candidates(g.N);
            if (tma_ok)
                for (int e : fft_candidates(g.N)) col_shapes.push_back(e + kTmaCols);
            // the tensor-core passes have no FFT shapes to tune
            if (!use_tc) {
                sh.e_rows = tu.best(fft_candidates(g.M), [&](int e) { sh.e_rows = e; run_all(); });
                sh.e_cols = tu.best(col_shapes, [&](int e) { sh.e_cols = e; run_all(); });
            }
            // the visibility pass alone decides its shape (the spectrum passes
            // before it do not depend on it and only add noise): one complete
            // call sets up the window, then each candidate reruns the pass
            // (the gradient records it accumulates are zeroed by the next call)
            run_all();
            sh.pts = tu.best(real ? std::vector<int>{2, 4, 8} : std::vector<int>{2, 4}, [&](int p) { vis(p); });
            if (grad && !use_tc) {
                sh.e_colsT = tu.best(fft_candidates(g.N), [&](int e) { sh.e_colsT = e; run_all(); });
                sh.e_rowsT = tu.best(fft_candidates(g.M), [&](int e) { sh.e_rowsT = e; run_all(); });
            }
            ws.shapes[key] = sh;
            tune_file().store(fkey, sh);
        }

        // First call of a combination: eager (it also sets the kernels'
        // attributes and creates the tables); from the second on, one
        // captured CUDA graph per combination, fed through staging buffers.
        const GraphKey gk{key, d->serial, Rmin, dR, dxy, g.vo, chi2_sets ? 1 : 0};
        GraphEntry* ge = nullptr;
        if (graphs_enabled()) {
            auto git = ws.graphs.find(gk);
            if (git == ws.graphs.end()) {
                if (ws.graphs.size() >= kMaxGraphs) ws.drop_graphs();
                git = ws.graphs.emplace(gk, GraphEntry{}).first;
            }
            ge = &git->second;
        }
        if (!ge || ge->calls++ == 0) {
            run_all();
            return;
        }
        const size_t nI = (size_t)B * (image ? (size_t)nxy * nxy : (size_t)nr), nP = (size_t)B * pstride;
        const size_t nS = (size_t)B * d->nsets;
        float* in_I = ws.in_I.get<float>(nI);
        float* in_p = ws.in_p.get<float>(nP);
        double* o_chi2 = ws.out_chi2.get<double>((size_t)B);
        double* o_sets = chi2_sets ? ws.out_sets.get<double>(nS) : nullptr;
        float* o_gI = grad ? ws.out_gI.get<float>(nI) : nullptr;
        float* o_gp = grad ? ws.out_gp.get<float>(nP) : nullptr;
        float* const user_gI = grad_intensity;
        float* const user_gp = grad_params;
        double* const user_chi2 = chi2;
        double* const user_sets = chi2_sets;
        BCK(cudaMemcpyAsync(in_I, intensity, sizeof(float) * nI, cudaMemcpyDeviceToDevice, s_user));
        BCK(cudaMemcpyAsync(in_p, params, sizeof(float) * nP, cudaMemcpyDeviceToDevice, s_user));
        intensity = in_I;
        params = in_p;
        chi2 = o_chi2;
        chi2_sets = o_sets;
        grad_intensity = o_gI;
        grad_params = o_gp;
        if (!ge->exec || ge->gen != g_buf_gen.load()) {
            if (!ws.cap) BCK(cudaStreamCreateWithFlags(&ws.cap, cudaStreamNonBlocking));
            cudaGraph_t graph = nullptr;
            BCK(cudaStreamBeginCapture(ws.cap, cudaStreamCaptureModeThreadLocal));
            s = ws.cap;
            t_capturing = true;
            try {
                run_all();
            } catch (...) {
                t_capturing = false;
                s = s_user;
                cudaStreamEndCapture(ws.cap, &graph);
                if (graph) cudaGraphDestroy(graph);
                throw;
            }
            t_capturing = false;
            s = s_user;
            BCK(cudaStreamEndCapture(ws.cap, &graph));
            if (ge->exec) cudaGraphExecDestroy(ge->exec);
            ge->exec = nullptr;
            const cudaError_t ie = cudaGraphInstantiate(&ge->exec, graph, 0);
            cudaGraphDestroy(graph);
            BCK(ie);
            ge->gen = g_buf_gen.load();
        }
        BCK(cudaGraphLaunch(ge->exec, s_user));
        BCK(cudaMemcpyAsync(user_chi2, o_chi2, sizeof(double) * B, cudaMemcpyDeviceToDevice, s_user));
        if (user_sets)
            BCK(cudaMemcpyAsync(user_sets, o_sets, sizeof(double) * nS, cudaMemcpyDeviceToDevice, s_user));
        if (grad) {
            BCK(cudaMemcpyAsync(user_gI, o_gI, sizeof(float) * nI, cudaMemcpyDeviceToDevice, s_user));
            BCK(cudaMemcpyAsync(user_gp, o_gp, sizeof(float) * nP, cudaMemcpyDeviceToDevice, s_user));
        }
}

API int galario_chi2_profile_batch_f(void* dataset, int B, int nr, const float* intensity, float Rmin, float dR,
                                     float dxy, int nxy, const float* params, double* chi2, double* chi2_sets,
                                     float* grad_intensity, float* grad_params, void* stream) {
    return bguard([&] {
        BatchCall c;
        c.d = static_cast<Dataset*>(dataset);
        c.B = B;
        c.nr = nr;
        c.input = intensity;
        c.Rmin = Rmin;
        c.dR = dR;
        c.dxy = dxy;
        c.nxy = nxy;
        c.vo = 1.f;  // profiles: origin 'upper' (reference src/galario.cpp:1411)
        c.params = params;
        c.pstride = 4;
        c.chi2 = chi2;
        c.chi2_sets = chi2_sets;
        c.grad_input = grad_intensity;
        c.grad_params = grad_params;
        c.stream = stream;
        batch_run(c);
    });
}

API int galario_chi2_image_batch_f(void* dataset, int B, int nxy, const float* images, float dxy, float v_origin,
                                   const float* params, double* chi2, double* chi2_sets, float* grad_images,
                                   float* grad_params, void* stream) {
    return bguard([&] {
        if (!(v_origin == 1.f || v_origin == -1.f))
            throw Err{GALARIO_EINVAL, "Error in batch: v_origin must be +1 ('upper') or -1 ('lower')"};
        BatchCall c;
        c.d = static_cast<Dataset*>(dataset);
        c.B = B;
        c.image = true;
        c.input = images;
        c.dxy = dxy;
        c.nxy = nxy;
        c.vo = v_origin;
        c.params = params;
        c.pstride = 3;
        c.chi2 = chi2;
        c.chi2_sets = chi2_sets;
        c.grad_input = grad_images;
        c.grad_params = grad_params;
        c.stream = stream;
        batch_run(c);
    });
}
