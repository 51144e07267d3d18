// Spectrum window of a swept FP64 profile on the tensor cores.
//
// A swept image is even in x and y about pixel (N/2, N/2).  With F[a][c] its
// quadrant (a = |y|, c = |x| in pixels, a, c < nF), w_0 = w_{N/2} = 1 and
// w_j = 2 otherwise (the number of mirror pixels), the reference's shifted
// spectrum fftshift_axis0(rfft2(fftshift(image))) (src/galario.cpp:595-612,
// :495-506, :674-688) is real and
//
//     S[r][k] = sum_a C[|r - N/2|][a] sum_c C[k][c] F[a][c],
//     C[j][c] = w_c cos(2 pi c j / N),
//
// two products with one fixed cosine matrix: D1 = C[0:K] F^T (K x nF), then
// S' = D1 C[0:T+1]^T (K x (T + 1)), T = max |r - N/2| over the window rows, and
// window row r takes S'[.][|r - N/2|].  Both run transposed (D1^T = F C^T,
// S'^T = C D1^T), so that the row of D1 that the next pass splits, and the
// column of S' that becomes a window column, are contiguous in the products'
// output (whose fastest index is the row of the first factor).  Both are
// FP64-grade products on the bf16 tensor cores (gb_ozaki.cuh): each operand
// row as eight balanced base-128 digits relative to the row's exponent, the
// 36 digit-pair products with i + j <= 7 summed exactly in integer levels
// and folded into one 64-bit integer sum per element.
//
// Passes (no host round trip; K, r0, W come from the device window written
// by the extent pass, which runs on a side stream beside the fold; the
// passes after the first product are programmatic dependent launches):
//   oz_fold_kernel       the quadrant of the sweep (reference sweep_core
//                        :1048-1071, central pixel :1136-1153), one row per
//                        block, its row exponent and digits
//   ozaki_levels_kernel  D1^T = F C[0:K]^T as integer sums
//   oz_mid_kernel        D1 from its sums (which it clears), one row per
//                        block, its row exponent and digits
//   ozaki_levels_kernel  S'^T = C[0:T+1] D1^T as integer sums
//   oz_out_kernel        S' from its sums (which it clears) -> window rows
//                        N/2 - t and N/2 + t and their moduli (the cell
//                        records are built from the window afterwards)
// The sum buffers are zero between calls: allocated zeroed, and every entry
// the level kernel adds to is read and cleared by the pass after it.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <cmath>
#include <cstdlib>
#include <vector>

#include "gb_device.cuh"
#include "gb_internal.cuh"
#include "gb_ozaki.cuh"

namespace gbg {

namespace {

constexpr int kFoldThreads = 256;
constexpr int kPerThread = 8;                 // values of a row per thread: rows of up to 2048
constexpr int kMaxRow = kFoldThreads * kPerThread;
constexpr int kBadRow = -0x7fffffff;          // row exponent of a row with a NaN or infinite value

__device__ __forceinline__ double block_max(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double m = red[0];
#pragma unroll
    for (int w = 1; w < kFoldThreads / 32; ++w) m = fmax(m, red[w]);
    __syncthreads();
    return m;
}

// digits of a row: v[i] at column threadIdx.x + kFoldThreads i (< n), relative to exponent e
__device__ __forceinline__ void write_digits(const double* v, int n, int e, unsigned short* __restrict__ dst,
                                             long long plane) {
#pragma unroll
    for (int i = 0; i < kPerThread; ++i) {
        const int c = threadIdx.x + kFoldThreads * i;
        if (c >= n) break;
        int d[oz::kPlanes];
        oz::digits8(v[i], e, d);
#pragma unroll
        for (int s = 0; s < oz::kPlanes; ++s) dst[(long long)s * plane + c] = oz::bf16_of_int(d[s]);
    }
}

// sum_L 2^(-7 L) lev_L of one product element from its integer sum (see
// ozaki_levels_kernel), clearing it for the next call
__device__ __forceinline__ double take_sum(long long* __restrict__ p) {
    const long long v = *p;
    *p = 0;
    return oz::combine_levels(v);
}

// x 2^n from exponent-field arithmetic (exact while the result is a normal number)
__device__ __forceinline__ double pow2i(int n) { return __longlong_as_double((long long)(n + 1023) << 52); }
__device__ __forceinline__ double scale2(double x, int n) {
    if (n >= -1022 && n <= 1023) return x * pow2i(n);
    const int h = n / 2;
    return (x * pow2i(h)) * pow2i(n - h);
}

// Block a: quadrant row a (image row N/2 - a), columns c < nF (image column
// N/2 - c), the central pixel at (0, 0).  F row a as digits, plane stride
// nF * ldF, row stride ldF.
__global__ void __launch_bounds__(kFoldThreads) oz_fold_kernel(const double* __restrict__ intensity, int nr,
                                                               double Rmin, double dR, double inv_dR, double dxy,
                                                               double inv_cos_inc, int rmax, double central, int N,
                                                               int nF, int ldF, unsigned short* __restrict__ fd,
                                                               int* __restrict__ ef) {
    __shared__ double red[kFoldThreads / 32];
    const int a = blockIdx.x;
    const int n = N / 2, off = N / 2 - rmax;
    const double sr_to_px = dxy * dxy;
    double v[kPerThread];
    double mx = 0.0;
#pragma unroll
    for (int i = 0; i < kPerThread; ++i) {
        const int c = threadIdx.x + kFoldThreads * i;
        v[i] = 0.0;
        if (c < nF) {
            v[i] = (a == 0 && c == 0) ? central
                                      : sweep_pixel<double>(n - a, n - c, intensity, nr, Rmin, dR, inv_dR, dxy,
                                                            inv_cos_inc, rmax, off, sr_to_px);
            const double m = fabs(v[i]);
            mx = (m > mx || m != m) ? m : mx;  // NaN propagates
        }
    }
    mx = block_max(isfinite(mx) ? mx : INFINITY, red);
    const bool bad = !isfinite(mx);
    const int e = bad ? kBadRow : oz::row_exponent(mx);
    if (threadIdx.x == 0) ef[a] = e;
    if (!bad) write_digits(v, nF, e, fd + (long long)a * ldF, (long long)nF * ldF);
}

// Rows k of D1 from the sums of D1^T (which it clears; D1[k][a] at column k,
// row a, so a row of D1 is contiguous), as digits of a row-major K x nF
// operand (plane stride planeD, row stride ldF).
__global__ void __launch_bounds__(kFoldThreads) oz_mid_kernel(oz::Params p, const int* __restrict__ ec,
                                                              const int* __restrict__ ef, int nF, int ldF,
                                                              long long planeD, unsigned short* __restrict__ dd,
                                                              int* __restrict__ ed) {
    __shared__ double red[kFoldThreads / 32];
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");  // the second product may set up
    asm volatile("griddepcontrol.wait;" ::: "memory");  // programmatic dependent of the first product
    const oz::Dims dm = oz::item_dims(p);  // M = nF rows (a), N = K columns (k)
    for (int k = blockIdx.x; k < dm.N; k += gridDim.x) {
        const int eck = ec[k];
        double v[kPerThread];
        double mx = 0.0;
#pragma unroll
        for (int i = 0; i < kPerThread; ++i) {
            const int a = threadIdx.x + kFoldThreads * i;
            v[i] = 0.0;
            if (a < nF) {
                const double acc = take_sum(p.P + (long long)k * dm.ldm + a);
                const int ea = ef[a];
                v[i] = (ea == kBadRow || eck == kBadRow) ? (double)NAN : scale2(acc, eck + ea - 12);
                const double m = fabs(v[i]);
                mx = (m > mx || m != m) ? m : mx;
            }
        }
        mx = block_max(isfinite(mx) ? mx : INFINITY, red);
        const bool bad = !isfinite(mx);
        const int e = bad ? kBadRow : oz::row_exponent(mx);
        if (threadIdx.x == 0) ed[k] = e;
        if (!bad) write_digits(v, nF, e, dd + (long long)k * ldF, planeD);
    }
}

// S'[k][t] from the sums of S'^T (which it clears; consecutive threads take
// consecutive t), written to window rows N/2 -+ t of column k: the spectrum
// value and its modulus.
__global__ void __launch_bounds__(256) oz_out_kernel(oz::Params p, const int* __restrict__ ed,
                                                     const int* __restrict__ ec, int N,
                                                     const DevState* __restrict__ st, C2<double>* __restrict__ out,
                                                     double* __restrict__ amp, long long s_row, long long s_col) {
    asm volatile("griddepcontrol.wait;" ::: "memory");  // programmatic dependent of the product
    const oz::Dims dm = oz::item_dims(p);  // M = T + 1 rows (t), N = K columns (k)
    const Window w = get_window(-1, -1, -1, st);
    const long long total = (long long)dm.N * dm.ldm;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e / dm.ldm), t = (int)(e - (long long)k * dm.ldm);
        if (t >= dm.M) continue;
        const double acc = take_sum(p.P + e);
        const int ek = ed[k];
        const double f = ek == kBadRow ? (double)NAN : scale2(acc, ek + ec[t] - 12);
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            if (side == 1 && t == 0) break;
            const int q = (side ? N / 2 + t : N / 2 - t) - w.r0;
            if (q < 0 || q >= w.W) continue;
            const long long o = (long long)q * s_row + (long long)k * s_col;
            out[o] = C2<double>{f, 0.0};
            amp[o] = fabs(f);
        }
    }
}

// grow-only device buffer; `zero` clears a fresh allocation
struct Buf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t get(size_t bytes, bool zero, bool* fresh) {
        *fresh = false;
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) return e;
        if (zero) {
            e = cudaMemset(p, 0, bytes);
            if (e != cudaSuccess) return e;
        }
        cap = bytes;
        *fresh = true;
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

// Launch as a programmatic dependent of the stream's previous kernel: its
// CTAs may start (and run up to griddepcontrol.wait) while that kernel's last
// CTAs finish, which hides the gap between the short passes of the chain.
template <typename... KArgs, typename... Args>
cudaError_t launch_dependent(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t s,
                             Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

}  // namespace

struct ProfileTc {
    int N = 0, nF = 0, ldF = 0;  // geometry of the cosine digits and of the operands
    Buf cd, ec, fd, ef, dd, ed, p1, p2;
    CUtensorMap map_ca{}, map_cb{}, map_f{}, map_d{};  // C as A / B, F as A, D1 as B
    bool maps = false;
    bool smem_attr = false;  // the level kernel's shared-memory limit raised (per device, as this state)
};

ProfileTc* profile_tc_new() { return new ProfileTc(); }
void profile_tc_free(ProfileTc* t) {
    if (!t) return;
    Buf* bufs[] = {&t->cd, &t->ec, &t->fd, &t->ef, &t->dd, &t->ed, &t->p1, &t->p2};
    for (Buf* b : bufs) b->release();
    delete t;
}

int profile_tc_quadrant(int N, int rmax) {
    const int n = N / 2;
    return rmax >= n ? n + 1 : rmax;
}

bool profile_tc_ok(int N, int rmax) {
    const char* v = std::getenv("GALARIO_TC");
    if (v && v[0] == '0') return false;
    const int nF = profile_tc_quadrant(N, rmax);
    return N >= 16 && N % 2 == 0 && N <= 16384 && nF >= 1 && nF <= kMaxRow && nF <= oz::kMaxK &&
           tc::encode_fn() != nullptr;
}

// the digits of C[j][c] = w_c cos(2 pi c j / N), j <= N/2, c < nF (cosines
// from long double, rounded once to double)
static cudaError_t build_cosines(ProfileTc* t, int N, int nF, int ldF) {
    const int C = N / 2 + 1;
    const long double two_pi = 6.283185307179586476925286766559005768L;
    std::vector<double> cosv((size_t)N);
    for (int m = 0; m < N; ++m) cosv[(size_t)m] = (double)cosl(two_pi * (long double)m / (long double)N);
    const long long plane = (long long)C * ldF;
    std::vector<unsigned short> h((size_t)(oz::kPlanes * plane), 0);
    std::vector<int> ex((size_t)C);
    std::vector<double> row((size_t)nF);
    for (int j = 0; j < C; ++j) {
        double mx = 0.0;
        for (int c = 0; c < nF; ++c) {
            const double wc = (c == 0 || c == N / 2) ? 1.0 : 2.0;
            row[(size_t)c] = wc * cosv[(size_t)(((long long)c * j) % N)];
            mx = std::max(mx, std::fabs(row[(size_t)c]));
        }
        const int e = oz::row_exponent(mx);
        ex[(size_t)j] = e;
        for (int c = 0; c < nF; ++c) {
            int d[oz::kPlanes];
            oz::digits8(row[(size_t)c], e, d);
            for (int s = 0; s < oz::kPlanes; ++s) h[(size_t)(s * plane + (long long)j * ldF + c)] = oz::bf16_of_int(d[s]);
        }
    }
    bool fresh = false;
    cudaError_t e = t->cd.get(h.size() * sizeof(unsigned short), false, &fresh);
    if (e == cudaSuccess) e = t->ec.get(ex.size() * sizeof(int), false, &fresh);
    if (e == cudaSuccess) e = cudaMemcpy(t->cd.p, h.data(), h.size() * sizeof(unsigned short), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->ec.p, ex.data(), ex.size() * sizeof(int), cudaMemcpyHostToDevice);
    return e;
}

// buffers, cosine digits and tensor maps for (N, nF)
static cudaError_t prepare(ProfileTc* t, int N, int nF) {
    const int C = N / 2 + 1, ldF = round_up(nF, 8);
    cudaError_t e = cudaSuccess;
    bool moved = false, fresh = false;
    if (t->N != N || t->nF != nF) {
        e = build_cosines(t, N, nF, ldF);
        if (e != cudaSuccess) {
            t->N = t->nF = 0;
            return e;
        }
        t->N = N;
        t->nF = nF;
        t->ldF = ldF;
        moved = true;
    }
    const long long planeF = (long long)nF * ldF, planeD = (long long)C * ldF;
    const int ldmF = round_up(nF, 32), ldmC = round_up(C, 32);  // rows of the products' sums
    e = t->fd.get(sizeof(unsigned short) * oz::kPlanes * planeF, false, &fresh);
    moved |= fresh;
    if (e == cudaSuccess) e = t->ef.get(sizeof(int) * nF, false, &fresh);
    if (e == cudaSuccess) e = t->dd.get(sizeof(unsigned short) * oz::kPlanes * planeD, true, &fresh);
    moved |= fresh;
    if (e == cudaSuccess) e = t->ed.get(sizeof(int) * C, false, &fresh);
    if (e == cudaSuccess) e = t->p1.get(sizeof(long long) * (size_t)ldmF * C, true, &fresh);
    if (e == cudaSuccess) e = t->p2.get(sizeof(long long) * (size_t)ldmC * C, true, &fresh);
    if (e != cudaSuccess) return e;
    if (moved || !t->maps) {
        t->maps = oz::make_map(&t->map_ca, t->cd.p, nF, C, ldF, planeD, oz::BM) &&
                  oz::make_map(&t->map_cb, t->cd.p, nF, C, ldF, planeD, oz::BN) &&
                  oz::make_map(&t->map_f, t->fd.p, nF, nF, ldF, planeF, oz::BM) &&
                  oz::make_map(&t->map_d, t->dd.p, nF, C, ldF, planeD, oz::BN);
        if (!t->maps) return cudaErrorInvalidValue;
    }
    return cudaSuccess;
}

cudaError_t profile_tc_fold(ProfileTc* t, const double* intensity, int nr, double Rmin, double dR, double dxy,
                            double cos_inc, int rmax, double central, int N, cudaStream_t s) {
    const int nF = profile_tc_quadrant(N, rmax);
    cudaError_t e = prepare(t, N, nF);
    if (e != cudaSuccess) return e;
    oz_fold_kernel<<<nF, kFoldThreads, 0, s>>>(intensity, nr, Rmin, dR, 1.0 / dR, dxy, 1.0 / cos_inc, rmax, central, N,
                                               nF, t->ldF, static_cast<unsigned short*>(t->fd.p),
                                               static_cast<int*>(t->ef.p));
    return cudaGetLastError();
}

cudaError_t profile_tc_window(ProfileTc* t, int N, DevState* st, C2<double>* out, double* amp, long long s_row,
                              long long s_col, cudaStream_t s) {
    if (!t->maps || t->N != N) return cudaErrorInvalidValue;  // profile_tc_fold prepares the geometry
    const int C = N / 2 + 1, nF = t->nF, ldF = t->ldF;
    if (!t->smem_attr) {
        const cudaError_t e = cudaFuncSetAttribute(oz::ozaki_levels_kernel,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, oz::kSmem);
        if (e != cudaSuccess) return e;
        t->smem_attr = true;
    }
    const int grid = num_sms();
    // a launch that fails after the first product has added to the sums
    // leaves them for the next call: clear both buffers before reporting it
    auto failed = [&](cudaError_t err) {
        (void)cudaMemsetAsync(t->p1.p, 0, t->p1.cap, s);
        (void)cudaMemsetAsync(t->p2.p, 0, t->p2.cap, s);
        return err;
    };
    // D1^T = F C[0:K]^T: rows a < nF, columns k < K (the window)
    oz::Params p1{};
    p1.m_max = nF;
    p1.n_max = C;
    p1.K = nF;
    p1.n_dev = &st->win_K;
    p1.half = N / 2;
    p1.P = static_cast<long long*>(t->p1.p);
    p1.err = &st->err;
    // an ordinary launch: the stream's previous operations include the join
    // with the extent pass, whose window this product reads
    oz::ozaki_levels_kernel<<<grid, oz::kThreads, oz::kSmem, s>>>(t->map_f, t->map_cb, p1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = launch_dependent(oz_mid_kernel, 2 * grid, kFoldThreads, 0, s, p1, static_cast<const int*>(t->ec.p),
                         static_cast<const int*>(t->ef.p), nF, ldF, (long long)C * ldF,
                         static_cast<unsigned short*>(t->dd.p), static_cast<int*>(t->ed.p));
    if (e != cudaSuccess) return failed(e);
    // S'^T = C[0:T+1] D1^T: rows t <= T (the window rows' distances), columns k < K
    oz::Params p2{};
    p2.m_max = C;
    p2.n_max = C;
    p2.K = nF;
    p2.n_dev = &st->win_K;
    p2.win_r0 = &st->win_r0;
    p2.win_W = &st->win_W;
    p2.win_rows = 1;
    p2.half = N / 2;
    p2.P = static_cast<long long*>(t->p2.p);
    p2.err = &st->err;
    e = launch_dependent(oz::ozaki_levels_kernel, grid, oz::kThreads, (size_t)oz::kSmem, s, t->map_ca, t->map_d, p2);
    if (e != cudaSuccess) return failed(e);
    e = launch_dependent(oz_out_kernel, 2 * grid, 256, 0, s, p2, static_cast<const int*>(t->ed.p),
                         static_cast<const int*>(t->ec.p), N, static_cast<const DevState*>(st), out, amp, s_row,
                         s_col);
    if (e != cudaSuccess) return failed(e);
    return cudaGetLastError();
}

}  // namespace gbg
