// FP64-grade products on the bf16 tensor cores (the Ozaki splitting scheme:
// K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59, 2012).
//
// Each FP64 row x of an operand is written relative to a row exponent e
// (|x_k| < 2^e) as eight balanced base-128 digits,
//
//     x_k = 2^e sum_{i<8} d_i[k] 2^(-6-7i),   d_i integers, |d_i| <= 64,
//
// exact to 2^(e-55) (the digits of 55 bits of x below 2^e, rounded once).
// Digit planes are bf16 arrays (integers up to 64 in magnitude are exact in
// bf16).  The product of two rows is then
//
//     sum_k a_k b_k = 2^(e_a + e_b - 12) sum_{L} 2^(-7L) lev_L,
//     lev_L = sum_{i + j = L} sum_k d^a_i[k] d^b_j[k],
//
// and levels L <= 7 (36 digit pairs) keep it to about 2^-53 of
// K max|a| max|b|.  Every lev_L is a sum of integer products of at most
// 64 x 64: over one K tile of 64 values, at most 8 x 64 x 4096 = 2^21 in
// magnitude, so the tensor core's FP32 accumulation adds integers that are
// all exactly representable and the level sums are exact; the partial sums
// of the K tiles stay exact in FP32 while (L + 1) K 4096 < 2^24, i.e. for
// K <= 511.
//
// ozaki_levels_kernel: C = A B^T in levels, A (M x K) and B (N x K) given as
// digit planes, K-major bf16 (plane stride a multiple of the row stride).
// One work item = one 128 x 64 output tile and one K tile of 64: TMA loads
// the eight A planes (128 x 64) and eight B planes (64 x 64) into shared
// memory (128-byte swizzle), one thread issues the 36 digit-pair products
// (4 K steps of tcgen05.mma kind::f16, M = 128, N = 64, K = 16 each) into
// eight FP32 accumulators in tensor memory (8 x 64 = 512 columns), and four
// epilogue warps add the eight level tiles of the item into the level buffer
// P[L][m][n] with vector reductions (red.global.add.v4.f32): the values are
// integers and every partial and total sum stays below 2^24, so the adds are
// exact and their order does not matter.  P must be zero before the call;
// the kernel that reads it clears it.  The grid is persistent (items
// round-robin over the CTAs): the tile counts come from device-side sizes
// (the spectrum window).
// Every wait is bounded; a wait that runs out sets the error bit, each role
// stops, the CTA waits (bounded) for what it issued, frees its tensor memory
// and returns.  Single-GPU code: no multicast.
#pragma once

#include <cstring>

#include "gb_tc.cuh"

namespace gbg {
namespace oz {

constexpr int kPlanes = 8;       // digits per value
constexpr int kLevels = 8;       // levels L = i + j <= 7
constexpr int BM = 128;
constexpr int BN = 64;
constexpr int BK = 64;           // bf16 values per K tile: one 128-byte swizzle row
constexpr int kThreads = 192;    // producer warp, MMA warp, four epilogue warps
constexpr int kMaxK = 511;       // exact FP32 sums of the K tiles
constexpr int kABytes = BM * BK * 2;  // one A plane tile
constexpr int kBBytes = BN * BK * 2;  // one B plane tile
constexpr int kSmem = 1024 + kPlanes * (kABytes + kBBytes) + 256;
constexpr int kTmemCols = kLevels * BN;  // 512

// Sizes of one product.  M and N may come from the device (the spectrum
// window): rows = min(*m_dev, m_max) when m_dev is set; with win_r0/win_W
// the column count is 1 + the largest |r - N/2| over the window rows.  The
// level buffer is compact for those sizes: P[(L * Mp + m) * ldp + n] with
// Mp = M rounded up to 128 and ldp = N rounded up to 4 (Dims below).
struct Params {
    int m_max, n_max, K;
    const int* m_dev;            // window K (rows of the first factor), or null
    const int* win_r0;           // window r0 and W (columns from the window), or null
    const int* win_W;
    int half;                    // N/2 of the image
    float* P;                    // level buffer (zero on entry)
    unsigned* err;
};
struct Dims {
    int M, N, Mp, ldp;
};

__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    // D F32 (bits 4-5 = 1), A and B bf16 (bits 7-9, 10-12 = 1), K-major, N >> 3 at 17, M >> 4 at 24
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__host__ __device__ inline Dims dims_of(int m, int n) {
    Dims d;
    d.M = m > 0 ? m : 0;
    d.N = n > 0 ? n : 0;
    d.Mp = (d.M + BM - 1) / BM * BM;
    d.ldp = (d.N + 3) / 4 * 4;
    return d;
}
__device__ __forceinline__ Dims item_dims(const Params& p) {
    int m = p.m_max, n = p.n_max;
    if (p.m_dev) m = min(m, *((volatile const int*)p.m_dev));
    if (p.win_r0) {
        const int r0 = *((volatile const int*)p.win_r0), W = *((volatile const int*)p.win_W);
        n = min(n, max(p.half - r0, r0 + W - 1 - p.half) + 1);
    }
    return dims_of(m, n);
}
__device__ __forceinline__ void red_add_v4(float* dst, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst), "f"(__uint_as_float(a)),
                 "f"(__uint_as_float(b)), "f"(__uint_as_float(c)), "f"(__uint_as_float(d))
                 : "memory");
}

__global__ void __launch_bounds__(kThreads, 1)
    ozaki_levels_kernel(const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap bmap, Params p) {
    using namespace gbg::tc;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                           ~uintptr_t(1023));
    unsigned char* a_tiles = base;                                  // kPlanes x kABytes
    unsigned char* b_tiles = base + kPlanes * kABytes;              // kPlanes x kBBytes
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + kPlanes * (kABytes + kBBytes));
    uint64_t* full = bars;                 // [kPlanes] plane i of A and B landed
    uint64_t* empty = bars + kPlanes;      // every MMA of the item has read shared memory
    uint64_t* accf = bars + kPlanes + 1;   // the item's levels are in tensor memory
    uint64_t* acce = bars + kPlanes + 2;   // the epilogue has read them (128 arrivals)
    uint64_t* done = bars + kPlanes + 3;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + kPlanes + 4);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const Dims dm = item_dims(p);
    const int mt_n = dm.Mp / BM, nt_n = (dm.N + BN - 1) / BN, kt_n = (p.K + BK - 1) / BK;
    const int items = mt_n * nt_n * kt_n;
    if ((int)blockIdx.x >= items) return;  // uniform: nothing allocated yet

    if (threadIdx.x == 0) {
        for (int s = 0; s < kPlanes; ++s) mbar_init(&full[s], 1);
        mbar_init(empty, 1);
        mbar_init(accf, 1);
        mbar_init(acce, 128);
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"((uint32_t)kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    auto fail = [&]() {
        atomicOr(p.err, kErrSpin);
        *abort_flag = 1;
    };
    // item t of this CTA (the t-th it processes): barrier phase t & 1
    auto decode = [&](int item, int* m0, int* n0, int* kt) {
        *kt = item % kt_n;
        const int r = item / kt_n;
        *n0 = (r % nt_n) * BN;
        *m0 = (r / nt_n) * BM;
    };

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer ----
            int t = 0, issued = 0;
            for (int item = blockIdx.x; item < items && !*abort_flag; item += gridDim.x, ++t) {
                int m0, n0, kt;
                decode(item, &m0, &n0, &kt);
                // shared memory is free once the previous item's MMAs have read it
                if (t > 0 && !mbar_wait(empty, (uint32_t)((t - 1) & 1))) {
                    fail();
                    break;
                }
                for (int s = 0; s < kPlanes; ++s) {
                    mbar_expect_tx(&full[s], (uint32_t)(kABytes + kBBytes));
                    tma_load_3d(a_tiles + s * kABytes, &amap, kt * BK, m0, s, &full[s]);
                    tma_load_3d(b_tiles + s * kBBytes, &bmap, kt * BK, n0, s, &full[s]);
                }
                issued = t + 1;
            }
            // at an abort, wait (bounded) until the copies in flight have landed
            if (*abort_flag && issued > 0)
                for (int s = 0; s < kPlanes; ++s) (void)mbar_wait(&full[s], (uint32_t)((issued - 1) & 1));
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer: planes in arrival order; pair (i, j) once both have landed ----
            constexpr uint32_t idesc = idesc_bf16(BM, BN);
            int t = 0;
            for (int item = blockIdx.x; item < items && !*abort_flag; item += gridDim.x, ++t) {
                // the levels of the previous item must have been read out
                if (t > 0 && !mbar_wait(acce, (uint32_t)((t - 1) & 1))) {
                    fail();
                    break;
                }
                unsigned started = 0u;  // levels whose accumulator has been written
                bool ok = true;
                for (int s = 0; s < kPlanes && ok; ++s) {
                    if (!mbar_wait(&full[s], (uint32_t)(t & 1))) {
                        fail();
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    // pairs with max(i, j) = s and i + j <= 7
                    for (int o = 0; o <= s; ++o) {
                        for (int side = 0; side < (o == s ? 1 : 2); ++side) {
                            const int i = side == 0 ? s : o, j = side == 0 ? o : s;
                            const int L = i + j;
                            if (L >= kLevels) continue;
                            const uint32_t acc = tmem + (uint32_t)(L * BN);
                            const uint32_t ab = smem_addr(a_tiles + i * kABytes), bb = smem_addr(b_tiles + j * kBBytes);
#pragma unroll
                            for (int kk = 0; kk < BK / 16; ++kk) {
                                const uint32_t off = kk * 32;  // 16 bf16 = 32 bytes along the swizzled row
                                const uint32_t accumulate = ((started >> L) & 1u) || kk > 0 ? 1u : 0u;
                                mma_bf16(acc, sdesc(ab + off), sdesc(bb + off), idesc, accumulate);
                            }
                            started |= 1u << L;
                        }
                    }
                }
                if (!ok) break;
                mma_commit(empty);  // shared memory free once these MMAs have read it
                mma_commit(accf);   // the levels are complete
            }
            mma_commit(done);
            if (!mbar_wait(done, 0u)) fail();  // every MMA complete before the tensor memory is freed
        }
    } else {
        // ---- epilogue: lane = tile row; 8 levels x 64 columns per item ----
        const int quarter = warp & 3;
        const uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
        int t = 0;
        for (int item = blockIdx.x; item < items; item += gridDim.x, ++t) {
            int m0, n0, kt;
            decode(item, &m0, &n0, &kt);
            if (*abort_flag || !mbar_wait(accf, (uint32_t)(t & 1))) {
                if (!*abort_flag) fail();
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int row = m0 + quarter * 32 + lane;  // < Mp
            (void)kt;
            for (int L = 0; L < kLevels; ++L) {
                uint32_t x[32], y[32];
                tmem_ld32_async(tmem + lane_off + (uint32_t)(L * BN), x);
                tmem_ld32_async(tmem + lane_off + (uint32_t)(L * BN + 32), y);
                tmem_wait32(x);
                tmem_wait32(y);
                float* dst = p.P + ((size_t)L * dm.Mp + row) * dm.ldp + n0;
                // ldp is a multiple of 4 and n0 of 64: 16-byte reductions inside the row
#pragma unroll
                for (int c = 0; c < 32; c += 4) {
                    if (n0 + c < dm.ldp) red_add_v4(dst + c, x[c], x[c + 1], x[c + 2], x[c + 3]);
                    if (n0 + 32 + c < dm.ldp) red_add_v4(dst + 32 + c, y[c], y[c + 1], y[c + 2], y[c + 3]);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(acce);
        }
    }
    __syncwarp();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)kTmemCols)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------
// digits
// ---------------------------------------------------------------------------
// Row exponent: the smallest e with |x| < 2^e for the row's largest |x|
// (0 for a zero row).
__host__ __device__ inline int row_exponent(double amax) {
    if (!(amax > 0.0)) return 0;
    unsigned long long b;
    memcpy(&b, &amax, 8);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0) return -1022;  // subnormal: below 2^-1022
    return ex - 1023 + 1;
}

// The eight balanced base-128 digits of x relative to 2^e (|x| < 2^e):
// x = 2^e sum_i d[i] 2^(-6-7i) + r, |r| <= 2^(e-56), |d[i]| <= 64.  Integer
// operations on the bit pattern: X = round(|x| 2^(55-e)) < 2^55, then the
// digits of X from the lowest, each taken in [-64, 63] with a carry.
__host__ __device__ inline void digits8(double x, int e, int d[kPlanes]) {
    unsigned long long b;
    memcpy(&b, &x, 8);
    const bool neg = (b >> 63) != 0;
    const int ex = (int)((b >> 52) & 0x7ff);
    unsigned long long m = b & 0xfffffffffffffULL;
    int exu;  // x = m 2^(exu - 52)
    if (ex == 0) {
        exu = -1022;
    } else {
        m |= 1ULL << 52;
        exu = ex - 1023;
    }
    // X = m 2^(exu - 52 + 55 - e) = m 2^(sh)
    const int sh = exu + 3 - e;
    unsigned long long X;
    if (m == 0) {
        X = 0;
    } else if (sh >= 0) {
        X = sh > 2 ? 0ULL : (m << sh);  // |x| < 2^e bounds sh by 2; larger means a bad exponent
    } else if (sh > -64) {
        const int r = -sh;
        X = (m >> r) + ((m >> (r - 1)) & 1ULL);  // round half up on the magnitude
    } else {
        X = 0;
    }
    long long v = (long long)X;
    for (int i = kPlanes - 1; i > 0; --i) {
        long long q = v & 127;
        if (q >= 64) q -= 128;
        d[i] = (int)q;
        v = (v - q) >> 7;
    }
    d[0] = (int)v;
    if (neg)
        for (int i = 0; i < kPlanes; ++i) d[i] = -d[i];
}

// bf16 bit pattern of a small integer (|v| <= 256: exact)
__host__ __device__ inline unsigned short bf16_of_int(int v) {
    const float f = (float)v;
    unsigned int u;
    memcpy(&u, &f, 4);
    return (unsigned short)(u >> 16);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// tensor map of a digit-plane array: dims (K, rows, planes), plane stride
// `plane` and row stride `ld` in elements (ld a multiple of 8), box (64, box_rows, 1)
inline bool make_map(CUtensorMap* m, const void* ptr, int K, int rows, int ld, long long plane, int box_rows) {
    auto enc = gbg::tc::encode_fn();
    if (!enc) return false;
    cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)kPlanes};
    cuuint64_t strides[2] = {(cuuint64_t)ld * 2, (cuuint64_t)plane * 2};
    cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(ptr), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace oz
}  // namespace gbg
