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
// all exactly representable and the level sums of a K tile are exact.
//
// ozaki_levels_kernel: C = A B^T, A (M x K) and B (N x K) given as digit
// planes, K-major bf16 (plane stride a multiple of the row stride).  One work
// item = one 128 x 64 output tile and one K tile of 64: TMA loads the eight A
// planes (128 x 64) and eight B planes (64 x 64) into shared memory (128-byte
// swizzle), one thread issues the 36 digit-pair products (4 K steps of
// tcgen05.mma kind::f16, M = 128, N = 64, K = 16 each; fully unrolled, the
// shared-memory descriptors computed once) into eight FP32 accumulators in
// tensor memory (8 x 64 = 512 columns).  Eight epilogue warps (two per lane
// quarter, 32 columns each) read the eight levels of each element and fold
// them into one integer in units of 2^-35,
//
//     V = sum_{L<=5} 2^(7 (5 - L)) lev_L + round((2^7 lev_6 + lev_7) / 2^14),
//
// (the last two levels rounded to that unit, half up: at most 2^-36 of
// 2^(7*5) per K tile, below 2^-52 of K max|a| max|b| in the product) and add
// it into the output P with a 64-bit integer reduction (red.global.add.u64):
// integer sums, exact and independent of the order of the K tiles, below
// 2^62 for up to 32 K tiles.  Layout P[n * ldm + m], m fastest: the 32 lanes
// of a warp hold 32 consecutive rows, so every reduction instruction covers
// 256 contiguous bytes.  Only m < M, n < N are written; P must be zero there
// on entry, and the kernel that reads it clears it.  The grid is persistent
// (items round-robin over the CTAs): the tile counts come from device-side
// sizes (the spectrum window).
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
constexpr int kEpiWarps = 8;     // two per TMEM lane quarter
constexpr int kThreads = 64 + 32 * kEpiWarps;  // producer warp, MMA warp, epilogue warps
constexpr int kMaxK = 32 * BK;   // K tiles whose integer sums stay below 2^62
constexpr int kABytes = BM * BK * 2;  // one A plane tile
constexpr int kBBytes = BN * BK * 2;  // one B plane tile
constexpr int kSmem = 1024 + kPlanes * (kABytes + kBBytes) + 256;
constexpr int kTmemCols = kLevels * BN;  // 512

// Sizes of one product.  M and N may come from the device (the spectrum
// window): rows = min(*m_dev, m_max) when m_dev is set, columns =
// min(*n_dev, n_max) when n_dev is set; with win_r0/win_W the rows (win_rows)
// or the columns number at most 1 + the largest |r - N/2| over the window
// rows.  The output is compact for those sizes: P[n * ldm + m] with ldm = M
// rounded up to 32 (Dims below).
struct Params {
    int m_max, n_max, K;
    const int* m_dev;            // rows from the device, or null
    const int* n_dev;            // columns from the device, or null
    const int* win_r0;           // window r0 and W, or null
    const int* win_W;
    int win_rows;                // the window bounds the rows (1) or the columns (0)
    int half;                    // N/2 of the image
    long long* P;                // integer sums in units of 2^-35 (zero on entry where m < M, n < N)
    unsigned* err;
};
struct Dims {
    int M, N, Mp, ldm;           // Mp: M rounded up to the 128-row tiles
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
    d.ldm = (d.M + 31) / 32 * 32;
    return d;
}
__device__ __forceinline__ Dims item_dims(const Params& p) {
    int m = p.m_max, n = p.n_max;
    if (p.m_dev) m = min(m, *((volatile const int*)p.m_dev));
    if (p.n_dev) n = min(n, *((volatile const int*)p.n_dev));
    if (p.win_r0) {
        const int r0 = *((volatile const int*)p.win_r0), W = *((volatile const int*)p.win_W);
        const int t1 = max(p.half - r0, r0 + W - 1 - p.half) + 1;
        if (p.win_rows) m = min(m, t1);
        else n = min(n, t1);
    }
    return dims_of(m, n);
}
__device__ __forceinline__ void red_add_u64(long long* dst, long long v) {
    asm volatile("red.global.add.u64 [%0], %1;" ::"l"(dst), "l"(v) : "memory");
}
// 8 consecutive accumulator columns of this thread's TMEM lane (values valid after tmem_wait8)
__device__ __forceinline__ void tmem_ld8_async(uint32_t taddr, uint32_t* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}
// wait for every outstanding tcgen05.ld of this thread; the 64 registers pass
// through the wait so that no use is scheduled before it
__device__ __forceinline__ void tmem_wait64(uint32_t* r) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                   "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                   "+r"(r[29]), "+r"(r[30]), "+r"(r[31]), "+r"(r[32]), "+r"(r[33]), "+r"(r[34]), "+r"(r[35]),
                   "+r"(r[36]), "+r"(r[37]), "+r"(r[38]), "+r"(r[39]), "+r"(r[40]), "+r"(r[41]), "+r"(r[42]),
                   "+r"(r[43]), "+r"(r[44]), "+r"(r[45]), "+r"(r[46]), "+r"(r[47]), "+r"(r[48]), "+r"(r[49]),
                   "+r"(r[50]), "+r"(r[51]), "+r"(r[52]), "+r"(r[53]), "+r"(r[54]), "+r"(r[55]), "+r"(r[56]),
                   "+r"(r[57]), "+r"(r[58]), "+r"(r[59]), "+r"(r[60]), "+r"(r[61]), "+r"(r[62]), "+r"(r[63])
                 :
                 : "memory");
}
// sum_L 2^(-7L) lev_L from the integer sum V (units of 2^-35; one rounding)
__host__ __device__ inline double combine_levels(long long v) { return (double)v * 0x1p-35; }
// V of one element of one K tile from its eight (exact, integer) FP32 levels
__host__ __device__ inline long long level_int(float x) {  // |x| < 2^24, an integer
#ifdef __CUDA_ARCH__
    return (long long)__float2int_rz(x);
#else
    return (long long)x;
#endif
}
__host__ __device__ inline long long fold_levels(const float* lev) {
    long long v = 0;
    for (int L = 0; L < 6; ++L) v = v * 128 + level_int(lev[L]);
    const long long tail = level_int(lev[6]) * 128 + level_int(lev[7]);
    return v + ((tail + 8192) >> 14);
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
    uint64_t* acce = bars + kPlanes + 2;   // the epilogue has read them (one arrival per epilogue thread)
    uint64_t* done = bars + kPlanes + 3;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + kPlanes + 4);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // the next kernel of the stream (launched as a programmatic dependent)
    // may start its set-up now; it reads this kernel's output only after its
    // griddepcontrol.wait, which waits for this grid to complete
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

    if (threadIdx.x == 0) {
        for (int s = 0; s < kPlanes; ++s) mbar_init(&full[s], 1);
        mbar_init(empty, 1);
        mbar_init(accf, 1);
        mbar_init(acce, 32 * kEpiWarps);
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
    // launched as a programmatic dependent of the kernel before it: the set-up
    // above overlaps that kernel's tail; its outputs (the operands, the
    // window sizes) are read only after this wait (a no-op otherwise)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const Dims dm = item_dims(p);
    const int mt_n = dm.Mp / BM, nt_n = (dm.N + BN - 1) / BN, kt_n = (p.K + BK - 1) / BK;
    const int items = mt_n * nt_n * kt_n;  // CTAs past it only free their tensor memory
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
            // ---- MMA issuer: planes in arrival order; pair (i, j) once both
            // have landed.  The order is fixed, so whether a level's
            // accumulator is fresh is a compile-time fact of the unrolled loops.
            constexpr uint32_t idesc = idesc_bf16(BM, BN);
            uint64_t da[kPlanes], db[kPlanes];
#pragma unroll
            for (int i = 0; i < kPlanes; ++i) {
                da[i] = sdesc(smem_addr(a_tiles + i * kABytes));
                db[i] = sdesc(smem_addr(b_tiles + i * kBBytes));
            }
            int t = 0;
            for (int item = blockIdx.x; item < items && !*abort_flag; item += gridDim.x, ++t) {
                // the levels of the previous item must have been read out
                if (t > 0 && !mbar_wait(acce, (uint32_t)((t - 1) & 1))) {
                    fail();
                    break;
                }
                bool ok = true;
                unsigned started = 0u;
#pragma unroll
                for (int s = 0; s < kPlanes; ++s) {
                    if (!ok) break;
                    if (!mbar_wait(&full[s], (uint32_t)(t & 1))) {
                        fail();
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    // pairs with max(i, j) = s and i + j <= 7
#pragma unroll
                    for (int o = 0; o <= s; ++o) {
#pragma unroll
                        for (int side = 0; side < 2; ++side) {
                            if (side == 1 && o == s) continue;
                            const int i = side == 0 ? s : o, j = side == 0 ? o : s;
                            const int L = i + j;
                            if (L >= kLevels) continue;
                            const uint32_t acc = tmem + (uint32_t)(L * BN);
#pragma unroll
                            for (int kk = 0; kk < BK / 16; ++kk) {
                                // a K step of 16 bf16 = 32 bytes along the swizzled row: +2 in the address field
                                const uint32_t accumulate = ((started >> L) & 1u) || kk > 0 ? 1u : 0u;
                                mma_bf16(acc, da[i] + 2 * kk, db[j] + 2 * kk, idesc, accumulate);
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
        // ---- epilogue: lane = tile row; warp w reads TMEM lane quarter w % 4
        // and columns [32 h, 32 h + 32), h = (w - 2) / 4; 8 levels of 8
        // columns at a time, folded into one integer per element
        const int quarter = warp & 3, half = (warp - 2) >> 2;
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
            const int row = m0 + quarter * 32 + lane;
            (void)kt;
            const bool live = row < dm.M;
            long long* out_row = p.P + row;
#pragma unroll 1
            for (int c0 = half * 32; c0 < half * 32 + 32; c0 += 8) {
                uint32_t x[kLevels * 8];
#pragma unroll
                for (int L = 0; L < kLevels; ++L) tmem_ld8_async(tmem + lane_off + (uint32_t)(L * BN + c0), x + 8 * L);
                tmem_wait64(x);
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const int n = n0 + c0 + c;
                    float lev[kLevels];
#pragma unroll
                    for (int L = 0; L < kLevels; ++L) lev[L] = __uint_as_float(x[8 * L + c]);
                    const long long v = fold_levels(lev);
                    if (live && n < dm.N) red_add_u64(out_row + (long long)n * dm.ldm, v);
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
