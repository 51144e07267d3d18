// Tensor-core (tcgen05) batched products for the spectrum passes of the
// batched profile path: C[z] = A[z] B[z]^T with FP32 data, computed as three
// TF32 products of a hi/lo split (A_hi B_hi + A_hi B_lo + A_lo B_hi, the
// "3xTF32" scheme: x = hi + lo with hi = tf32(x), lo = tf32(x - hi), so the
// dropped lo*lo term and the rounding of lo are both ~2^-22 |x y|), FP32
// accumulation in tensor memory.
//
// Operands are K-major (row r of A or B holds its K values contiguously),
// stored as separate hi and lo arrays whose values are already rounded to TF32
// (low 13 mantissa bits zero).  Either operand may be shared by every batch
// entry (batch stride 0).  The tensor maps declare the logical extents, so
// the TMA zero-fills tile parts past M, N or K and no padding has to be
// cleared in memory; rows of every operand must start 16-byte aligned (leading
// dimension a multiple of 4 floats).
//
// One CTA computes one BM x BN tile of one batch entry (grid: M tiles, N
// tiles, batch), with 192 threads in three roles:
//   warp 0       TMA producer (one thread): per K tile of 32 values, the four
//                boxes (A_hi, A_lo: BM x 32; B_hi, B_lo: BN x 32) into a ring
//                of shared-memory stages (128-byte swizzle), completion counted
//                on the stage's "full" mbarrier
//   warp 1       allocates the TMEM columns; one thread issues, per K tile,
//                4 K-steps of tcgen05.mma (M = 128, N = BN, K = 8, kind::tf32):
//                A_hi B_hi into accumulator X, A_hi B_lo + A_lo B_hi into Y,
//                both fresh for every K tile and alternating between two X/Y
//                pairs; tcgen05.commit frees the stage ("empty") and hands the
//                pair to the epilogue ("acc full")
//   warps 2-5    epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows
//                of the tile), adds X + Y of every K tile into FP32 registers,
//                releases the pair ("acc empty") and, after the last tile,
//                writes the row out (plain, or as a TF32 hi/lo pair)
// The tensor core therefore chains at most 4 products into an accumulator
// (its accumulation truncates: a product chained over the whole of K = 343 lost
// about 2^-20 of the sum of |terms|, K tiles of 32 summed in FP32 keep it near
// 2^-23).  TMEM holds 4 BN columns, so BN <= 128.
// Every wait is bounded; a wait that runs out sets ERR_SPIN in the error word,
// every role stops issuing work, the CTA waits (bounded) for what it already
// issued, frees its TMEM and returns.  Single-GPU code: no multicast.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>

namespace gbg {
namespace tc {

constexpr int BM = 128;
constexpr int BK = 32;          // FP32 values per K tile: one 128-byte swizzle row
constexpr int kThreads = 192;   // producer warp, MMA warp, four epilogue warps
constexpr unsigned kErrSpin = 8u;  // the error bit of a wait that ran out (ERR_SPIN of the batched path)

enum Epilogue : int {
    kStore = 0,     // C = A B^T
    kStoreTf32 = 1, // C = hi, C2 = lo of the TF32 split of A B^T
    kStoreMirror = 2  // column t of A B^T to columns h0 - t and h0 + t of C (those in [0, ldc))
};

struct Params {
    int M, N, K;                // logical sizes
    float* C;                   // output (row-major, leading dimension ldc, batch stride c_stride)
    float* C2;                  // lo part for kStoreTf32
    long long c_stride;
    int ldc;                    // columns written per row: [0, ldc) (columns >= N are zeros)
    int mode;
    int a_batched, b_batched;   // 0: the operand is shared by all batch entries
    unsigned* err;              // error word (ERR_SPIN)
    int mirror_h0 = 0;          // kStoreMirror: the column of t = 0
};

template <int BN> struct Cfg {
    static_assert(BN == 64 || BN == 128, "two X/Y accumulator pairs of BN columns fit in TMEM");
    static constexpr int kABytes = BM * BK * 4;                 // one of A_hi / A_lo
    static constexpr int kBBytes = BN * BK * 4;                 // one of B_hi / B_lo
    static constexpr int kStageBytes = 2 * kABytes + 2 * kBBytes;
    static constexpr int kStages = (192 * 1024) / kStageBytes >= 4 ? 4 : (192 * 1024) / kStageBytes;
    static_assert(kStages >= 2, "stage ring");
    static constexpr int kTmemCols = 4 * BN;                     // X0, Y0, X1, Y1
    // dynamic shared memory: 1024-byte alignment slack + stages + barriers
    static constexpr int kSmem = 1024 + kStages * kStageBytes + 256;
};

// ---------------------------------------------------------------------------
// device helpers (inline PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// true once the phase with this parity has completed; false after `limit` polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = 1 << 22) {
    const uint32_t a = smem_addr(bar);
    for (int it = 0; it < limit; ++it) {
        uint32_t done;
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
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
        : "memory");
}

// 1D bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned)
// from global to shared memory, counted on `bar`, which expects the bytes
__device__ __forceinline__ void bulk_load_1d(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    mbar_expect_tx(bar, bytes);
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Shared-memory matrix descriptor of a K-major tile with the 128-byte swizzle:
// rows of 128 bytes, 8-row groups 1024 bytes apart (stride byte offset); the
// leading byte offset is unused by this layout (set to 1); descriptor
// version 1; layout type 2 = 128-byte swizzle.  The tile starts 1024-aligned;
// a K step inside the 128-byte row advances the start address.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}
// Instruction descriptor of kind::tf32: D F32 (bits 4-5 = 1), A and B TF32
// (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bit 17,
// M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// 32 consecutive accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// 32 accumulator columns of this thread's TMEM lane into r, without waiting:
// the values are valid after tmem_wait32(r)
__device__ __forceinline__ void tmem_ld32_async(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}
// wait for every outstanding tcgen05.ld of this thread; r passes through the
// wait so that no use of the loaded values is scheduled before it
__device__ __forceinline__ void tmem_wait32(uint32_t* r) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                   "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                   "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
                 :
                 : "memory");
}

// 16 consecutive accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------
template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    gemm_3xtf32_kernel(const __grid_constant__ CUtensorMap a_hi, const __grid_constant__ CUtensorMap a_lo,
                       const __grid_constant__ CUtensorMap b_hi, const __grid_constant__ CUtensorMap b_lo, Params p) {
    using CF = Cfg<BN>;
    constexpr int S = CF::kStages;
    extern __shared__ unsigned char smem_raw[];
    // 1024-byte aligned base for the swizzled tiles
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                           ~uintptr_t(1023));
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + S * CF::kStageBytes);
    uint64_t* full = bars;            // [S]  TMA -> MMA
    uint64_t* empty = bars + S;       // [S]  MMA -> TMA
    uint64_t* accf = bars + 2 * S;    // [2]  MMA -> epilogue
    uint64_t* acce = bars + 2 * S + 2;  // [2] epilogue -> MMA
    uint64_t* done = bars + 2 * S + 4;  // [1] every MMA complete
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * S + 5);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN, z = blockIdx.z;
    const int za = p.a_batched ? z : 0, zb = p.b_batched ? z : 0;
    const int ktiles = (p.K + BK - 1) / BK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int j = 0; j < 2; ++j) {
            mbar_init(&accf[j], 1);
            mbar_init(&acce[j], 128);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"((uint32_t)CF::kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    auto stage_ptr = [&](int s, int which) -> unsigned char* {  // 0 A_hi, 1 A_lo, 2 B_hi, 3 B_lo
        unsigned char* st = base + s * CF::kStageBytes;
        return which < 2 ? st + which * CF::kABytes : st + 2 * CF::kABytes + (which - 2) * CF::kBBytes;
    };
    auto fail = [&]() {
        atomicOr(p.err, kErrSpin);
        *abort_flag = 1;
    };

    float acc[BN];
#pragma unroll
    for (int i = 0; i < BN; ++i) acc[i] = 0.f;

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer ----
            int loaded = 0;
            for (int kt = 0; kt < ktiles && !*abort_flag; ++kt) {
                const int s = kt % S;
                if (kt >= S && !mbar_wait(&empty[s], (uint32_t)((kt / S - 1) & 1))) {
                    fail();
                    break;
                }
                mbar_expect_tx(&full[s], (uint32_t)CF::kStageBytes);
                const int k0 = kt * BK;
                tma_load_3d(stage_ptr(s, 0), &a_hi, k0, m0, za, &full[s]);
                tma_load_3d(stage_ptr(s, 1), &a_lo, k0, m0, za, &full[s]);
                tma_load_3d(stage_ptr(s, 2), &b_hi, k0, n0, zb, &full[s]);
                tma_load_3d(stage_ptr(s, 3), &b_lo, k0, n0, zb, &full[s]);
                ++loaded;
            }
            // at an abort, wait (bounded) until the copies in flight have landed
            if (*abort_flag)
                for (int kt = max(0, loaded - S); kt < loaded; ++kt)
                    (void)mbar_wait(&full[kt % S], (uint32_t)((kt / S) & 1));
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer ----
            constexpr uint32_t idesc = idesc_tf32(BM, BN);
            for (int kt = 0; kt < ktiles && !*abort_flag; ++kt) {
                const int s = kt % S, j = kt & 1;
                if (!mbar_wait(&full[s], (uint32_t)((kt / S) & 1))) {
                    fail();
                    break;
                }
                if (kt >= 2 && !mbar_wait(&acce[j], (uint32_t)(((kt >> 1) - 1) & 1))) {
                    fail();
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t tx = tmem + (uint32_t)(j * 2 * BN), ty = tx + (uint32_t)BN;
                const uint32_t ah = smem_addr(stage_ptr(s, 0)), al = smem_addr(stage_ptr(s, 1));
                const uint32_t bh = smem_addr(stage_ptr(s, 2)), bl = smem_addr(stage_ptr(s, 3));
#pragma unroll
                for (int kk = 0; kk < BK / 8; ++kk) {
                    const uint32_t off = kk * 32;  // 8 TF32 values = 32 bytes along the swizzled row
                    const uint32_t first = kk > 0 ? 1u : 0u;
                    mma_tf32(tx, sdesc(ah + off), sdesc(bh + off), idesc, first);
                    mma_tf32(ty, sdesc(ah + off), sdesc(bl + off), idesc, first);
                    mma_tf32(ty, sdesc(al + off), sdesc(bh + off), idesc, 1u);
                }
                mma_commit(&empty[s]);  // the stage is free once these MMAs have read it
                mma_commit(&accf[j]);   // and the pair holds this K tile's products
            }
            mma_commit(done);
            if (!mbar_wait(done, 0u)) fail();  // every MMA complete before the TMEM is freed
        }
    } else {
        // ---- epilogue: sum the K tiles in registers ----
        const int quarter = warp & 3;
        const uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
        for (int kt = 0; kt < ktiles; ++kt) {
            const int j = kt & 1;
            if (*abort_flag || !mbar_wait(&accf[j], (uint32_t)((kt >> 1) & 1))) {
                if (!*abort_flag) fail();
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t tx = tmem + lane_off + (uint32_t)(j * 2 * BN), ty = tx + (uint32_t)BN;
#pragma unroll
            for (int c0 = 0; c0 < BN; c0 += 32) {
                uint32_t x[32], y[32];
                tmem_ld32_async(tx + (uint32_t)c0, x);
                tmem_ld32_async(ty + (uint32_t)c0, y);
                tmem_wait32(x);
                tmem_wait32(y);
#pragma unroll
                for (int i = 0; i < 32; ++i) acc[c0 + i] += __uint_as_float(x[i]) + __uint_as_float(y[i]);
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(&acce[j]);
        }
    }
    __syncwarp();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    const bool good = __syncthreads_and(*abort_flag == 0);
    if (good && warp >= 2) {
        const int row = m0 + (warp & 3) * 32 + lane;
        if (row < p.M) {
            float* crow = p.C + (size_t)z * p.c_stride + (size_t)row * p.ldc;
            float* crow2 = p.C2 ? p.C2 + (size_t)z * p.c_stride + (size_t)row * p.ldc : nullptr;
            if (p.mode == kStoreMirror) {
                // an even output: column t holds the values of columns h0 -+ t
#pragma unroll
                for (int i = 0; i < BN; ++i) {
                    const int t = n0 + i;
                    if (t < p.N) {
                        const int q1 = p.mirror_h0 - t, q2 = p.mirror_h0 + t;
                        if (q1 >= 0 && q1 < p.ldc) crow[q1] = acc[i];
                        if (t > 0 && q2 >= 0 && q2 < p.ldc) crow[q2] = acc[i];
                    }
                }
            } else if ((p.ldc & 3) == 0 && (p.c_stride & 3) == 0) {
                // 16-byte stores: the row starts 16-byte aligned and col, ldc are multiples of 4
#pragma unroll
                for (int i = 0; i < BN; i += 4) {
                    const int col = n0 + i;
                    if (col < p.ldc) {
                        float4 v = make_float4(acc[i], acc[i + 1], acc[i + 2], acc[i + 3]);
                        if (p.mode == kStoreTf32) {
                            const float4 h = make_float4(tf32_rna(v.x), tf32_rna(v.y), tf32_rna(v.z), tf32_rna(v.w));
                            *reinterpret_cast<float4*>(crow2 + col) = make_float4(
                                tf32_rna(v.x - h.x), tf32_rna(v.y - h.y), tf32_rna(v.z - h.z), tf32_rna(v.w - h.w));
                            v = h;
                        }
                        *reinterpret_cast<float4*>(crow + col) = v;
                    }
                }
            } else {
#pragma unroll
                for (int i = 0; i < BN; ++i) {
                    const int col = n0 + i;
                    if (col < p.ldc) {
                        if (p.mode == kStoreTf32) {
                            const float hi = tf32_rna(acc[i]);
                            crow[col] = hi;
                            crow2[col] = tf32_rna(acc[i] - hi);
                        } else {
                            crow[col] = acc[i];
                        }
                    }
                }
            }
        }
    }
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)CF::kTmemCols)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// An operand: rows x K FP32 values (hi and lo arrays), leading dimension ld
// (floats, a multiple of 4), batch stride bstride (floats; 0 for a shared operand).
struct Operand {
    const float* hi;
    const float* lo;
    int rows, K, ld;
    long long bstride;
    int batch;  // entries the tensor map covers (1 for a shared operand)
};

inline PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }();
    return fn;
}

// tensor map of one hi or lo array: dims (K, rows, batch), box (32, box_rows, 1), 128-byte swizzle
inline bool make_map(CUtensorMap* m, const float* ptr, const Operand& o, int box_rows) {
    auto enc = encode_fn();
    if (!enc) return false;
    cuuint64_t dims[3] = {(cuuint64_t)o.K, (cuuint64_t)o.rows, (cuuint64_t)(o.batch > 0 ? o.batch : 1)};
    const long long bs = o.bstride > 0 ? o.bstride : (long long)o.ld * o.rows;
    cuuint64_t strides[2] = {(cuuint64_t)o.ld * 4, (cuuint64_t)bs * 4};
    cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(ptr), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace tc
}  // namespace gbg
