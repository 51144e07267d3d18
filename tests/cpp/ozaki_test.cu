// Unit test of the bf16 tensor-core digit products (galario_gb300/csrc/gb_ozaki.cuh).
//
// 1. Exactness: random integer digit planes (|d| <= 64) for A (M x K) and
//    B (N x K); the kernel's integer sum per element, the sum over its K
//    tiles of V = sum_{L<=5} 2^(7(5-L)) lev_L + round((2^7 lev_6 + lev_7) / 2^14)
//    with lev_L = sum_{i+j=L} sum_{k in the tile} A_i B_j, must equal the
//    int64 result exactly, including M, N, K that are not multiples of the
//    tiles (zero fill), every digit at +-64 (the largest level sums of a K
//    tile) and K of many tiles.
// 2. FP64 products: random doubles with rows of widely different scales, the
//    digits of digits8, the kernel, and the sums combined in double;
//    compared with a long double product, the error must stay below
//    2^-50 K max|a_row| max|b_row| for every element.
// Prints one line per case and exits nonzero on the first failure.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "gb_ozaki.cuh"

using namespace gbg;

#define CK(x)                                                                                   \
    do {                                                                                        \
        cudaError_t e_ = (x);                                                                   \
        if (e_ != cudaSuccess) {                                                                \
            std::printf("CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
            std::exit(2);                                                                       \
        }                                                                                       \
    } while (0)

struct Planes {
    int rows, K, ld;
    std::vector<unsigned short> h;  // [plane][row][ld]
    std::vector<int> v;             // integer digits, same layout
    unsigned short* d = nullptr;
    Planes(int r, int k) : rows(r), K(k), ld((k + 7) / 8 * 8) {
        h.assign((size_t)oz::kPlanes * rows * ld, 0);
        v.assign(h.size(), 0);
    }
    size_t at(int s, int r, int k) const { return ((size_t)s * rows + r) * ld + k; }
    void set(int s, int r, int k, int x) {
        v[at(s, r, k)] = x;
        h[at(s, r, k)] = oz::bf16_of_int(x);
    }
    void upload() {
        CK(cudaMalloc(&d, h.size() * 2));
        CK(cudaMemcpy(d, h.data(), h.size() * 2, cudaMemcpyHostToDevice));
    }
    ~Planes() {
        if (d) cudaFree(d);
    }
};

// the kernel's sums on the GPU: P[n * ldm + m]
static std::vector<long long> run_levels(const Planes& A, const Planes& B, oz::Dims* dims) {
    CUtensorMap am, bm;
    if (!oz::make_map(&am, A.d, A.K, A.rows, A.ld, (long long)A.rows * A.ld, oz::BM) ||
        !oz::make_map(&bm, B.d, B.K, B.rows, B.ld, (long long)B.rows * B.ld, oz::BN)) {
        std::printf("tensor map encoding failed\n");
        std::exit(2);
    }
    const oz::Dims dm = oz::dims_of(A.rows, B.rows);
    long long* P = nullptr;
    unsigned* err = nullptr;
    const size_t np = (size_t)dm.N * dm.ldm;
    CK(cudaMalloc(&P, np * 8));
    CK(cudaMemset(P, 0, np * 8));
    CK(cudaMalloc(&err, 4));
    CK(cudaMemset(err, 0, 4));
    oz::Params p{};
    p.m_max = A.rows;
    p.n_max = B.rows;
    p.K = A.K;
    p.P = P;
    p.err = err;
    CK(cudaFuncSetAttribute(oz::ozaki_levels_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, oz::kSmem));
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0));
    oz::ozaki_levels_kernel<<<nsm, oz::kThreads, oz::kSmem>>>(am, bm, p);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    unsigned herr = 0;
    CK(cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost));
    if (herr) {
        std::printf("kernel reported error %u\n", herr);
        std::exit(1);
    }
    std::vector<long long> out(np);
    CK(cudaMemcpy(out.data(), P, np * 8, cudaMemcpyDeviceToHost));
    cudaFree(P);
    cudaFree(err);
    *dims = dm;
    return out;
}

static int exact_case(int M, int N, int K, bool extreme, unsigned seed) {
    std::mt19937 rng(seed);
    std::uniform_int_distribution<int> dig(-64, 64);
    Planes A(M, K), B(N, K);
    for (int s = 0; s < oz::kPlanes; ++s) {
        for (int r = 0; r < M; ++r)
            for (int k = 0; k < K; ++k) A.set(s, r, k, extreme ? 64 : dig(rng));
        for (int r = 0; r < N; ++r)
            for (int k = 0; k < K; ++k) B.set(s, r, k, extreme ? 64 : dig(rng));
    }
    A.upload();
    B.upload();
    oz::Dims dm;
    const std::vector<long long> P = run_levels(A, B, &dm);
    long long bad = 0, maxabs = 0;
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            long long want = 0;
            for (int k0 = 0; k0 < K; k0 += oz::BK) {  // one K tile at a time, as the kernel folds them
                float lev[oz::kLevels];
                for (int L = 0; L < oz::kLevels; ++L) {
                    long long l = 0;
                    for (int i = 0; i <= L; ++i) {
                        const int j = L - i;
                        if (i >= oz::kPlanes || j >= oz::kPlanes) continue;
                        for (int k = k0; k < std::min(K, k0 + oz::BK); ++k)
                            l += (long long)A.v[A.at(i, m, k)] * B.v[B.at(j, n, k)];
                    }
                    maxabs = std::max(maxabs, std::llabs(l));
                    lev[L] = (float)l;  // below 2^24: exact
                }
                want += oz::fold_levels(lev);
            }
            const long long got = P[(size_t)n * dm.ldm + m];
            if (got != want) {
                if (bad < 5) std::printf("  (%d, %d): got %lld want %lld\n", m, n, got, want);
                ++bad;
            }
        }
    std::printf("exact M=%d N=%d K=%d%s: %lld mismatches, max |level of a K tile| %lld (2^%.1f)\n", M, N, K,
                extreme ? " (every digit 64)" : "", bad, maxabs, std::log2((double)maxabs));
    return bad == 0 ? 0 : 1;
}

static int fp64_case(int M, int N, int K, unsigned seed) {
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    std::vector<double> a((size_t)M * K), b((size_t)N * K);
    // rows of widely different scales, and elements spanning 2^-30 .. 1 of their row
    for (int r = 0; r < M; ++r) {
        const double sc = std::ldexp(1.0, (int)(rng() % 80) - 40);
        for (int k = 0; k < K; ++k) a[(size_t)r * K + k] = sc * u(rng) * std::ldexp(1.0, -(int)(rng() % 31));
    }
    for (int r = 0; r < N; ++r) {
        const double sc = std::ldexp(1.0, (int)(rng() % 80) - 40);
        for (int k = 0; k < K; ++k) b[(size_t)r * K + k] = sc * u(rng) * std::ldexp(1.0, -(int)(rng() % 31));
    }
    Planes A(M, K), B(N, K);
    std::vector<int> ea(M), eb(N);
    auto slice = [](const std::vector<double>& x, int rows, int K, Planes& P, std::vector<int>& e) {
        for (int r = 0; r < rows; ++r) {
            double mx = 0;
            for (int k = 0; k < K; ++k) mx = std::max(mx, std::fabs(x[(size_t)r * K + k]));
            e[r] = oz::row_exponent(mx);
            for (int k = 0; k < K; ++k) {
                int d[oz::kPlanes];
                oz::digits8(x[(size_t)r * K + k], e[r], d);
                for (int s = 0; s < oz::kPlanes; ++s) P.set(s, r, k, d[s]);
            }
        }
    };
    slice(a, M, K, A, ea);
    slice(b, N, K, B, eb);
    A.upload();
    B.upload();
    oz::Dims dm;
    const std::vector<long long> P = run_levels(A, B, &dm);
    double worst = 0;
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            const double acc = oz::combine_levels(P[(size_t)n * dm.ldm + m]);
            const double got = std::ldexp(acc, ea[m] + eb[n] - 12);
            long double ref = 0, amax = 0, bmax = 0;
            for (int k = 0; k < K; ++k) {
                ref += (long double)a[(size_t)m * K + k] * (long double)b[(size_t)n * K + k];
                amax = std::max(amax, (long double)std::fabs(a[(size_t)m * K + k]));
                bmax = std::max(bmax, (long double)std::fabs(b[(size_t)n * K + k]));
            }
            const double scale = (double)(K * amax * bmax);
            const double rel = scale > 0 ? (double)std::fabs((long double)got - ref) / scale : 0.0;
            worst = std::max(worst, rel);
        }
    std::printf("fp64 M=%d N=%d K=%d: max |err| / (K max|a| max|b|) = %.3g (2^%.1f)\n", M, N, K, worst,
                worst > 0 ? std::log2(worst) : -999.0);
    return worst <= std::ldexp(1.0, -50) ? 0 : 1;
}

int main() {
    int fails = 0;
    fails += exact_case(128, 64, 64, false, 1);
    fails += exact_case(240, 130, 343, false, 2);   // ragged sizes of the nxy=4096 profile products
    fails += exact_case(200, 130, 511, true, 3);    // the largest level sums of every K tile
    fails += exact_case(37, 5, 9, false, 4);        // one partial tile
    fails += exact_case(130, 70, 2000, true, 7);    // many K tiles (32), every digit 64
    fails += fp64_case(240, 242, 343, 5);
    fails += fp64_case(130, 70, 100, 6);
    fails += fp64_case(150, 200, 1500, 8);
    std::printf(fails ? "FAILED %d\n" : "OK\n", fails);
    return fails ? 1 : 0;
}
