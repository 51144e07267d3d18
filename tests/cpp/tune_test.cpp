// CPU test of the batched path's launch-shape tuner (galario_gb300/csrc/gb_tune.h):
// the choice of the fastest candidate from (fake) timings, and the cache file
// that keeps the choices across processes.  Prints "ok" and exits 0 on success.
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "gb_tune.h"

using namespace gbg::tune;

static int fails = 0;
#define EXPECT(c)                                                 \
    do {                                                          \
        if (!(c)) {                                               \
            std::fprintf(stderr, "FAILED %s:%d %s\n", __FILE__, __LINE__, #c); \
            ++fails;                                              \
        }                                                         \
    } while (0)

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string path = std::string(argv[1]) + "/sub/dir/autotune.txt";

    // best_of: the candidate with the smallest best-of-3 time wins, whatever
    // the order and a drift that favours later timings
    {
        int warm = 0, calls = 0;
        const std::vector<int> cand{8, 16, 4};
        auto t = [&](int c) {
            ++calls;
            const double base = c == 16 ? 1.0 : (c == 8 ? 1.2 : 1.5);
            return base - 0.01 * calls;  // drift: later runs look faster
        };
        EXPECT(best_of(cand, [&](int) { ++warm; }, t) == 16);
        EXPECT(warm == 3 && calls == 9);
        // a failing timer returns the first candidate
        EXPECT(best_of(cand, [](int) {}, [](int) { return -1.0; }) == 8);
        EXPECT(best_of(std::vector<int>{}, [](int) {}, [](int) { return 1.0; }) == 8);
        // noisy timings: the best of three decides, not the mean
        int n = 0;
        auto noisy = [&](int c) { ++n; return (c == 4 && n % 3 == 0) ? 0.5 : (c == 4 ? 9.0 : 1.0); };
        EXPECT(best_of(cand, [](int) {}, noisy) == 4);
    }
    // keys
    EXPECT(nvis_bucket(1) == 0 && nvis_bucket(2) == 1 && nvis_bucket(1024) == 10 && nvis_bucket(1025) == 11);
    EXPECT(gpu_token("NVIDIA GB300") == "NVIDIA_GB300");
    const Key k1{"NVIDIA_GB300", 4096, 240, 482, 684, 64, nvis_bucket(2000896), 1, 4096, 0};
    const Key k2{"NVIDIA_GB300", 2048, 101, 205, 656, 256, nvis_bucket(7742651), 0, 4096, 0};
    const Shape s1{16, 8, 8, 16, 8}, s2{8, 108, 8, 8, 4};
    {
        Shape got;
        Key kk;
        EXPECT(parse_line(format_line(k1, s1), &kk, &got) && got.e_rows == 16 && kk.nvis_bucket == 21);
        EXPECT(parse_line(format_line(k2, s2), &kk, &got));
        EXPECT(!(kk < k2) && !(k2 < kk) && got.e_cols == 108 && got.pts == 4);
        EXPECT(!parse_line("garbage", &kk, &got));
        EXPECT(!parse_line(format_line(k1, s1) + " extra", &kk, &got));
    }
    // a first "process" tunes and stores; a second one finds the choices
    {
        Cache c(path);
        Shape got;
        EXPECT(!c.lookup(k1, &got));
        c.store(k1, s1);
        c.store(k2, s2);
        EXPECT(c.lookup(k1, &got) && got.e_rows == 16 && got.pts == 8);
    }
    {
        std::ofstream app(path, std::ios::app);
        app << "this line does not parse\n";
    }
    {
        Cache c(path);
        Shape got;
        EXPECT(c.lookup(k1, &got) && got.e_rows == 16 && got.e_cols == 8 && got.e_rowsT == 16 && got.pts == 8);
        EXPECT(c.lookup(k2, &got) && got.e_cols == 108);
        Key other = k1;
        other.gpu = "NVIDIA_B200";
        EXPECT(!c.lookup(other, &got));  // another kind of GPU tunes again
        c.store(k1, Shape{8, 8, 8, 8, 2});  // a later line for the same key wins
    }
    {
        Cache c(path);
        Shape got;
        EXPECT(c.lookup(k1, &got) && got.e_rows == 8 && got.pts == 2);
    }
    // no file: lookups miss, stores are kept in memory only
    {
        Cache c("");
        Shape got;
        EXPECT(!c.lookup(k1, &got));
        c.store(k1, s1);
        EXPECT(c.lookup(k1, &got) && got.pts == 8);
    }
    if (fails) return 1;
    std::printf("ok\n");
    return 0;
}
