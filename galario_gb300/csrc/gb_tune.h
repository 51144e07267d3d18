// Launch-shape autotuner of the batched passes: the choice of the fastest
// candidate from timings, and a cache file that keeps the choices across
// processes.  Host-only C++17 (no CUDA), so the logic builds and is tested on
// a machine without a GPU.
//
// Cache file: one line per tuned configuration,
//
//   <gpu> f32 <N> <K> <W> <R> <B> <nvis bucket> <grad> <nr> <image> : <e_rows> <e_cols> <e_colsT> <e_rowsT> <pts>
//
// <gpu> is the device name with blanks replaced by '_'; <image> is the pass
// variant (0 profiles with FFT passes, 1 images, 2 profiles with tensor-core
// passes); the visibility count
// enters as its bucket, ceil(log2(padded visibilities)), so datasets of
// similar size share an entry.  Lines that do not parse are skipped; when a
// key appears more than once the last line wins.  Path: GALARIO_TUNE_CACHE if
// set ("" or "0" turns the file off), else $XDG_CACHE_HOME/galario_gb300/
// autotune.txt, else $HOME/.cache/galario_gb300/autotune.txt.
#pragma once

#include <sys/stat.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

namespace gbg {
namespace tune {

struct Shape {
    int e_rows, e_cols, e_colsT, e_rowsT, pts;
};

struct Key {
    std::string gpu;
    int N, K, W, R, B, nvis_bucket, grad, nr, image;
    bool operator<(const Key& o) const {
        return std::tie(gpu, N, K, W, R, B, nvis_bucket, grad, nr, image) <
               std::tie(o.gpu, o.N, o.K, o.W, o.R, o.B, o.nvis_bucket, o.grad, o.nr, o.image);
    }
};

inline int nvis_bucket(long long nd) {
    int b = 0;
    while (b < 62 && (1LL << b) < nd) ++b;
    return b;
}

inline std::string gpu_token(const char* name) {
    std::string s = name ? name : "unknown";
    for (char& c : s)
        if (c == ' ' || c == '\t' || c == ':') c = '_';
    return s.empty() ? std::string("unknown") : s;
}

inline std::string format_line(const Key& k, const Shape& s) {
    std::ostringstream o;
    o << k.gpu << " f32 " << k.N << ' ' << k.K << ' ' << k.W << ' ' << k.R << ' ' << k.B << ' ' << k.nvis_bucket << ' '
      << k.grad << ' ' << k.nr << ' ' << k.image << " : " << s.e_rows << ' ' << s.e_cols << ' ' << s.e_colsT << ' '
      << s.e_rowsT << ' ' << s.pts;
    return o.str();
}

inline bool parse_line(const std::string& line, Key* k, Shape* s) {
    std::istringstream in(line);
    std::string prec, colon;
    if (!(in >> k->gpu >> prec >> k->N >> k->K >> k->W >> k->R >> k->B >> k->nvis_bucket >> k->grad >> k->nr >>
          k->image >> colon >> s->e_rows >> s->e_cols >> s->e_colsT >> s->e_rowsT >> s->pts))
        return false;
    std::string rest;
    if (in >> rest) return false;  // trailing garbage
    return prec == "f32" && colon == ":";
}

inline std::string default_path() {
    const char* env = std::getenv("GALARIO_TUNE_CACHE");
    if (env) {
        if (env[0] == '\0' || (env[0] == '0' && env[1] == '\0')) return std::string();
        return std::string(env);
    }
    const char* xdg = std::getenv("XDG_CACHE_HOME");
    if (xdg && xdg[0]) return std::string(xdg) + "/galario_gb300/autotune.txt";
    const char* home = std::getenv("HOME");
    if (home && home[0]) return std::string(home) + "/.cache/galario_gb300/autotune.txt";
    return std::string();
}

// mkdir -p of the directory part of `path` (best effort)
inline void make_parent_dirs(const std::string& path) {
    for (size_t i = 1; i < path.size(); ++i) {
        if (path[i] != '/') continue;
        const std::string dir = path.substr(0, i);
        if (mkdir(dir.c_str(), 0755) != 0 && errno != EEXIST) return;
    }
}

// The cache file's contents, loaded once; store() appends one line.  A file
// that cannot be read or written only costs a re-tune: it is never an error.
class Cache {
public:
    explicit Cache(std::string path) : path_(std::move(path)) {}
    const std::string& path() const { return path_; }

    bool lookup(const Key& k, Shape* s) {
        std::lock_guard<std::mutex> lk(mu_);
        load_locked();
        auto it = map_.find(k);
        if (it == map_.end()) return false;
        *s = it->second;
        return true;
    }

    void store(const Key& k, const Shape& s) {
        std::lock_guard<std::mutex> lk(mu_);
        load_locked();
        map_[k] = s;
        if (path_.empty()) return;
        make_parent_dirs(path_);
        // one write() of a whole line with O_APPEND semantics: concurrent
        // processes interleave whole lines
        std::FILE* f = std::fopen(path_.c_str(), "a");
        if (!f) return;
        const std::string line = format_line(k, s) + "\n";
        std::fwrite(line.data(), 1, line.size(), f);
        std::fclose(f);
    }

private:
    void load_locked() {
        if (loaded_) return;
        loaded_ = true;
        if (path_.empty()) return;
        std::ifstream in(path_);
        std::string line;
        while (std::getline(in, line)) {
            Key k;
            Shape s;
            if (parse_line(line, &k, &s)) map_[k] = s;
        }
    }
    std::string path_;
    std::mutex mu_;
    bool loaded_ = false;
    std::map<Key, Shape> map_;
};

// The fastest candidate: one untimed run of each, then `reps` rounds of
// timings with the candidates interleaved (so that clock or cache drift
// between them does not decide), each candidate scored by its best time.
// time_ms(c) runs candidate c and returns its time in milliseconds, or a
// negative value on failure (the first candidate is then returned).
template <class Run, class Time>
int best_of(const std::vector<int>& cand, Run&& warm, Time&& time_ms, int reps = 3) {
    if (cand.empty()) return 8;
    std::vector<double> best(cand.size(), 1e300);
    for (int c : cand) warm(c);
    for (int r = 0; r < reps; ++r) {
        for (size_t i = 0; i < cand.size(); ++i) {
            const double ms = time_ms(cand[i]);
            if (ms < 0) return cand[0];
            if (ms < best[i]) best[i] = ms;
        }
    }
    size_t k = 0;
    for (size_t i = 1; i < cand.size(); ++i)
        if (best[i] < best[k]) k = i;
    return cand[k];
}

}  // namespace tune
}  // namespace gbg
