// C ABI of galario_gb300: the drop-in boundary for galario's
// sampleImage / chi2Image / sampleProfile / chi2Profile (reference
// src/galario_py.h:30-46) plus the expert stages and runtime helpers
// (src/galario.h:24-59).  See include/galario_gb300.h for the contract.
//
// Every entry point returns a status (GALARIO_OK, GALARIO_EINVAL,
// GALARIO_ENOMEM, GALARIO_ERUNTIME) and leaves a message for the calling
// thread in galario_last_error(), the way the reference throws
// std::invalid_argument / std::bad_alloc / std::runtime_error
// (src/galario.cpp:89-198) and Cython maps them to ValueError / MemoryError /
// RuntimeError (python/galario_defs.pxd:24-46).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/galario_gb300.h"
#include "gb_device.cuh"
#include "gb_internal.cuh"

namespace gbg {
void noalloc_forget_scratch();  // gb_noalloc.cu

namespace {

thread_local std::string g_msg;
thread_local int g_tpb = 16;  // galario threads(): accepted for API compatibility

struct InvalidArg : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct OutOfMemory : std::runtime_error {
    using std::runtime_error::runtime_error;
};

void cuda_check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return;
    cudaGetLastError();  // clear sticky-free errors
    if (e == cudaErrorMemoryAllocation) throw OutOfMemory(std::string("cuda out of memory in ") + what);
    if (e == cudaErrorInitializationError || e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        throw std::runtime_error("Error in cuda: Could not initialize cuda. Is a CUDA GPU available at all?");
    throw std::runtime_error(std::string("Error in cuda (") + what + "): " + cudaGetErrorString(e));
}
#define CK(x) cuda_check((x), #x)

template <class F> int guarded(F&& f) {
    try {
        f();
        return GALARIO_OK;
    } catch (const InvalidArg& e) {
        g_msg = e.what();
        return GALARIO_EINVAL;
    } catch (const OutOfMemory& e) {
        g_msg = e.what();
        return GALARIO_ENOMEM;
    } catch (const std::bad_alloc&) {
        g_msg = "std::bad_alloc";
        return GALARIO_ENOMEM;
    } catch (const std::exception& e) {
        g_msg = e.what();
        return GALARIO_ERUNTIME;
    }
}

// reference CHECK_INPUT / CHECK_INPUTXY, src/galario.cpp:101-111
void check_input(long long nx) {
    if (nx < 2)
        throw InvalidArg("Error in check input image: x dimension = " + std::to_string(nx) + " is less than 2");
    if (nx % 2 != 0) throw InvalidArg("Error in check input image: x dimension = " + std::to_string(nx) + " is odd");
}
void check_square(long long nx, long long ny) {
    if (nx != ny)
        throw InvalidArg("Error in check input image: Expect a square image but got shape (" + std::to_string(nx) +
                         ", " + std::to_string(ny) + ")");
    check_input(nx);
}
void check_nd(int nd) {
    if (nd < 0) throw InvalidArg("Error: negative number of visibilities " + std::to_string(nd));
}

// ---------------------------------------------------------------------------
// per-device context: stream, grow-only device buffers, twiddle tables
// ---------------------------------------------------------------------------
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    void* get(size_t bytes) {
        if (bytes == 0) bytes = 16;
        if (bytes > cap) {
            if (p) cudaFree(p);
            p = nullptr;
            cap = 0;
            CK(cudaMalloc(&p, bytes));
            cap = bytes;
        }
        return p;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct Ctx {
    int device = 0;
    std::mutex mu;
    cudaStream_t stream = nullptr;
    // second stream: the host-pointer chi2 calls upload the observations
    // (Re, Im, w) on it while the spectrum passes run on `stream`
    cudaStream_t side = nullptr;
    cudaEvent_t ev_side_start = nullptr, ev_obs = nullptr;
    // overlapped host-pointer chi2Profile: (u, v) uploaded, then each chunk's observations
    static constexpr int kMaxChunks = 4;
    cudaEvent_t ev_uv = nullptr, ev_chunk[kMaxChunks] = {};
    // odd chunks of the visibility pass run on vis2, so that one chunk's
    // tail overlaps the next chunk's start
    cudaStream_t vis2 = nullptr;
    cudaEvent_t ev_win = nullptr, ev_vis2 = nullptr;
    // device-resident FP64 profiles: the extent pass runs on `side` beside
    // the sweep's fold (which does not need the window)
    cudaEvent_t ev_ext_start = nullptr, ev_ext_done = nullptr;
    DevBuf state, partials, img, prof, u, v, re, im, w, vis, zt, win, amp, quad, urot, vrot;
    double2* phase_tab = nullptr;  // table of the FP64 phase shift (PHASE_T entries)
    ProfileTc* ptc = nullptr;      // tensor-core spectrum of FP64 profiles (created on first use)
    ProfileTc* profile_tc() {
        if (!ptc) ptc = profile_tc_new();
        return ptc;
    }
    std::map<std::pair<int, int>, void*> tw;   // (N, sizeof(T)) -> table
    std::map<std::pair<int, int>, void*> stw;  // (L * 32 + E, sizeof(T)) -> stage twiddles
    DevState* host_state = nullptr;           // pinned mirror of DevState
    // the device reads pageable host memory coherently (address translation
    // services, e.g. NVLink-C2C on Grace): kernels can read the caller's arrays
    bool host_readable = false;
    // optional per-stage CUDA-event timing (galario_stage_timing)
    bool timing = false;
    struct Rec {
        int stage;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> spare;
    cudaEvent_t event() {
        cudaEvent_t e;
        if (!spare.empty()) {
            e = spare.back();
            spare.pop_back();
            return e;
        }
        CK(cudaEventCreate(&e));
        return e;
    }

    void init(int dev) {
        device = dev;
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ev_side_start, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ev_obs, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ev_uv, cudaEventDisableTiming));
        CK(cudaStreamCreateWithFlags(&vis2, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ev_win, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ev_vis2, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ev_ext_start, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ev_ext_done, cudaEventDisableTiming));
        for (auto& e : ev_chunk) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        CK(cudaMallocHost(&host_state, sizeof(DevState)));
        int pageable = 0;
        CK(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
        host_readable = pageable != 0;
        // exp(2 pi i j / T), j in [0, T), as exp(2 pi i jh / 2^10) exp(2 pi i jl / T)
        // with j = 2^10 jh + jl: the two factors of 2^10 entries each from long
        // double, kept as double-double pairs, multiplied in double-double
        // arithmetic (products by fma, Dekker/Knuth) and rounded once
        std::vector<double2> h(PHASE_T);
        {
            constexpr int kLo = 1 << 10, kHi = PHASE_T / kLo;
            const long double two_pi = 6.283185307179586476925286766559005768L;
            struct DD {
                double hi, lo;
            };
            auto dd = [](long double x) {
                const double hi = (double)x;
                return DD{hi, (double)(x - (long double)hi)};
            };
            std::vector<DD> ch(kHi), sh(kHi), cl(kLo), sl(kLo);
            for (int i = 0; i < kHi; ++i) {
                const long double a = two_pi * (long double)i / (long double)kHi;
                ch[i] = dd(cosl(a));
                sh[i] = dd(sinl(a));
            }
            for (int i = 0; i < kLo; ++i) {
                const long double a = two_pi * (long double)i / (long double)PHASE_T;
                cl[i] = dd(cosl(a));
                sl[i] = dd(sinl(a));
            }
            auto mul = [](DD x, DD y) {  // x y to about 2^-104
                const double p = x.hi * y.hi;
                return DD{p, std::fma(x.hi, y.hi, -p) + (x.hi * y.lo + x.lo * y.hi)};
            };
            auto add = [](DD x, DD y) {  // two-sum of the high parts, then the low parts
                const double s = x.hi + y.hi, bb = s - x.hi;
                const double e = (x.hi - (s - bb)) + (y.hi - bb);
                return DD{s, e + (x.lo + y.lo)};
            };
            auto neg = [](DD x) { return DD{-x.hi, -x.lo}; };
            for (int jh = 0; jh < kHi; ++jh)
                for (int jl = 0; jl < kLo; ++jl) {
                    const DD c = add(mul(ch[jh], cl[jl]), neg(mul(sh[jh], sl[jl])));
                    const DD sn = add(mul(sh[jh], cl[jl]), mul(ch[jh], sl[jl]));
                    h[(size_t)jh * kLo + jl] = make_double2(c.hi + c.lo, sn.hi + sn.lo);
                }
        }
        CK(cudaMalloc(&phase_tab, sizeof(double2) * PHASE_T));
        CK(cudaMemcpy(phase_tab, h.data(), sizeof(double2) * PHASE_T, cudaMemcpyHostToDevice));
    }
    void release_all() {
        DevBuf* bufs[] = {&state, &partials, &img, &prof, &u, &v, &re, &im, &w, &vis, &zt, &win, &amp, &quad,
                          &urot, &vrot};
        for (DevBuf* b : bufs) b->release();
        profile_tc_free(ptc);
        ptc = nullptr;
        for (auto& kv : tw) cudaFree(kv.second);
        tw.clear();
        for (auto& kv : stw) cudaFree(kv.second);
        stw.clear();
    }
    // stage twiddles of the shared-memory FFT of length L (power of two), cached per (L, precision)
    // stage twiddles of the length-L FFT with E values per thread (E <= 0: fft_e)
    template <typename T> const C2<T>* stage_tw(int L, int E = 0) {
        if (E <= 0) E = fft_e<T>(L);
        auto key = std::make_pair(L * 32 + E, (int)sizeof(T));
        auto it = stw.find(key);
        if (it != stw.end()) return static_cast<const C2<T>*>(it->second);
        std::vector<C2<T>> h = stage_twiddles<T>(L, E);
        void* d = nullptr;
        CK(cudaMalloc(&d, sizeof(C2<T>) * h.size()));
        CK(cudaMemcpy(d, h.data(), sizeof(C2<T>) * h.size(), cudaMemcpyHostToDevice));
        stw[key] = d;
        return static_cast<const C2<T>*>(d);
    }
    // twiddles exp(-2 pi i m / N), m in [0, N), from long double, cached per (N, precision)
    template <typename T> const C2<T>* twiddles(int N) {
        auto key = std::make_pair(N, (int)sizeof(T));
        auto it = tw.find(key);
        if (it != tw.end()) return static_cast<const C2<T>*>(it->second);
        std::vector<C2<T>> h((size_t)N);
        const long double two_pi = 6.283185307179586476925286766559005768L;
        for (int m = 0; m < N; ++m) {
            // exact symmetry folding keeps the argument small: angle = 2 pi m / N
            long double a = -two_pi * (long double)m / (long double)N;
            h[(size_t)m].x = (T)cosl(a);
            h[(size_t)m].y = (T)sinl(a);
        }
        void* d = nullptr;
        CK(cudaMalloc(&d, sizeof(C2<T>) * (size_t)N));
        CK(cudaMemcpy(d, h.data(), sizeof(C2<T>) * (size_t)N, cudaMemcpyHostToDevice));
        tw[key] = d;
        return static_cast<const C2<T>*>(d);
    }
};

std::mutex g_ctx_mu;
std::map<int, Ctx*> g_ctx;

Ctx& ctx() {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    auto it = g_ctx.find(dev);
    if (it != g_ctx.end()) return *it->second;
    Ctx* c = new Ctx();
    c->init(dev);
    g_ctx[dev] = c;
    return *c;
}

// Run f (which enqueues work on s); with timing on, bracket it with events.
template <class F> void timed(Ctx& c, cudaStream_t s, int stage, F&& f) {
    if (!c.timing) {
        f();
        return;
    }
    cudaEvent_t a = c.event(), b = c.event();
    CK(cudaEventRecord(a, s));
    f();
    CK(cudaEventRecord(b, s));
    c.recs.push_back(Ctx::Rec{stage, a, b});
}
enum { ST_H2D = 0, ST_EXTENT, ST_ROWS, ST_COLS, ST_VIS, ST_D2H, ST_QUAD, ST_COUNT };
const char* const kStageNames[ST_COUNT] = {"h2d", "extent", "rows", "cols", "vis", "d2h", "quad"};

template <typename T> T* as(DevBuf& b, size_t count) { return static_cast<T*>(b.get(sizeof(T) * count)); }

// Host-pointer chi2 calls read the caller's arrays from the kernels where the
// device can (GALARIO_ZERO_COPY=0 keeps the copy-engine uploads).
bool zero_copy(const Ctx& c) {
    const char* v = std::getenv("GALARIO_ZERO_COPY");
    return c.host_readable && !(v && v[0] == '0');
}
// visibilities whose observations the staged schedule copies ahead (while
// the column pass runs); the rest are read in place by the visibility pass
inline int staged_head(int nd) { return std::min(nd / 4, 3 << 17) & ~255; }
// page-locked (or registered) host memory: the copy engines read it without
// blocking the host
bool is_pinned(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

void h2d(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    if (bytes) CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
}
void d2h(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    if (bytes) CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
}

// Read back DevState and turn device-side error bits into exceptions.
void finish(Ctx& c, DevState* st_d) {
    d2h(c.host_state, st_d, sizeof(DevState), c.stream);
    CK(cudaStreamSynchronize(c.stream));
    const DevState& h = *c.host_state;
    if (h.err & ERR_UV_NONFINITE)
        throw InvalidArg("Error in interpolate: u or v is not finite (first at index " +
                         std::to_string((long long)h.err_index - 1) + ")");
    if (h.err & ERR_UV_OUTSIDE)
        throw InvalidArg(
            "Error in interpolate: a (u, v) point lies outside the image spectrum, |u|/duv or |v|/duv is too large "
            "for nxy (first at index " + std::to_string((long long)h.err_index - 1) +
            "); use check=True or a larger nxy / smaller dxy");
    if (h.err & ERR_WINDOW) throw std::runtime_error("Error in interpolate: internal spectrum window error");
    if (h.err) throw std::runtime_error("Error: device reported error bits " + std::to_string(h.err));
}

// central pixel of the swept image (reference create_image_d, src/galario.cpp:1135-1153)
double central_pixel(const double* I, int nr, double Rmin, double dR, double dxy) {
    const int iIN = (int)std::floor((dxy / 2 - Rmin) / dR);
    if (iIN < 0 || iIN + 1 >= nr)
        throw InvalidArg("Error in create image: the intensity profile (nr = " + std::to_string(nr) +
                         ") does not reach the edge of the central pixel (needs index " + std::to_string(iIN + 1) +
                         ")");
    double flux = 0.;
    for (int i = 1; i < iIN; ++i) flux += (Rmin + dR * i) * I[i];
    flux *= 2.;
    flux += Rmin * I[0] + (Rmin + iIN * dR) * I[iIN];
    flux *= dR;
    const double I_interp = (I[iIN + 1] - I[iIN]) / dR * (dxy / 2. - (Rmin + dR * iIN)) + I[iIN];
    flux += ((Rmin + iIN * dR) * I[iIN] + dxy / 2. * I_interp) * (dxy / 2. - (Rmin + iIN * dR));
    const double area = std::pow(dxy / 2., 2) - std::pow(Rmin, 2);
    return dxy * dxy * flux / area;
}

// reference CHECK_CENTRAL_PIXEL, src/galario.cpp:113-121
void check_central_pixel(double dxy, double Rmin, double dR) {
    const double ratio = (dxy / 2. - Rmin) / dR;
    if (ratio < 5)
        throw InvalidArg(
            "Error in create image: Expect (dxy/2-Rmin)/dR > 5, i.e. dR small enough to ensure reliable "
            "interpolation the inside central pixel but got (dxy/2-Rmin)/dR = " + std::to_string(ratio) +
            ". Try reducing dR.");
}

struct ProfileGeom {
    int rmax;
    double central;
};

template <typename T>
ProfileGeom profile_geom(const T* I_host, int nr, double Rmin, double dR, double dxy, int nxy) {
    check_central_pixel(dxy, Rmin, dR);
    if (nr < 2) throw InvalidArg("Error in create image: the intensity profile needs at least 2 samples");
    if (nr >= (1 << 22)) throw InvalidArg("Error in create image: the intensity profile is limited to 2^22 samples");
    std::vector<double> Id((size_t)nr);
    for (int i = 0; i < nr; ++i) Id[(size_t)i] = (double)I_host[i];
    ProfileGeom g;
    g.central = central_pixel(Id.data(), nr, Rmin, dR, dxy);
    long long r = (long long)std::ceil((Rmin + nr * dR) / dxy);
    g.rmax = (int)(r < nxy / 2 ? r : nxy / 2);
    if (g.rmax < 0) g.rmax = 0;
    return g;
}

// ---------------------------------------------------------------------------
// the pipeline, device side
// ---------------------------------------------------------------------------
// A host-pointer call whose uploads run on the side stream while the
// spectrum passes run: the row pass writes every column (it does not wait
// for the extent), the extent pass waits for ev_uv, and the visibility pass
// runs in `nchunks` launches over consecutive ranges, chunk c after
// ev_chunk[c] (its Re, Im, w uploaded), alternately on `stream` and `vis2`;
// the chi2 reduction is finished by the last block of all chunks.
struct Overlap {
    cudaEvent_t ev_uv = nullptr;
    int nchunks = 1;
    const cudaEvent_t* ev_chunk = nullptr;
    // Staged mode (a device that reads host memory directly): the pass that
    // copied (u, v) to the device also computed the extent; visibilities
    // [0, n0) have their (Re, Im, w) copied to re0/im0/w0 (ready at
    // ev_chunk[0]) and [n0, nd) are read from the caller's arrays by the
    // visibility pass itself.
    bool staged = false;
    bool extent_done = false;  // the staging pass computed the extent (else the pipeline runs it after ev_uv)
    int n0 = 0;
    const void *re0 = nullptr, *im0 = nullptr, *w0 = nullptr;
};
// chunk c of nd visibilities in n chunks: [chunk_begin(nd, n, c), chunk_begin(nd, n, c + 1))
// (equal sizes: chunks falling in size, so that less is left after the last
// upload, measured no faster)
inline int chunk_begin(int nd, int n, int c) { return (int)((long long)nd * c / n); }

template <typename T> struct Pipe {
    using CT = C2<T>;
    using L = Launch<T>;

    // Enqueue spectrum window + visibility pass.  All pointers are device
    // pointers.  img != nullptr selects the image path, else the profile path.
    static void enqueue(Ctx& c, cudaStream_t s, int N, double duv, const T* img, const T* prof, int nr, double Rmin,
                        double dR, double dxy, double inc, const ProfileGeom* pg, double v_origin, double dRA,
                        double dDec, double PA, int nd, const T* u, const T* v, const T* re, const T* im, const T* w,
                        CT* vis_out, bool chi2, double* chi2_out, DevState* st, bool have_extent,
                        const std::function<void()>& before_vis = std::function<void()>(),
                        const Overlap* ov = nullptr) {
        const int C = N / 2 + 1;
        const CT* tw = c.twiddles<T>(N);
        CT* zt = as<CT>(c.zt, (size_t)C * N);
        CT* win = as<CT>(c.win, (size_t)C * N);
        T* amp = as<T>(c.amp, (size_t)C * N);
        const long long qcap = std::min<long long>((long long)C * N, QUAD_CAP);
        T* quads = as<T>(c.quad, (size_t)qcap * QUAD_REC);
        const int nchunks = (ov && nd > 0) ? ov->nchunks : 1;
        const bool staged = ov && ov->staged && nd > 0;
        // visibility ranges of the launches: staged, [0, n0) and [n0, nd); else the chunks
        std::vector<std::pair<int, int>> ranges;
        if (staged) {
            ranges.emplace_back(0, nd);
        } else {
            for (int k = 0; k < nchunks; ++k) ranges.emplace_back(chunk_begin(nd, nchunks, k), chunk_begin(nd, nchunks, k + 1));
        }
        size_t nparts = 0;
        for (const auto& r : ranges) nparts += (size_t)L::vis_grid(std::max(1, r.second - r.first));
        double* partials = as<double>(c.partials, nparts);
        // FP64 swept profiles whose quadrant fits the tensor-core products:
        // the window as two cosine-matrix products (gb_profile_tc.cu) instead
        // of the row and column transforms
        const bool tc_prof = !img && sizeof(T) == 8 && profile_tc_ok(N, pg->rmax);
        // the extent pass beside the tensor-core path's fold, on the side stream
        const bool ext_side = tc_prof && !have_extent && !ov;
        if (ext_side) {
            CK(cudaEventRecord(c.ev_ext_start, s));
            CK(cudaStreamWaitEvent(c.side, c.ev_ext_start, 0));
            timed(c, c.side, ST_EXTENT, [&] { CK(L::extent(u, v, nd, N, duv, st, c.side)); });
            CK(cudaEventRecord(c.ev_ext_done, c.side));
        } else if (!have_extent && !ov) {
            timed(c, s, ST_EXTENT, [&] { CK(L::extent(u, v, nd, N, duv, st, s)); });
        }
        int band0 = 0, band1 = N;
        const CT* stw_rows = c.stage_tw<T>(N / 2 > 0 ? N / 2 : 1);
        const CT* stw_cols = c.stage_tw<T>(N);
        // FP64 swept profiles: rows and columns as even-sequence transforms (FFT
        // length N/4); the FP32 passes are faster as paired transforms
        const CT* stw_q = (!img && !tc_prof && sizeof(T) == 8 && even_dft_ok<T>(N))
                              ? c.stage_tw<T>(N / 4, even_dft_e<T>(N))
                              : nullptr;
        if (img) {
            timed(c, s, ST_ROWS, [&] { CK(L::rows_image(img, N, tw, stw_rows, zt, -1, st, duv, true, s)); });
        } else if (tc_prof) {
            if constexpr (sizeof(T) == 8) {
                timed(c, s, ST_ROWS, [&] {
                    CK(profile_tc_fold(c.profile_tc(), prof, nr, Rmin, dR, dxy, std::cos(inc), pg->rmax, pg->central,
                                       N, s));
                });
            }
        } else {
            band0 = N / 2 - pg->rmax;
            band1 = N / 2 + pg->rmax;
            timed(c, s, ST_ROWS, [&] {
                CK(L::rows_profile(prof, nr, Rmin, dR, dxy, std::cos(inc), pg->rmax, pg->central, N, tw, stw_rows, zt,
                                   st, duv, s, ov ? C : -1, stw_q));
            });
        }
        if (ov) {
            CK(cudaStreamWaitEvent(s, ov->ev_uv, 0));
            if (!ov->extent_done) timed(c, s, ST_EXTENT, [&] { CK(L::extent(u, v, nd, N, duv, st, s)); });
        }
        if (ext_side) CK(cudaStreamWaitEvent(s, c.ev_ext_done, 0));
        // window layout: column k at win + k*N, rows [r0, r0+W) contiguous
        timed(c, s, ST_COLS, [&] {
            if (img) {
                CK(L::cols(zt, N, band0, band1, tw, stw_cols, win, amp, 1, N, -1, -1, -1, st, duv, true, s));
            } else if (tc_prof) {
                if constexpr (sizeof(T) == 8)
                    CK(profile_tc_window(c.profile_tc(), N, st, win, amp, 1, N, s));
            } else {
                CK(L::cols_profile(zt, N, band0, band1, tw, stw_cols, win, amp, 1, N, st, duv, s, stw_q));
            }
        });
        // a swept profile's spectrum is real: 4 real corners per cell record
        const bool real_spec = img == nullptr;
        // the tensor-core chain's last passes, the cell records and the
        // visibility pass follow one another on s: programmatic dependents
        const bool pdl = tc_prof && !ov && !before_vis && !c.timing;  // no event records between the kernels
        timed(c, s, ST_QUAD, [&] {
            if (real_spec)
                CK(L::quads_real(win, 1, N, C, st, quads, qcap, s, pdl));
            else
                CK(L::quads(win, amp, 1, N, C, st, quads, qcap, -1, -1, -1, s));
        });
        typename L::VisArgs a;
        a.spec = win;
        a.amp = amp;
        a.quads = quads;
        a.real_quads = real_spec;
        a.quad_cap = qcap;
        a.phase_tab = c.phase_tab;
        a.s_row = 1;
        a.s_col = N;
        a.nrow = N;
        a.ncol = C;
        a.host_K = a.host_r0 = a.host_W = -1;
        a.duv = duv;
        a.v_origin = v_origin;
        a.rotate = (PA != 0.);
        a.cos_pa = a.rotate ? std::cos(PA) : 1.;
        a.sin_pa = a.rotate ? std::sin(PA) : 0.;
        // rotated offsets, computed on the host as in the reference (:1305)
        double dra = dRA, ddec = dDec;
        if (a.rotate) {
            dra = dRA * a.cos_pa - dDec * a.sin_pa;
            ddec = dRA * a.sin_pa + dDec * a.cos_pa;
        }
        a.dra = dra;
        a.ddec = ddec;
        a.phase = !(dra == 0. && ddec == 0.);
        a.u = u;
        a.v = v;
        a.re = re;
        a.im = im;
        a.w = w;
        a.nd = nd;
        a.vis_out = vis_out;
        a.partials = chi2 ? partials : nullptr;
        a.chi2_out = chi2_out;
        a.state = st;
        if (before_vis) before_vis();
        if (staged) {
            // one launch: the first n0 visibilities' observations from their
            // device copies (ready at ev_chunk[0]), the rest read in place
            a.re = static_cast<const T*>(ov->re0);
            a.im = static_cast<const T*>(ov->im0);
            a.w = static_cast<const T*>(ov->w0);
            a.re2 = re;
            a.im2 = im;
            a.w2 = w;
            a.split = ov->n0;
            CK(cudaStreamWaitEvent(s, ov->ev_chunk[0], 0));
            timed(c, s, ST_VIS, [&] { CK(L::vis(a, s)); });
        } else if (nd > 0 && ov) {
            int total = 0;
            for (int k = 0; k < nchunks; ++k)
                total += L::vis_grid(std::max(1, chunk_begin(nd, nchunks, k + 1) - chunk_begin(nd, nchunks, k)));
            CK(cudaEventRecord(c.ev_win, s));
            CK(cudaStreamWaitEvent(c.vis2, c.ev_win, 0));
            int off = 0;
            for (int k = 0; k < nchunks; ++k) {
                const int b0 = chunk_begin(nd, nchunks, k), b1 = chunk_begin(nd, nchunks, k + 1);
                typename L::VisArgs ak = a;
                ak.u = u + b0;
                ak.v = v + b0;
                ak.re = re ? re + b0 : nullptr;
                ak.im = im ? im + b0 : nullptr;
                ak.w = w ? w + b0 : nullptr;
                ak.vis_out = vis_out ? vis_out + b0 : nullptr;
                ak.nd = b1 - b0;
                ak.base = b0;
                ak.part_off = off;
                ak.parts_total = total;
                cudaStream_t sk = (k & 1) ? c.vis2 : s;
                CK(cudaStreamWaitEvent(sk, ov->ev_chunk[k], 0));
                CK(L::vis(ak, sk));
                off += L::vis_grid(std::max(1, ak.nd));
            }
            CK(cudaEventRecord(c.ev_vis2, c.vis2));
            CK(cudaStreamWaitEvent(s, c.ev_vis2, 0));
        } else if (nd > 0) {
            timed(c, s, ST_VIS, [&] { CK(L::vis(a, s, pdl)); });
        }
    }
};

// Upload the observations of a host-pointer chi2 call on the side stream,
// ordered after everything already on `s`; returns the hook that makes `s`
// wait for them just before the visibility pass, so that the copies overlap
// the extent, row, column and cell-record passes.
template <typename T>
std::function<void()> upload_obs(Ctx& c, cudaStream_t s, T* re_d, const T* re, T* im_d, const T* im, T* w_d,
                                 const T* w, int nd) {
    CK(cudaEventRecord(c.ev_side_start, s));
    CK(cudaStreamWaitEvent(c.side, c.ev_side_start, 0));
    return [&c, s, re_d, re, im_d, im, w_d, w, nd] {
        h2d(re_d, re, sizeof(T) * (size_t)nd, c.side);
        h2d(im_d, im, sizeof(T) * (size_t)nd, c.side);
        h2d(w_d, w, sizeof(T) * (size_t)nd, c.side);
        CK(cudaEventRecord(c.ev_obs, c.side));
        CK(cudaStreamWaitEvent(s, c.ev_obs, 0));
    };
}

template <typename T> struct Api {
    using CT = C2<T>;
    using L = Launch<T>;

    static void reject_big(int N) {
        if ((long long)N * (N / 2 + 1) > (1LL << 40)) throw InvalidArg("Error: image too large");
    }

    // ---- the four user functions --------------------------------------
    static void sample_image(int nx, int ny, const T* img, T v_origin, T dRA, T dDec, T duv, T PA, int nd,
                             const T* u, const T* v, T* vis) {
        check_input(nx);  // reference sample_image :1364
        check_square(nx, ny);
        check_nd(nd);
        reject_big(nx);
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        cudaStream_t s = c.stream;
        const int N = nx;
        T* img_d = as<T>(c.img, (size_t)N * N);
        T* u_d = as<T>(c.u, (size_t)nd);
        T* v_d = as<T>(c.v, (size_t)nd);
        CT* vis_d = as<CT>(c.vis, (size_t)nd);
        DevState* st = as<DevState>(c.state, 1);
        h2d(img_d, img, sizeof(T) * (size_t)N * N, s);
        h2d(u_d, u, sizeof(T) * (size_t)nd, s);
        h2d(v_d, v, sizeof(T) * (size_t)nd, s);
        CK(cudaMemsetAsync(st, 0, sizeof(DevState), s));
        Pipe<T>::enqueue(c, s, N, (double)duv, img_d, nullptr, 0, 0, 0, 0, 0, nullptr, (double)v_origin, (double)dRA,
                         (double)dDec, (double)PA, nd, u_d, v_d, nullptr, nullptr, nullptr, vis_d, false, nullptr, st,
                         false);
        d2h(vis, vis_d, sizeof(CT) * (size_t)nd, s);
        finish(c, st);
    }

    static void chi2_image(int nx, int ny, const T* img, T v_origin, T dRA, T dDec, T duv, T PA, int nd, const T* u,
                           const T* v, const T* re, const T* im, const T* w, T* chi2) {
        check_square(nx, ny);  // reference chi2_image :1559
        check_nd(nd);
        reject_big(nx);
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        cudaStream_t s = c.stream;
        const int N = nx;
        T* img_d = as<T>(c.img, (size_t)N * N);
        T* u_d = as<T>(c.u, (size_t)nd);
        T* v_d = as<T>(c.v, (size_t)nd);
        T* re_d = as<T>(c.re, (size_t)nd);
        T* im_d = as<T>(c.im, (size_t)nd);
        T* w_d = as<T>(c.w, (size_t)nd);
        DevState* st = as<DevState>(c.state, 1);
        const auto obs = upload_obs<T>(c, s, re_d, re, im_d, im, w_d, w, nd);
        timed(c, s, ST_H2D, [&] {
            h2d(img_d, img, sizeof(T) * (size_t)N * N, s);
            h2d(u_d, u, sizeof(T) * (size_t)nd, s);
            h2d(v_d, v, sizeof(T) * (size_t)nd, s);
        });
        CK(cudaMemsetAsync(st, 0, sizeof(DevState), s));
        Pipe<T>::enqueue(c, s, N, (double)duv, img_d, nullptr, 0, 0, 0, 0, 0, nullptr, (double)v_origin, (double)dRA,
                         (double)dDec, (double)PA, nd, u_d, v_d, re_d, im_d, w_d, nullptr, true, nullptr, st, false,
                         obs);
        finish(c, st);
        *chi2 = (T)c.host_state->chi2;
    }

    static void sample_profile(int nr, const T* I, T Rmin, T dR, T dxy, int nxy, T inc, T dRA, T dDec, T duv, T PA,
                               int nd, const T* u, const T* v, T* vis) {
        check_input(nxy);  // reference sample_profile :1409
        check_nd(nd);
        reject_big(nxy);
        ProfileGeom pg = profile_geom<T>(I, nr, Rmin, dR, dxy, nxy);
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        cudaStream_t s = c.stream;
        const int N = nxy;
        T* I_d = as<T>(c.prof, (size_t)nr);
        T* u_d = as<T>(c.u, (size_t)nd);
        T* v_d = as<T>(c.v, (size_t)nd);
        CT* vis_d = as<CT>(c.vis, (size_t)nd);
        DevState* st = as<DevState>(c.state, 1);
        h2d(I_d, I, sizeof(T) * (size_t)nr, s);
        h2d(u_d, u, sizeof(T) * (size_t)nd, s);
        h2d(v_d, v, sizeof(T) * (size_t)nd, s);
        CK(cudaMemsetAsync(st, 0, sizeof(DevState), s));
        Pipe<T>::enqueue(c, s, N, (double)duv, nullptr, I_d, nr, Rmin, dR, dxy, inc, &pg, 1.0, dRA, dDec, PA, nd, u_d,
                         v_d, nullptr, nullptr, nullptr, vis_d, false, nullptr, st, false);
        d2h(vis, vis_d, sizeof(CT) * (size_t)nd, s);
        finish(c, st);
    }

    static void chi2_profile(int nr, const T* I, T Rmin, T dR, T dxy, int nxy, T inc, T dRA, T dDec, T duv, T PA,
                             int nd, const T* u, const T* v, const T* re, const T* im, const T* w, T* chi2) {
        check_input(nxy);  // reference chi2_profile :1619
        check_nd(nd);
        reject_big(nxy);
        ProfileGeom pg = profile_geom<T>(I, nr, Rmin, dR, dxy, nxy);
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        cudaStream_t s = c.stream;
        const int N = nxy;
        T* I_d = as<T>(c.prof, (size_t)nr);
        T* u_d = as<T>(c.u, (size_t)nd);
        T* v_d = as<T>(c.v, (size_t)nd);
        T* re_d = as<T>(c.re, (size_t)nd);
        T* im_d = as<T>(c.im, (size_t)nd);
        T* w_d = as<T>(c.w, (size_t)nd);
        DevState* st = as<DevState>(c.state, 1);
        // the profile first (host-to-device copies run in the order they
        // are issued, whatever their stream), then the uploads on the side
        // stream: (u, v) first so that the extent pass can start early, then
        // the observations chunk by chunk; meanwhile the row pass (which needs
        // only the profile) runs on `s`
        timed(c, s, ST_H2D, [&] { h2d(I_d, I, sizeof(T) * (size_t)nr, s); });
        CK(cudaMemsetAsync(st, 0, sizeof(DevState), s));
        if (zero_copy(c) && nd > 0) {
            // Staged schedule: the side stream's extent pass reads (u, v)
            // from the caller's arrays, writes their device copies and the
            // window; then the observations of the first visibilities are
            // copied while the row and column passes run; the visibility
            // pass reads the rest in place.  Kernel launches only: the host
            // never blocks on a pageable copy.
            Overlap ov;
            ov.ev_uv = c.ev_uv;
            ov.ev_chunk = c.ev_chunk;
            ov.staged = true;
            ov.n0 = staged_head(nd);
            ov.re0 = re_d;
            ov.im0 = im_d;
            ov.w0 = w_d;
            CK(cudaEventRecord(c.ev_side_start, s));
            CK(cudaStreamWaitEvent(c.side, c.ev_side_start, 0));
            const bool pinned = is_pinned(u) && is_pinned(v) && is_pinned(re) && is_pinned(im) && is_pinned(w);
            if (pinned) {
                // copy engines: the SMs stay free for the row pass
                h2d(u_d, u, sizeof(T) * (size_t)nd, c.side);
                h2d(v_d, v, sizeof(T) * (size_t)nd, c.side);
                CK(cudaEventRecord(c.ev_uv, c.side));
                h2d(re_d, re, sizeof(T) * (size_t)ov.n0, c.side);
                h2d(im_d, im, sizeof(T) * (size_t)ov.n0, c.side);
                h2d(w_d, w, sizeof(T) * (size_t)ov.n0, c.side);
            } else {
                // a pageable copy would block the host: kernels read the arrays
                CK(L::extent(u, v, nd, N, (double)duv, st, c.side, u_d, v_d));
                CK(cudaEventRecord(c.ev_uv, c.side));
                ov.extent_done = true;
                CK(L::stage3(re, im, w, re_d, im_d, w_d, ov.n0, c.side));
            }
            CK(cudaEventRecord(c.ev_chunk[0], c.side));
            Pipe<T>::enqueue(c, s, N, (double)duv, nullptr, I_d, nr, Rmin, dR, dxy, inc, &pg, 1.0, dRA, dDec, PA, nd,
                             u_d, v_d, re, im, w, nullptr, true, nullptr, st, false, std::function<void()>(), &ov);
            finish(c, st);
            *chi2 = (T)c.host_state->chi2;
            return;
        }
        Overlap ov;
        ov.ev_uv = c.ev_uv;
        ov.nchunks = std::max(1, std::min(Ctx::kMaxChunks, nd >> 18));
        ov.ev_chunk = c.ev_chunk;
        CK(cudaEventRecord(c.ev_side_start, s));
        CK(cudaStreamWaitEvent(c.side, c.ev_side_start, 0));
        h2d(u_d, u, sizeof(T) * (size_t)nd, c.side);
        h2d(v_d, v, sizeof(T) * (size_t)nd, c.side);
        CK(cudaEventRecord(c.ev_uv, c.side));
        for (int k = 0; k < ov.nchunks; ++k) {
            const size_t b0 = (size_t)chunk_begin(nd, ov.nchunks, k), n = (size_t)chunk_begin(nd, ov.nchunks, k + 1) - b0;
            h2d(re_d + b0, re + b0, sizeof(T) * n, c.side);
            h2d(im_d + b0, im + b0, sizeof(T) * n, c.side);
            h2d(w_d + b0, w + b0, sizeof(T) * n, c.side);
            CK(cudaEventRecord(c.ev_chunk[k], c.side));
        }
        Pipe<T>::enqueue(c, s, N, (double)duv, nullptr, I_d, nr, Rmin, dR, dxy, inc, &pg, 1.0, dRA, dDec, PA, nd, u_d,
                         v_d, re_d, im_d, w_d, nullptr, true, nullptr, st, false, std::function<void()>(), &ov);
        finish(c, st);
        *chi2 = (T)c.host_state->chi2;
    }

    // ---- device-resident variants (no host copies, no synchronisation) ----
    static void chi2_profile_device(int nr, const T* I_host, const T* I_d, T Rmin, T dR, T dxy, int nxy, T inc,
                                    T dRA, T dDec, T duv, T PA, int nd, const T* u_d, const T* v_d, const T* re_d,
                                    const T* im_d, const T* w_d, double* chi2_d, cudaStream_t s) {
        check_input(nxy);
        check_nd(nd);
        ProfileGeom pg = profile_geom<T>(I_host, nr, Rmin, dR, dxy, nxy);
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        DevState* st = as<DevState>(c.state, 1);
        CK(cudaMemsetAsync(st, 0, sizeof(DevState), s));
        Pipe<T>::enqueue(c, s, nxy, (double)duv, nullptr, I_d, nr, Rmin, dR, dxy, inc, &pg, 1.0, dRA, dDec, PA, nd,
                         u_d, v_d, re_d, im_d, w_d, nullptr, true, chi2_d, st, false);
    }

    static void chi2_image_device(int nx, int ny, const T* img_d, T v_origin, T dRA, T dDec, T duv, T PA, int nd,
                                  const T* u_d, const T* v_d, const T* re_d, const T* im_d, const T* w_d,
                                  double* chi2_d, cudaStream_t s) {
        check_square(nx, ny);
        check_nd(nd);
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        DevState* st = as<DevState>(c.state, 1);
        CK(cudaMemsetAsync(st, 0, sizeof(DevState), s));
        Pipe<T>::enqueue(c, s, nx, (double)duv, img_d, nullptr, 0, 0, 0, 0, 0, nullptr, (double)v_origin, dRA, dDec,
                         PA, nd, u_d, v_d, re_d, im_d, w_d, nullptr, true, chi2_d, st, false);
    }

    // ---- expert stages -------------------------------------------------
    static void sweep(int nr, const T* I, T Rmin, T dR, int nxy, T dxy, T inc, T* image_padded) {
        check_input(nxy);
        reject_big(nxy);
        ProfileGeom pg = profile_geom<T>(I, nr, Rmin, dR, dxy, nxy);
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        cudaStream_t s = c.stream;
        const size_t nreal = (size_t)nxy * 2 * (size_t)(nxy / 2 + 1);
        T* buf = as<T>(c.img, nreal);
        T* I_d = as<T>(c.prof, (size_t)nr);
        h2d(I_d, I, sizeof(T) * (size_t)nr, s);
        CK(cudaMemsetAsync(buf, 0, sizeof(T) * nreal, s));
        CK(L::sweep_image(I_d, nr, Rmin, dR, dxy, std::cos((double)inc), pg.rmax, pg.central, nxy, buf, s));
        d2h(image_padded, buf, sizeof(T) * nreal, s);
        CK(cudaStreamSynchronize(s));
    }

    static void uv_rotate(T PA, T dRA, T dDec, T* dRArot, T* dDecrot, int nd, const T* u, const T* v, T* urot,
                          T* vrot) {
        check_nd(nd);
        if (PA == 0) {  // reference :1294-1299
            *dRArot = dRA;
            *dDecrot = dDec;
            if (nd) {
                std::memmove(urot, u, sizeof(T) * (size_t)nd);
                std::memmove(vrot, v, sizeof(T) * (size_t)nd);
            }
            return;
        }
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        cudaStream_t s = c.stream;
        const double cs = std::cos((double)PA), sn = std::sin((double)PA);
        T* u_d = as<T>(c.u, (size_t)nd);
        T* v_d = as<T>(c.v, (size_t)nd);
        T* ur_d = as<T>(c.urot, (size_t)nd);
        T* vr_d = as<T>(c.vrot, (size_t)nd);
        h2d(u_d, u, sizeof(T) * (size_t)nd, s);
        h2d(v_d, v, sizeof(T) * (size_t)nd, s);
        CK(L::rotate(u_d, v_d, ur_d, vr_d, nd, cs, sn, s));
        d2h(urot, ur_d, sizeof(T) * (size_t)nd, s);
        d2h(vrot, vr_d, sizeof(T) * (size_t)nd, s);
        CK(cudaStreamSynchronize(s));
        *dRArot = (T)((double)dRA * cs - (double)dDec * sn);
        *dDecrot = (T)((double)dRA * sn + (double)dDec * cs);
    }

    static void interpolate(int nrow, int ncol, const T* data, T v_origin, int nd, const T* u, const T* v, T duv,
                            T* vis) {
        check_nd(nd);
        if (nrow < 2 || ncol < 2) throw InvalidArg("Error in interpolate: the spectrum must be at least 2 x 2");
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        cudaStream_t s = c.stream;
        CT* spec = as<CT>(c.win, (size_t)nrow * ncol);
        T* u_d = as<T>(c.u, (size_t)nd);
        T* v_d = as<T>(c.v, (size_t)nd);
        CT* vis_d = as<CT>(c.vis, (size_t)nd);
        DevState* st = as<DevState>(c.state, 1);
        h2d(spec, data, sizeof(CT) * (size_t)nrow * ncol, s);
        h2d(u_d, u, sizeof(T) * (size_t)nd, s);
        h2d(v_d, v, sizeof(T) * (size_t)nd, s);
        CK(cudaMemsetAsync(st, 0, sizeof(DevState), s));
        typename L::VisArgs a;
        a.spec = spec;
        a.amp = nullptr;
        a.quads = nullptr;
        a.quad_cap = 0;
        a.phase_tab = c.phase_tab;
        a.s_row = ncol;
        a.s_col = 1;
        a.nrow = nrow;
        a.ncol = ncol;
        a.host_K = ncol;
        a.host_r0 = 0;
        a.host_W = nrow;
        a.duv = (double)duv;
        a.v_origin = (double)v_origin;
        a.rotate = false;
        a.cos_pa = 1.;
        a.sin_pa = 0.;
        a.dra = a.ddec = 0.;
        a.phase = false;
        a.u = u_d;
        a.v = v_d;
        a.re = a.im = a.w = nullptr;
        a.nd = nd;
        a.vis_out = vis_d;
        a.partials = nullptr;
        a.chi2_out = nullptr;
        a.state = st;
        if (nd > 0) CK(L::vis(a, s));
        d2h(vis, vis_d, sizeof(CT) * (size_t)nd, s);
        finish(c, st);
    }

    static void apply_phase(T dRA, T dDec, int nd, const T* u, const T* v, T* vis) {
        check_nd(nd);
        if (dRA == 0 && dDec == 0) return;  // reference :890-892
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        cudaStream_t s = c.stream;
        T* u_d = as<T>(c.u, (size_t)nd);
        T* v_d = as<T>(c.v, (size_t)nd);
        CT* vis_d = as<CT>(c.vis, (size_t)nd);
        h2d(u_d, u, sizeof(T) * (size_t)nd, s);
        h2d(v_d, v, sizeof(T) * (size_t)nd, s);
        h2d(vis_d, vis, sizeof(CT) * (size_t)nd, s);
        CK(L::apply_phase(u_d, v_d, vis_d, nd, (double)dRA, (double)dDec, s));
        d2h(vis, vis_d, sizeof(CT) * (size_t)nd, s);
        CK(cudaStreamSynchronize(s));
    }

    static void reduce_chi2(int nd, const T* re, const T* im, const T* vis, const T* w, T* chi2) {
        check_nd(nd);
        if (nd == 0) {
            *chi2 = 0;
            return;
        }
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        cudaStream_t s = c.stream;
        T* re_d = as<T>(c.re, (size_t)nd);
        T* im_d = as<T>(c.im, (size_t)nd);
        T* w_d = as<T>(c.w, (size_t)nd);
        CT* vis_d = as<CT>(c.vis, (size_t)nd);
        double* partials = as<double>(c.partials, (size_t)L::vis_grid(nd));
        DevState* st = as<DevState>(c.state, 1);
        h2d(re_d, re, sizeof(T) * (size_t)nd, s);
        h2d(im_d, im, sizeof(T) * (size_t)nd, s);
        h2d(w_d, w, sizeof(T) * (size_t)nd, s);
        h2d(vis_d, vis, sizeof(CT) * (size_t)nd, s);
        CK(cudaMemsetAsync(st, 0, sizeof(DevState), s));
        CK(L::reduce(re_d, im_d, vis_d, w_d, nd, partials, st, s));
        finish(c, st);
        *chi2 = (T)c.host_state->chi2;
    }

    // in-place R2C of the padded layout (reference fft2d :531-541, _copy_input :460-487)
    static void fft2d(int nx, int ny, T* data) {
        check_square(nx, ny);
        reject_big(nx);
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        cudaStream_t s = c.stream;
        const int N = nx, C = N / 2 + 1;
        T* img_d = as<T>(c.img, (size_t)N * N);
        CT* zt = as<CT>(c.zt, (size_t)C * N);
        CT* out = as<CT>(c.win, (size_t)C * N);
        DevState* st = as<DevState>(c.state, 1);
        CK(cudaMemcpy2DAsync(img_d, sizeof(T) * N, data, sizeof(T) * 2 * C, sizeof(T) * N, N, cudaMemcpyHostToDevice,
                             s));
        const CT* tw = c.twiddles<T>(N);
        CK(L::rows_image(img_d, N, tw, c.stage_tw<T>(N / 2), zt, C, st, 1.0, false, s));
        CK(L::cols(zt, N, 0, N, tw, c.stage_tw<T>(N), out, nullptr, C, 1, C, 0, N, st, 1.0, false, s));
        d2h(data, out, sizeof(CT) * (size_t)N * C, s);
        CK(cudaStreamSynchronize(s));
    }

    static void fftshift(int nx, int ny, T* data) {
        check_square(nx, ny);
        reject_big(nx);
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        cudaStream_t s = c.stream;
        const size_t nreal = (size_t)nx * 2 * (size_t)(ny / 2 + 1);
        T* buf = as<T>(c.img, nreal);
        h2d(buf, data, sizeof(T) * nreal, s);
        CK(L::fftshift_real(buf, nx, s));
        d2h(data, buf, sizeof(T) * nreal, s);
        CK(cudaStreamSynchronize(s));
    }

    static void fftshift_axis0(int nrow, int ncol, T* data) {
        check_input(nrow);
        Ctx& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        cudaStream_t s = c.stream;
        const size_t n = (size_t)nrow * ncol;
        CT* buf = as<CT>(c.win, n);
        h2d(buf, data, sizeof(CT) * n, s);
        CK(L::fftshift_axis0(buf, nrow, ncol, s));
        d2h(data, buf, sizeof(CT) * n, s);
        CK(cudaStreamSynchronize(s));
    }
};

}  // namespace
}  // namespace gbg

namespace gbg {
// message for galario_last_error() from entry points defined in other translation units
void set_error_message(const std::string& msg) { g_msg = msg; }
}  // namespace gbg

using gbg::Api;
using gbg::guarded;

#define API extern "C" __attribute__((visibility("default")))

API const char* galario_last_error(void) { return gbg::g_msg.c_str(); }
API const char* galario_version(void) { return "galario_gb300 0.1.0 (reference API galario 1.2.2)"; }

API int galario_threads(int num) {
    if (num > 0) gbg::g_tpb = num;
    return gbg::g_tpb;
}
API int galario_ngpus(int* out) {
    return guarded([&] {
        int n = 0;
        gbg::cuda_check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        *out = n;
    });
}
API int galario_use_gpu(int device_id) {
    return guarded([&] { gbg::cuda_check(cudaSetDevice(device_id), "cudaSetDevice"); });
}
API int galario_init(void) {
    return guarded([&] { (void)gbg::ctx(); });
}
API int galario_cleanup(void) {
    return guarded([&] {
        gbg::noalloc_forget_scratch();
        std::lock_guard<std::mutex> lk(gbg::g_ctx_mu);
        for (auto& kv : gbg::g_ctx) {
            std::lock_guard<std::mutex> l2(kv.second->mu);
            int cur = 0;
            cudaGetDevice(&cur);
            cudaSetDevice(kv.first);
            cudaStreamSynchronize(kv.second->stream);
            kv.second->release_all();
            cudaSetDevice(cur);
        }
    });
}

// precision-specific entry points, generated for double (_d) and float (_f)
#define GALARIO_DEFINE(R, SFX)                                                                                        \
    API int galario_sample_image##SFX(int nx, int ny, const R* image, R v_origin, R dRA, R dDec, R duv, R PA, int nd, \
                                      const R* u, const R* v, R* vis) {                                               \
        return guarded([&] { Api<R>::sample_image(nx, ny, image, v_origin, dRA, dDec, duv, PA, nd, u, v, vis); });   \
    }                                                                                                                 \
    API int galario_chi2_image##SFX(int nx, int ny, const R* image, R v_origin, R dRA, R dDec, R duv, R PA, int nd,   \
                                    const R* u, const R* v, const R* re, const R* im, const R* w, R* chi2) {          \
        return guarded(                                                                                               \
            [&] { Api<R>::chi2_image(nx, ny, image, v_origin, dRA, dDec, duv, PA, nd, u, v, re, im, w, chi2); });     \
    }                                                                                                                 \
    API int galario_sample_profile##SFX(int nr, const R* intensity, R Rmin, R dR, R dxy, int nxy, R inc, R dRA,       \
                                        R dDec, R duv, R PA, int nd, const R* u, const R* v, R* vis) {                \
        return guarded([&] {                                                                                          \
            Api<R>::sample_profile(nr, intensity, Rmin, dR, dxy, nxy, inc, dRA, dDec, duv, PA, nd, u, v, vis);        \
        });                                                                                                           \
    }                                                                                                                 \
    API int galario_chi2_profile##SFX(int nr, const R* intensity, R Rmin, R dR, R dxy, int nxy, R inc, R dRA, R dDec, \
                                      R duv, R PA, int nd, const R* u, const R* v, const R* re, const R* im,          \
                                      const R* w, R* chi2) {                                                          \
        return guarded([&] {                                                                                          \
            Api<R>::chi2_profile(nr, intensity, Rmin, dR, dxy, nxy, inc, dRA, dDec, duv, PA, nd, u, v, re, im, w,     \
                                 chi2);                                                                               \
        });                                                                                                           \
    }                                                                                                                 \
    API int galario_chi2_profile_device##SFX(int nr, const R* intensity_host, const R* intensity_dev, R Rmin, R dR,   \
                                             R dxy, int nxy, R inc, R dRA, R dDec, R duv, R PA, int nd,               \
                                             const R* u_dev, const R* v_dev, const R* re_dev, const R* im_dev,        \
                                             const R* w_dev, double* chi2_dev, void* stream) {                        \
        return guarded([&] {                                                                                          \
            Api<R>::chi2_profile_device(nr, intensity_host, intensity_dev, Rmin, dR, dxy, nxy, inc, dRA, dDec, duv,   \
                                        PA, nd, u_dev, v_dev, re_dev, im_dev, w_dev, chi2_dev,                        \
                                        static_cast<cudaStream_t>(stream));                                          \
        });                                                                                                           \
    }                                                                                                                 \
    API int galario_chi2_image_device##SFX(int nx, int ny, const R* image_dev, R v_origin, R dRA, R dDec, R duv,      \
                                           R PA, int nd, const R* u_dev, const R* v_dev, const R* re_dev,             \
                                           const R* im_dev, const R* w_dev, double* chi2_dev, void* stream) {         \
        return guarded([&] {                                                                                          \
            Api<R>::chi2_image_device(nx, ny, image_dev, v_origin, dRA, dDec, duv, PA, nd, u_dev, v_dev, re_dev,      \
                                      im_dev, w_dev, chi2_dev, static_cast<cudaStream_t>(stream));                    \
        });                                                                                                           \
    }                                                                                                                 \
    API int galario_sweep##SFX(int nr, const R* intensity, R Rmin, R dR, int nxy, R dxy, R inc, R* image) {           \
        return guarded([&] { Api<R>::sweep(nr, intensity, Rmin, dR, nxy, dxy, inc, image); });                       \
    }                                                                                                                 \
    API int galario_uv_rotate##SFX(R PA, R dRA, R dDec, R* dRArot, R* dDecrot, int nd, const R* u, const R* v,        \
                                   R* urot, R* vrot) {                                                                \
        return guarded([&] { Api<R>::uv_rotate(PA, dRA, dDec, dRArot, dDecrot, nd, u, v, urot, vrot); });            \
    }                                                                                                                 \
    API int galario_interpolate##SFX(int nrow, int ncol, const R* data, R v_origin, int nd, const R* u, const R* v,   \
                                     R duv, R* vis) {                                                                 \
        return guarded([&] { Api<R>::interpolate(nrow, ncol, data, v_origin, nd, u, v, duv, vis); });                \
    }                                                                                                                 \
    API int galario_apply_phase_sampled##SFX(R dRA, R dDec, int nd, const R* u, const R* v, R* vis) {                \
        return guarded([&] { Api<R>::apply_phase(dRA, dDec, nd, u, v, vis); });                                      \
    }                                                                                                                 \
    API int galario_reduce_chi2##SFX(int nd, const R* re, const R* im, const R* vis, const R* w, R* chi2) {           \
        return guarded([&] { Api<R>::reduce_chi2(nd, re, im, vis, w, chi2); });                                      \
    }                                                                                                                 \
    API int galario_fft2d##SFX(int nx, int ny, R* data) {                                                             \
        return guarded([&] { Api<R>::fft2d(nx, ny, data); });                                                        \
    }                                                                                                                 \
    API int galario_fftshift##SFX(int nx, int ny, R* data) {                                                          \
        return guarded([&] { Api<R>::fftshift(nx, ny, data); });                                                     \
    }                                                                                                                 \
    API int galario_fftshift_axis0##SFX(int nrow, int ncol, R* data) {                                                \
        return guarded([&] { Api<R>::fftshift_axis0(nrow, ncol, data); });                                           \
    }

GALARIO_DEFINE(double, _d)
GALARIO_DEFINE(float, _f)

API int galario_stage_timing(int enable) {
    return guarded([&] {
        gbg::Ctx& c = gbg::ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        c.timing = enable != 0;
    });
}
API const char* galario_stage_name(int stage) {
    return (stage >= 0 && stage < gbg::ST_COUNT) ? gbg::kStageNames[stage] : "";
}
API int galario_stage_times(double* ms_sum, int* count, int nstages) {
    return guarded([&] {
        gbg::Ctx& c = gbg::ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        for (int i = 0; i < nstages; ++i) {
            ms_sum[i] = 0.;
            count[i] = 0;
        }
        for (auto& r : c.recs) {
            gbg::cuda_check(cudaEventSynchronize(r.b), "cudaEventSynchronize");
            float ms = 0.f;
            gbg::cuda_check(cudaEventElapsedTime(&ms, r.a, r.b), "cudaEventElapsedTime");
            if (r.stage < nstages) {
                ms_sum[r.stage] += ms;
                count[r.stage] += 1;
            }
            c.spare.push_back(r.a);
            c.spare.push_back(r.b);
        }
        c.recs.clear();
    });
}

API int galario_device_status(unsigned int* err_bits) {
    return guarded([&] {
        gbg::Ctx& c = gbg::ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        gbg::DevState* st = gbg::as<gbg::DevState>(c.state, 1);
        gbg::d2h(c.host_state, st, sizeof(gbg::DevState), c.stream);
        gbg::cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
        *err_bits = c.host_state->err;
    });
}
