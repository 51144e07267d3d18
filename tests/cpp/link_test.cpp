// Include, link and run galario_gb300 from plain C++ through the galario
// namespace facade (include/galario_gb300.hpp), as a program written against
// the reference's src/galario.h would (the reference's own check of this is
// src/galario_test.cpp).  Build with -DGALARIO_DOUBLE_PRECISION for doubles.
//
// Part 1 calls every function of the API once on valid inputs (compile, link
// and const-correctness check).  Part 2 evaluates chi2_profile, chi2_image and
// sample_profile on deterministic inputs and prints them with full precision;
// the Python test recomputes the same inputs and compares with the oracle.
#include "galario_gb300.hpp"

#include <cassert>
#include <cmath>
#include <cstdio>
#include <vector>

using namespace galario;

int main() {
    init();
    const int nx = 128, ny = nx;
    const dreal dxy = (dreal)(0.05 * 4.84813681109536e-06);

    // ---- part 1: every entry point once ----
    std::vector<dreal> real(nx * ny, (dreal)0);
    dcomplex* buf = copy_input(nx, ny, real.data());
    const int n = 4;
    std::vector<dreal> a(16, (dreal)0.5), b(16, (dreal)0.25), c(16), d(16);
    dreal dra = 0, ddec = 0;
    sweep(nx, real.data(), dxy / 100, dxy / (dreal)10.5, nx, dxy, (dreal)0.5, buf);
    uv_rotate((dreal)0.3, (dreal)1e-7, (dreal)2e-7, &dra, &ddec, n, a.data(), b.data(), c.data(), d.data());
    fft2d(nx, ny, buf);
    fftshift(n, n, buf);
    fftshift_axis0(n, n, buf);
    std::vector<dcomplex> vis4(n);
    const int ncomplex = nx * (ny / 2 + 1);
    std::vector<dcomplex> spectrum(buf, buf + ncomplex);
    interpolate(nx, ny / 2 + 1, spectrum.data(), (dreal)1, n, a.data(), b.data(), (dreal)0.25, vis4.data());
    apply_phase_sampled(dra, ddec, n, a.data(), b.data(), vis4.data());
    const dreal chi0 = reduce_chi2(n, a.data(), b.data(), vis4.data(), a.data());
    (void)chi0;
    for (int i = 0; i < ncomplex; ++i) assert(spectrum[i] == buf[i]);  // inputs are not modified
    galario_free(buf);
    assert(ngpus() >= 1);
    (void)threads();

    // ---- part 2: deterministic problem ----
    const int nr = 300, nd = 2000, nxy = 128;
    const dreal Rmin = dxy / 50, dR = dxy / 12, duv = (dreal)(1.0 / (nxy * (double)dxy));
    std::vector<dreal> I(nr), u(nd), v(nd), re(nd), im(nd), w(nd), img(nxy * nxy);
    for (int i = 0; i < nr; ++i) {
        const double R = Rmin + i * (double)dR, r0 = 20 * (double)dxy, s = 6 * (double)dxy;
        I[i] = (dreal)(1e10 * std::exp(-0.5 * (R - r0) * (R - r0) / (s * s)));
    }
    for (int k = 0; k < nd; ++k) {
        const double r = (double)duv * (1.0 + 40.0 * k / nd), th = 2.399963229728653 * k;
        u[k] = (dreal)(r * std::cos(th));
        v[k] = (dreal)(r * std::sin(th));
        re[k] = (dreal)(1e-3 * std::sin(0.1 * k));
        im[k] = (dreal)(1e-3 * std::cos(0.07 * k));
        w[k] = (dreal)(1e6 * (1 + k % 7));
    }
    for (int i = 0; i < nxy; ++i)
        for (int j = 0; j < nxy; ++j) {
            const double x = j - nxy / 2 + 3, y = i - nxy / 2 - 5;
            img[i * nxy + j] = (dreal)(1e-3 * std::exp(-(x * x) / 200.0 - (y * y) / 90.0));
        }
    const dreal inc = (dreal)0.6, PA = (dreal)1.1, dRA = (dreal)(0.1 * 4.84813681109536e-06),
                dDec = (dreal)(-0.2 * 4.84813681109536e-06);
    const dreal chi2p = chi2_profile(nr, I.data(), Rmin, dR, dxy, nxy, inc, dRA, dDec, duv, PA, nd, u.data(), v.data(),
                                     re.data(), im.data(), w.data());
    const dreal chi2i = chi2_image(nxy, nxy, img.data(), (dreal)1, dRA, dDec, duv, PA, nd, u.data(), v.data(),
                                   re.data(), im.data(), w.data());
    std::vector<dcomplex> vis(nd);
    sample_profile(nr, I.data(), Rmin, dR, dxy, nxy, inc, dRA, dDec, duv, PA, nd, u.data(), v.data(), vis.data());
    std::printf("chi2_profile %.17g\nchi2_image %.17g\nvis0 %.17g %.17g\nvis%d %.17g %.17g\n", (double)chi2p,
                (double)chi2i, (double)vis[0].real(), (double)vis[0].imag(), nd - 1, (double)vis[nd - 1].real(),
                (double)vis[nd - 1].imag());

    // errors come back as the reference's exception types
    bool raised = false;
    try {
        (void)chi2_profile(nr, I.data(), Rmin, dxy, dxy, nxy, inc, dRA, dDec, duv, PA, nd, u.data(), v.data(),
                           re.data(), im.data(), w.data());
    } catch (const std::invalid_argument&) {
        raised = true;
    }
    std::printf("invalid_argument %d\n", raised ? 1 : 0);
    cleanup();
    return raised ? 0 : 1;
}
