"""The spectrum window of a swept profile as two products with fixed cosine
matrices, checked on the CPU against the oracle's sweep -> fftshift -> R2C FFT
-> fftshift_axis0 chain (the reference's pipeline).

A swept image is even in x and y about pixel (N/2, N/2), so with f(a, c) its
quadrant (a = |y|, c = |x| in pixels, 0 <= a, c <= n = N/2), w_0 = w_n = 1 and
w_j = 2 otherwise, the shifted spectrum is real and

    S[r][k] = sum_a w_a cos(2 pi a |r - N/2| / N) sum_c w_c cos(2 pi c k / N) f(a, c),

i.e. S = Cv F Ck^T.  The row and column passes of the FP64 profile path
compute exactly these two even transforms (as DCT-Is from quarter-length
FFTs); for B models sharing a geometry the cosine matrices are common to all
models, which makes the batched passes dense products.
"""
import numpy as np
import pytest

from helpers import arcsec


@pytest.mark.parametrize("nxy,inc", [(64, 0.0), (256, 0.6)])
def test_window_is_two_cosine_products(oracle_port, nxy, inc):
    orc = oracle_port.get("port", "double")
    dxy = 0.05 * arcsec
    Rmin, dR, nr = 1e-4 * arcsec, 2e-3 * arcsec, 1500
    R = Rmin + dR * np.arange(nr)
    I = 1e10 * (np.exp(-0.5 * ((R - 0.6 * arcsec) / (0.1 * arcsec)) ** 2) + 0.3 * np.exp(-0.5 * (R / (0.3 * arcsec)) ** 2))
    img = orc.sweep(I, Rmin, dR, nxy, dxy, inc)
    N, n = nxy, nxy // 2
    # the reference's spectrum: fftshift_axis0(rfft2(fftshift(image)))
    shifted = orc._fftshift(img)
    spec = orc._fft2d(np.ascontiguousarray(shifted.view(np.float64)[:, :N]))
    orc._fftshift_axis0(spec)
    # the quadrant of the swept image, evenness checked
    F = np.empty((n + 1, n + 1))
    for a in range(n + 1):
        for c in range(n + 1):
            F[a, c] = img[(N // 2 - a) % N, (N // 2 - c) % N]
    assert np.array_equal(img[N // 2 - 1, N // 2 - 3], img[N // 2 + 1, N // 2 + 3])
    w = np.full(n + 1, 2.0)
    w[0] = w[n] = 1.0
    j = np.arange(n + 1)
    k = np.arange(n + 1)
    Ck = w[None, :] * np.cos(2 * np.pi * np.outer(k, j) / N)          # (k, c)
    r = np.arange(N)
    Cv = w[None, :] * np.cos(2 * np.pi * np.outer(np.abs(r - N // 2), j) / N)  # (r, a)
    S = Cv @ F @ Ck.T
    scale = np.abs(spec).max()
    assert np.abs(spec.imag).max() <= 1e-12 * scale  # real up to rounding
    assert np.abs(S - spec.real).max() <= 1e-12 * scale


def test_mirror_folded_products_equal_the_full_window():
    """The second product over the T1 distinct distances t = |r - N/2| of the
    window rows, written to rows N/2 - t and N/2 + t, equals the product over
    all W window rows; and its adjoint over the folded window gradient
    G'[k][t] = G[k][N/2 - t] + G[k][N/2 + t] (the rows inside the window)
    equals the adjoint over the full gradient (the batched tensor-core passes,
    gb_batch.cu)."""
    rng = np.random.default_rng(7)
    N, nF, K = 256, 40, 30
    r0, W = N // 2 - 50, 97            # window rows [r0, r0 + W), not symmetric about N/2
    h0 = N // 2 - r0
    T1 = max(N // 2 - r0, r0 + W - 1 - N // 2) + 1
    w = np.where(np.arange(nF) == 0, 1.0, 2.0)
    C = lambda t: w[None, :] * np.cos(2 * np.pi * np.outer(t, np.arange(nF)) / N)  # noqa: E731
    D1 = rng.standard_normal((K, nF))
    rows = np.abs(r0 + np.arange(W) - N // 2)
    S_full = D1 @ C(rows).T                        # K x W
    Sp = D1 @ C(np.arange(T1)).T                   # K x T1
    S_mirror = np.empty((K, W))
    for t in range(T1):
        for q in (h0 - t, h0 + t):
            if 0 <= q < W:
                S_mirror[:, q] = Sp[:, t]
    assert np.allclose(S_mirror, S_full, rtol=0, atol=1e-12 * np.abs(S_full).max())
    G = rng.standard_normal((K, W))
    Gp = np.zeros((K, T1))
    for t in range(T1):
        for q in sorted({h0 - t, h0 + t}):
            if 0 <= q < W:
                Gp[:, t] += G[:, q]
    adj_full = G @ C(rows)                         # K x nF
    adj_fold = Gp @ C(np.arange(T1))
    assert np.allclose(adj_fold, adj_full, rtol=0, atol=1e-12 * np.abs(adj_full).max())
