"""CPU restatement (numpy, integer arithmetic) of the FP64-grade digit products
of the FP64 profile path (galario_gb300/csrc/gb_ozaki.cuh, gb_profile_tc.cu).

- digits8: every value of a row relative to the row exponent e (|x| < 2^e)
  as eight balanced base-128 digits, x = 2^e sum_i d_i 2^(-6-7i) to within
  2^(e-56), |d_i| <= 64;
- the level sums lev_L = sum_{i+j=L} d^a_i . d^b_j over one K tile of 64,
  and the epilogue's fold of the eight levels into one integer in units of
  2^-35 (levels 6 and 7 rounded, half up), summed over the K tiles;
- a product A B^T from those sums against an exact (rational) product;
- the swept profile's spectrum window from the two transposed products
  (D1^T = F C^T, S'^T = C D1^T) against the oracle's FFT pipeline.

The GPU test (tests/test_gpu_ozaki.py) checks the tensor-core kernel's sums
bit for bit against the same integer arithmetic.
"""
import math
from fractions import Fraction

import numpy as np
import pytest

from helpers import arcsec

PLANES, LEVELS, BK = 8, 8, 64


def row_exponent(amax):
    """Smallest e with amax < 2^e (0 for a zero row)."""
    if not amax > 0:
        return 0
    return math.frexp(amax)[1]


def digits8(x, e):
    """Digits d[0..7] (int64) of the values x relative to 2^e, |x| < 2^e."""
    v = np.abs(x) * 2.0 ** (55 - e)           # exact: a power-of-two scaling, below 2^55
    fl = np.floor(v)
    X = (fl + (v - fl >= 0.5)).astype(np.int64)  # round half up on the magnitude
    d = np.zeros((PLANES,) + np.shape(x), dtype=np.int64)
    for i in range(PLANES - 1, 0, -1):
        q = X & 127
        q = np.where(q >= 64, q - 128, q)
        d[i] = q
        X = (X - q) >> 7
    d[0] = X
    return np.where(np.asarray(x) < 0, -d, d)


def split_rows(M):
    """Digit planes (8, rows, K) and row exponents of a matrix."""
    ex = np.array([row_exponent(float(np.abs(r).max())) for r in M])
    D = np.stack([digits8(M[r], ex[r]) for r in range(M.shape[0])], axis=1)
    return D, ex


def fold_levels(lev):
    """The epilogue's integer V of one K tile from its eight levels."""
    v = np.zeros_like(lev[0])
    for L in range(6):
        v = v * 128 + lev[L]
    tail = lev[6] * 128 + lev[7]
    return v + ((tail + 8192) >> 14)


def digit_product(A, B):
    """A B^T (M x N) in FP64 through the digit scheme, as the kernels do."""
    Da, ea = split_rows(A)
    Db, eb = split_rows(B)
    K = A.shape[1]
    V = np.zeros((A.shape[0], B.shape[0]), dtype=np.int64)
    for k0 in range(0, K, BK):
        sl = slice(k0, min(K, k0 + BK))
        lev = np.zeros((LEVELS,) + V.shape, dtype=np.int64)
        for i in range(PLANES):
            for j in range(PLANES - i):
                lev[i + j] += Da[i][:, sl] @ Db[j][:, sl].T
        assert np.abs(lev).max() < 2 ** 21  # exact in FP32 (tensor-core accumulation)
        V += fold_levels(lev)
    assert np.abs(V).max() < 2 ** 62
    scale = np.ldexp(1.0, (ea[:, None] + eb[None, :] - 12 - 35).astype(np.int64))
    return V.astype(np.float64) * scale


def test_digits_reconstruct_values():
    rng = np.random.default_rng(1)
    for sc in (1e-30, 1e-3, 1.0, 7.5e12):
        x = sc * rng.standard_normal(300) * np.exp(-rng.uniform(0, 30, 300))
        x[:3] = [0.0, sc, -sc]
        e = row_exponent(float(np.abs(x).max()))
        d = digits8(x, e)
        assert np.abs(d).max() <= 64
        rec = [sum(Fraction(int(d[i][k])) * Fraction(2) ** (e - 6 - 7 * i) for i in range(PLANES)) for k in range(len(x))]
        err = max(abs(Fraction(float(x[k])) - rec[k]) for k in range(len(x)))
        assert err <= Fraction(2) ** (e - 56)


def test_fold_is_the_level_sum_to_2_pow_minus_36():
    rng = np.random.default_rng(2)
    lev = rng.integers(-2 ** 21, 2 ** 21, size=(LEVELS, 5000))
    v = fold_levels(lev)
    for k in range(0, 5000, 97):
        exact = sum(Fraction(int(lev[L][k])) * Fraction(2) ** (35 - 7 * L) for L in range(LEVELS))
        assert abs(Fraction(int(v[k])) - exact) <= Fraction(1, 2)


@pytest.mark.parametrize("M,N,K", [(37, 5, 9), (70, 50, 343), (40, 30, 700)])
def test_digit_product_against_exact(M, N, K):
    rng = np.random.default_rng(M + N + K)
    A = rng.uniform(-1, 1, (M, K)) * np.ldexp(1.0, rng.integers(-40, 40, (M, 1))) * np.ldexp(1.0, -rng.integers(0, 30, (M, K)))
    B = rng.uniform(-1, 1, (N, K)) * np.ldexp(1.0, rng.integers(-40, 40, (N, 1))) * np.ldexp(1.0, -rng.integers(0, 30, (N, K)))
    got = digit_product(A, B)
    for m in range(0, M, 7):
        for n in range(0, N, 3):
            exact = sum(Fraction(float(A[m, k])) * Fraction(float(B[n, k])) for k in range(K))
            bound = K * float(np.abs(A[m]).max()) * float(np.abs(B[n]).max())
            assert abs(float(Fraction(float(got[m, n])) - exact)) <= 2.0 ** -50 * bound


def test_profile_window_from_two_digit_products(oracle_port):
    """The window of a swept profile, S[r][k] = sum_a C[|r-N/2|][a] sum_c C[k][c] F[a][c],
    through the transposed digit products, against the oracle's
    fftshift -> R2C FFT -> fftshift_axis0 of the swept image."""
    orc = oracle_port.get("port", "double")
    nxy, dxy, inc = 128, 0.05 * arcsec, 0.5
    Rmin, dR, nr = 1e-4 * arcsec, 2e-3 * arcsec, 1200
    R = Rmin + dR * np.arange(nr)
    I = 1e10 * (np.exp(-0.5 * ((R - 0.6 * arcsec) / (0.1 * arcsec)) ** 2) + 0.3 * np.exp(-0.5 * (R / (0.3 * arcsec)) ** 2))
    img = orc.sweep(I, Rmin, dR, nxy, dxy, inc)
    N, n = nxy, nxy // 2
    shifted = orc._fftshift(img)
    spec = orc._fft2d(np.ascontiguousarray(shifted.view(np.float64)[:, :N]))
    orc._fftshift_axis0(spec)
    rmax = min(int(np.ceil((Rmin + nr * dR) / dxy)), n)
    nF = n + 1 if rmax >= n else rmax
    F = np.array([[img[(n - a) % N, (n - c) % N] for c in range(nF)] for a in range(nF)])
    w = np.where((np.arange(nF) == 0) | (np.arange(nF) == n), 1.0, 2.0)
    C = w[None, :] * np.cos(2 * np.pi * ((np.outer(np.arange(n + 1), np.arange(nF))) % N) / N)
    D1T = digit_product(F, C)            # (nF, n + 1): D1[k][a] at [a, k]
    SpT = digit_product(C, D1T.T)        # (n + 1, n + 1): S'[k][t] at [t, k]
    S = np.array([[SpT[abs(r - n), k] for k in range(n + 1)] for r in range(N)])
    scale = np.abs(spec).max()
    assert np.abs(S - spec.real).max() <= 1e-13 * scale
