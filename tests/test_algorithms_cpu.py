"""CPU restatements (numpy) of the numerical schemes inside the FP64 kernels,
checked against direct evaluations.  They pin the derivations the CUDA code
follows; the GPU tests check the kernels themselves against the oracle.

- even-sequence transform (``even_dft_block``, gb_device.cuh): DCT-I of the
  half sequence from a quarter-length complex FFT, odd outputs by a prefix
  sum of Im Y;
- exact floor / fraction from a double's bit pattern (``floor_frac_bits``);
- FP32 upper bound of |x| from a double's high word (``abs_bound_f``);
- table-driven sin/cos of the phase with the magic-number reduction and the
  2^20-entry table built from double-double products (``sincos2pi_tab``);
- the FP32 sign estimate's error bound (``interp_cell_real``).
"""
import math
import struct
from fractions import Fraction

import numpy as np
import pytest


# ------------------------------------------------------------ even sequences
def even_dft_direct(x, xn, n):
    """C_k = sum_J s[J] exp(-2 pi i J k / N) for s even about 0, period N = 2n."""
    N = 2 * n
    s = np.zeros(N)
    s[:len(x)] = x
    s[n] = xn
    for j in range(1, n):
        s[N - j] = s[j]
    return np.fft.fft(s).real


def even_dft_quarter(x, xn, n, kmax):
    """The scheme of even_dft_block: y, the length-n/2 FFT of y[2m] + i y[2m+1],
    the even/odd split, C_2k = 2 Re Y_k, C_2k+1 = C_1 - 2 sum_{i<=k} Im Y_i."""
    nnz = len(x)
    xs = np.zeros(n + 1)
    xs[:nnz] = x
    xs[n] = xn
    j = np.arange(n)
    xj = xs[:n]
    xm = xs[n - j]  # x_{n-j}; j = 0 gives x_n
    sj = np.sin(np.pi * j / n)
    y = 0.5 * (xj + xm) - sj * (xj - xm)
    y[0] = 0.5 * (xs[0] + xs[n])
    c1 = (xs[0] - xs[n]) + 2.0 * np.sum(xs[1:n] * np.cos(np.pi * np.arange(1, n) / n))
    M = n // 2
    Z = np.fft.fft(y[0::2] + 1j * y[1::2])
    kh = kmax // 2
    k = np.arange(kh + 1)
    za = Z[np.where(k == M, 0, k)]
    zb = Z[np.where(k == 0, 0, (M - k) % M)]
    E = 0.5 * (za + np.conj(zb))
    O = (za - np.conj(zb)) / 2j
    Y = E + np.exp(-2j * np.pi * k / n) * O
    C = np.zeros(kmax + 1)
    C[0::2] = 2 * Y.real[: len(C[0::2])]
    if kmax >= 1:
        C[1] = c1
        run = 0.0
        for i in range(1, (kmax - 1) // 2 + 1):
            run += Y.imag[i]
            C[2 * i + 1] = c1 - 2.0 * run
    return C


@pytest.mark.parametrize("n,nnz,with_xn", [(16, 5, False), (64, 64, True), (512, 171, False), (2048, 342, False),
                                           (1024, 1024, True)])
def test_even_dft_quarter_length_scheme(n, nnz, with_xn):
    rng = np.random.default_rng(n + nnz)
    x = rng.normal(size=nnz)
    xn = rng.normal() if with_xn else 0.0
    kmax = n  # every output
    ref = even_dft_direct(x, xn, n)[: kmax + 1]
    got = even_dft_quarter(x, xn, n, kmax)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


# ------------------------------------------------------------- bit patterns
def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def from_bits(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def floor_frac_bits(x):
    """floor_frac_bits of gb_kernels.cu: exact for x in [0, 2^30)."""
    b = bits(x)
    if b >> 63:
        return None
    e = (b >> 52) - 1023
    if e > 29:
        return None
    if e < 0:
        return 0, x
    m = (b & 0xFFFFFFFFFFFFF) | 0x10000000000000
    sh = 52 - e
    fl = m >> sh
    f = m & ((1 << sh) - 1)
    if f == 0:
        return fl, 0.0
    p = f.bit_length() - 1
    mant = (f << (52 - p)) & 0xFFFFFFFFFFFFF
    return fl, from_bits(((p - sh + 1023) << 52) | mant)


def test_floor_frac_bits_exact():
    rng = np.random.default_rng(5)
    xs = list(rng.uniform(0, 4096, 20000)) + list(rng.uniform(0, 1, 2000)) + \
        [0.0, 1.0, 2.0 ** 29, 2.0 ** 30 - 2.0 ** -22, 4095.999999999999, 0.5, 5e-324, 2048.0 + 2.0 ** -41]
    for x in xs:
        fl, fr = floor_frac_bits(float(x))
        assert fl == math.floor(x)
        assert Fraction(fr) == Fraction(x) - math.floor(x)  # exact
    assert floor_frac_bits(-1.0) is None and floor_frac_bits(2.0 ** 30) is None


def abs_bound_f(x):
    """abs_bound_f of gb_kernels.cu (as float32 values)."""
    hi = (bits(x) >> 32) & 0x7FFFFFFF
    e = hi >> 20
    if e == 2047:
        return 0.0
    if e < 1023 - 126:
        return float(np.float32(1.17549435e-38))
    if e > 1023 + 127:
        return math.inf
    fb = (((e - 1023 + 127) << 23) | ((hi & 0xFFFFF) << 3)) + 8
    return float(np.frombuffer(struct.pack("<I", fb), dtype=np.float32)[0])


def test_abs_bound_is_an_upper_bound_with_small_slack():
    rng = np.random.default_rng(6)
    xs = np.concatenate([rng.normal(0, 1e7, 5000), rng.uniform(-1, 1, 5000), [0.0, -0.0, 1.0, -2.5e-30, 3.3e38]])
    for x in xs:
        b = abs_bound_f(float(x))
        assert b >= abs(x)
        if abs(x) > 1e-37 and b != math.inf:
            assert b <= abs(x) * (1 + 2.0 ** -19)
    assert abs_bound_f(math.nan) == 0.0 and abs_bound_f(math.inf) == 0.0


# --------------------------------------------------------- phase sin / cos
T = 1 << 20
MAGIC52 = 6755399441055744.0


def _cos_sin_2pi(frac):
    """cos and sin of 2 pi frac (a Fraction) to about 40 digits (decimal Taylor series)."""
    import decimal
    ctx = decimal.Context(prec=60)
    pi = decimal.Decimal("3.14159265358979323846264338327950288419716939937510582097494459")
    a = ctx.multiply(ctx.divide(decimal.Decimal(frac.numerator), decimal.Decimal(frac.denominator)), 2 * pi)
    c, s, term, k = decimal.Decimal(1), decimal.Decimal(0), decimal.Decimal(1), 0
    while True:
        k += 1
        term = ctx.divide(ctx.multiply(term, a), k)
        if k % 4 == 1:
            s += term
        elif k % 4 == 2:
            c -= term
        elif k % 4 == 3:
            s -= term
        else:
            c += term
        if abs(term) < decimal.Decimal(10) ** -50:
            break
    return c, s


def phase_table_entries(js):
    """The host construction of gb_api.cu: exp(2 pi i jh / 2^10) exp(2 pi i jl / T),
    products rounded once to double (the double-double arithmetic there is
    accurate to about 2^-104; exact decimals stand in for it here)."""
    out = []
    for j in js:
        ch, sh = _cos_sin_2pi(Fraction(j >> 10, 1 << 10))
        cl, sl = _cos_sin_2pi(Fraction(j & 1023, T))
        out.append((float(ch * cl - sh * sl), float(sh * cl + ch * sl)))
    return out


def sincos2pi_tab(a, table):
    r = math.fma(a, float(T), MAGIC52) if hasattr(math, "fma") else float(Fraction(a) * T + Fraction(MAGIC52))
    j = bits(r) & (T - 1)
    d = (r - MAGIC52) * (-1.0 / T) + a  # exact (Sterbenz): the fused form equals it
    x = d * 6.283185307179586476925286766559
    h = (0.5 * x) * x
    ex, ey = table[j]
    c = -ex * h + (-ey * x + ex)
    s = -ey * h + (ex * x + ey)
    return s, c


def test_phase_reduction_and_short_series():
    rng = np.random.default_rng(7)
    args = list(rng.uniform(-200, 200, 300)) + [0.0, 0.25, -0.5, 1e-9, 123456.789]
    rs = [math.fma(a, float(T), MAGIC52) if hasattr(math, "fma") else float(Fraction(a) * T + Fraction(MAGIC52))
          for a in args]
    js = sorted({bits(r) & (T - 1) for r in rs})
    table = dict(zip(js, phase_table_entries(js)))
    for a in args:
        s, c = sincos2pi_tab(float(a), table)
        frac = Fraction(a) - math.floor(Fraction(a))  # exact reduction
        ch, sh = _cos_sin_2pi(frac)
        assert abs(c - float(ch)) <= 3.4e-16 and abs(s - float(sh)) <= 3.4e-16  # a few units in the last place


# ------------------------------------------------------ FP32 sign estimate
def test_fp32_sign_estimate_bound():
    """|z_f32 - z| stays below the (8 * 2^-24 + 2 * 2^-23) sum|y| the kernel
    relies on when it trusts the FP32 sign beyond 4e-6 sum|y|."""
    rng = np.random.default_rng(8)
    f32 = np.float32
    worst = 0.0
    for _ in range(20000):
        y = rng.normal(size=4) * 10.0 ** rng.uniform(-8, 8)
        t, q = rng.uniform(0, 1, 2)
        f1, f3 = y[1] - y[0], y[3] - y[0]
        z = q * (t * ((y[2] - y[3]) - f1) + f3) + (t * f1 + y[0])
        yf = y.astype(f32)
        tf, qf = f32(t), f32(q)  # truncation is at most the rounding's double
        g1, g3 = yf[1] - yf[0], yf[3] - yf[0]
        zf = qf * (tf * ((yf[2] - yf[3]) - g1) + g3) + (tf * g1 + yf[0])
        worst = max(worst, abs(float(zf) - z) / np.sum(np.abs(y)))
    assert worst < 7.2e-7 < 4e-6
