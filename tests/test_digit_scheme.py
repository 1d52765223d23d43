"""The exact digit products of the tensor-core moment kernels, restated on the CPU.

kripke_gb300/csrc/tc_moments.cu writes every row of A (and, on the host, every
column of B) as 7 balanced 8-bit digits of a 54-bit fixed-point magnitude
relative to the row's largest exponent, accumulates every digit product of an
anti-diagonal i + j in FP32 (exact while each diagonal sum stays below 2^24),
keeps the diagonals i + j <= 8 and rounds their integer combination once to a
double.  This test restates that arithmetic with Python integers and checks the
properties the kernels rely on:

* the balanced digits (bytes of magnitude + 0x80 per byte, minus 128) rebuild
  the magnitude exactly and lie in [-128, 127] (exact in f16 and bf16);
* every diagonal sum for K <= 128 stays below 2^24, so the FP32 accumulation in
  tensor memory is exact;
* the once-rounded result lies within 2^-50 max|a| max|b| K of the exact dot
  product (the dropped diagonals and the truncation below each operand's
  window), on rows spanning many decades with zeros and sign changes.
"""
from fractions import Fraction
import random
import struct

S = 7          # digits per operand (FP64 form)
W = 8 * S - 2  # fixed-point bits
BIAS = sum(0x80 << (8 * j) for j in range(S))


def bexp(x):
    """Biased exponent, subnormals and zero counted as 1 (the kernels' expOf)."""
    e = (struct.unpack("<Q", struct.pack("<d", x))[0] >> 52) & 0x7FF
    return max(e, 1)


def fixed(x, emax):
    """(magnitude, sign) of x in the W-bit window whose top bit is emax's leading bit."""
    b = struct.unpack("<Q", struct.pack("<d", x))[0]
    e = (b >> 52) & 0x7FF
    m = (b & ((1 << 52) - 1)) | ((1 << 52) if e else 0)
    sh = emax - max(e, 1)
    f = (m << (W - 53)) >> sh if sh < 64 else 0
    return f, -1 if b >> 63 else 1


def digits(f, s):
    """Balanced digits, most significant first, times the sign."""
    y = f + BIAS
    return [s * (((y >> (8 * (S - 1 - i))) & 0xFF) - 128) for i in range(S)]


def test_balanced_digits_rebuild_the_magnitude():
    rng = random.Random(7)
    for _ in range(20000):
        f = rng.getrandbits(W)
        s = rng.choice((-1, 1))
        d = digits(f, s)
        assert all(-128 <= v * s <= 127 for v in d)
        assert sum(v << (8 * (S - 1 - i)) for i, v in enumerate(d)) == s * f


def test_diagonal_sums_fit_fp32():
    # worst case: every digit at magnitude 128 and K = 128 products per pair
    K = 128
    for m in range(2, S + 2):  # kept diagonals i + j = m
        pairs = m - 1
        assert pairs * K * 128 * 128 < 2 ** 24


def rounded_product(a_row, b_col):
    """The kernel's result for one output: digit products, kept diagonals, one rounding."""
    ea = max(bexp(x) for x in a_row)
    eb = max(bexp(x) for x in b_col)
    da = [digits(*fixed(x, ea)) for x in a_row]
    db = [digits(*fixed(x, eb)) for x in b_col]
    diag = [0] * (2 * S + 1)
    for ak, bk in zip(da, db):
        for i in range(S):
            for j in range(S):
                if i + j + 2 <= S + 1:  # digits are 1-based in the kernel: keep i + j <= S + 1
                    diag[i + j + 2] += ak[i] * bk[j]
    for m in range(2, S + 2):
        assert abs(diag[m]) < 2 ** 24
    # each operand is 2^(e - 1022 - W) * sum_i d_i 2^(8(S-1-i)); the product's
    # diagonal m carries 2^(8(S-1-i) + 8(S-1-j)) = 2^(8(2S - m))
    v = sum(diag[m] << (8 * (2 * S - m)) for m in range(2, S + 2))
    scale = (ea - 1022 - W) + (eb - 1022 - W)
    return float(Fraction(v) * Fraction(2) ** scale)


def test_rounded_products_against_exact_dot_products():
    rng = random.Random(11)
    worst = 0.0
    for trial in range(60):
        K = rng.choice((8, 25, 32, 64, 128))
        span = rng.choice((0, 3, 10, 23))
        a = [rng.uniform(-1, 1) * 10.0 ** rng.uniform(-span, 0) for _ in range(K)]
        b = [rng.uniform(-1, 1) * 10.0 ** rng.uniform(-span, 0) for _ in range(K)]
        for k in rng.sample(range(K), K // 7):
            a[k] = 0.0
        got = rounded_product(a, b)
        exact = sum(Fraction(x) * Fraction(y) for x, y in zip(a, b))
        scale = max(abs(x) for x in a) * max(abs(y) for y in b)
        err = abs(Fraction(got) - exact) / Fraction(scale)
        assert err <= Fraction(K, 2 ** 50), (trial, K, span, float(err))
        worst = max(worst, float(err))
    assert worst < 5e-15  # about 2e-15 observed on such rows
