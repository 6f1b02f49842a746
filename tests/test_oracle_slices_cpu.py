"""The oracle's restatement of the slice-digit form (oracle.c), pinned to
mathematics.  The reference has no slice-digit code to take golden vectors
from, so these properties are what the GPU's bit-exact agreement with the
oracle rests on: the digits are the stated fixed-point integer, nothing is
lost when no digit is truncated, the form commutes with transposition and
with scaling by powers of two, and it is no less accurate than the plain
form of the reference's arithmetic."""
import math
from fractions import Fraction

import numpy as np
import pytest

from conftest import pkg

SLICES = {2: 14, 4: 28, 8: 55, 16: 110}


def floor_scaled(v, shift):
    """floor(v * 2^shift) of a double v, exactly (Python's >> floors)."""
    if v == 0.0:
        return 0
    mf, e = math.frexp(v)
    m = int(mf * (1 << 53))
    q = e - 53 + shift
    return m << q if q >= 0 else m >> (-q)


@pytest.mark.parametrize("P", [2, 4, 8, 16])
def test_digits_are_the_scaled_fixed_point_integer(orc, inputs, P):
    """Row exponent E bounds every entry of the row (Σ|a_l| ≤ 2^E, exactly);
    the balanced base-256 digits d_0..d_{s-1} spell V = Σ_l floor(a_l 2^(S-E)),
    S = 7 + 8(s-1); every digit lies in [-128, 128]."""
    rng = np.random.default_rng(P)
    s, rows, cols = SLICES[P], 5, 7
    X = inputs.uniform_pd(rng, (rows, cols), P)
    X, _ = inputs.scale_rows(rng, X, -20, 20)
    X[1, 2] = 0.0
    X[3, 4] = -X[3, 4]
    E, _ = orc.scale_exps(P, X, np.zeros((cols, 1, P)), rows, 1, cols)
    d = orc.digits(P, s, X, rows, cols, E, 0)
    S = 7 + 8 * (s - 1)
    for r in range(rows):
        for c in range(cols):
            assert sum(abs(Fraction(float(a))) for a in X[r, c]) <= Fraction(2) ** int(E[r])
            V = sum(floor_scaled(float(a), S - int(E[r])) for a in X[r, c])
            W = 0
            for i in range(s):
                W = W * 256 + int(d[i, r, c])
            assert W == V, (r, c)
    assert np.abs(d).max() <= 128


@pytest.mark.parametrize("P", [2, 4, 8, 16])
def test_products_of_short_integers_are_exact(orc, P):
    """Entries that are small integers occupy the top digits only, so no
    digit pair reaches the truncated diagonals and C is the exact product."""
    rng = np.random.default_rng(10 + P)
    m, n, k = 6, 5, 9
    A = np.zeros((m, k, P))
    B = np.zeros((k, n, P))
    A[..., 0] = rng.integers(-100, 101, size=(m, k))
    B[..., 0] = rng.integers(-100, 101, size=(k, n))
    A[2, :, 0] = 64.0  # a row whose maximum is a power of two
    s = SLICES[P]
    C = orc.gemm_slices(P, s, s, A, B, m, n, k)
    assert np.array_equal(C[..., 0], A[..., 0] @ B[..., 0])  # |entries| < 2^17: exact
    assert not C[..., 1:].any()


@pytest.mark.parametrize("P", [2, 4, 8, 16])
def test_transposed_problem_gives_transposed_bits(orc, inputs, P):
    """C(Bᵀ, Aᵀ) = C(A, B)ᵀ bit for bit: row and column scales swap roles,
    the digit pairs of each diagonal are the same set, and the exact
    diagonal sums and their rounding do not depend on the order."""
    rng = np.random.default_rng(20 + P)
    m, n, k = 7, 5, 11
    A = inputs.uniform_pd(rng, (m, k), P)
    B = inputs.normal_pd(rng, (k, n), P)
    A, _ = inputs.scale_rows(rng, A, -9, 9)
    s = SLICES[P]
    C = orc.gemm_slices(P, s, s, A, B, m, n, k)
    At = np.ascontiguousarray(np.swapaxes(A, 0, 1))
    Bt = np.ascontiguousarray(np.swapaxes(B, 0, 1))
    Ct = orc.gemm_slices(P, s, s, Bt, At, n, m, k)
    assert np.array_equal(np.swapaxes(Ct, 0, 1).view(np.uint64), C.view(np.uint64))


@pytest.mark.parametrize("P", [2, 4, 8, 16])
@pytest.mark.parametrize("j", [-37, 5, 300])
def test_power_of_two_scaling_commutes(orc, inputs, P, j):
    """C(2^j A, B) = 2^j C(A, B) bit for bit: the row exponents move by j and
    the digits, diagonal sums and rounding stay the same."""
    rng = np.random.default_rng(30 + P)
    m, n, k = 4, 6, 8
    A = inputs.uniform_pd(rng, (m, k), P)
    B = inputs.uniform_pd(rng, (k, n), P)
    s = SLICES[P]
    C = orc.gemm_slices(P, s, s, A, B, m, n, k)
    Cj = orc.gemm_slices(P, s, s, np.ldexp(A, j), B, m, n, k)
    assert np.array_equal(Cj.view(np.uint64), np.ldexp(C, j).view(np.uint64))


@pytest.mark.parametrize("P", [2, 4, 8])
@pytest.mark.parametrize("dist", ["uniform", "normal", "spread"])
def test_slice_form_not_less_accurate_than_plain(orc, inputs, P, dist):
    """Against the exact product (Python integers), the slice form at the
    default digit count keeps at least the plain form's normwise bits, also
    with rows of A and columns of B scaled by 2^U{-32..32} (spread)."""
    ex = pkg("errors")
    rng = np.random.default_rng(40 + P)
    m = n = k = 12
    gen = inputs.normal_pd if dist == "normal" else inputs.uniform_pd
    A = gen(rng, (m, k), P)
    B = inputs.uniform_pd(rng, (k, n), P)
    if dist == "spread":
        A, _ = inputs.scale_rows(rng, A)
        B, _ = inputs.scale_cols(rng, B)
    s = SLICES[P]
    _, slice_bits = ex.error_bits(orc.gemm_slices(P, s, s, A, B, m, n, k), A, B,
                                  range(m), range(n))
    _, plain_bits = ex.error_bits(orc.gemm_plain(P, A, B, m, n, k), A, B, range(m), range(n))
    assert slice_bits >= plain_bits - 1.0, (slice_bits, plain_bits)
    assert slice_bits > {2: 95, 4: 205, 8: 415}[P]


DIGITS19 = {2: 6, 4: 12, 8: 24, 16: 47}


@pytest.mark.parametrize("P", [2, 4, 8])
@pytest.mark.parametrize("dist", ["uniform", "normal", "spread"])
def test_fp64_digit_form_not_less_accurate_than_plain(orc, inputs, P, dist):
    """The FP64 digit form (19-bit digits, the library's default counts)
    keeps at least the plain form's normwise bits against the exact
    product, like the BF16 digit form."""
    ex = pkg("errors")
    rng = np.random.default_rng(60 + P)
    m = n = k = 12
    gen = inputs.normal_pd if dist == "normal" else inputs.uniform_pd
    A = gen(rng, (m, k), P)
    B = inputs.uniform_pd(rng, (k, n), P)
    if dist == "spread":
        A, _ = inputs.scale_rows(rng, A)
        B, _ = inputs.scale_cols(rng, B)
    s = DIGITS19[P]
    _, bits = ex.error_bits(orc.gemm_digits(P, s, s, A, B, m, n, k), A, B, range(m), range(n))
    _, plain_bits = ex.error_bits(orc.gemm_plain(P, A, B, m, n, k), A, B, range(m), range(n))
    assert bits >= plain_bits - 1.0, (bits, plain_bits)


@pytest.mark.parametrize("P", [2, 4])
def test_digit_width_does_not_matter_without_truncation(orc, P):
    """With inputs short enough that neither digit form truncates anything
    (integers of a few bits), both forms return the exact product: the same
    bits whatever the digit width."""
    rng = np.random.default_rng(P + 90)
    m, n, k = 4, 5, 6
    A = np.zeros((m, k, P)); B = np.zeros((k, n, P))
    A[..., 0] = rng.integers(-7, 8, size=(m, k))
    B[..., 0] = rng.integers(-7, 8, size=(k, n))
    s8, s19 = SLICES[P], DIGITS19[P]
    C8 = orc.gemm_slices(P, s8, s8, A, B, m, n, k)
    C19 = orc.gemm_digits(P, s19, s19, A, B, m, n, k)
    exact = A[..., 0] @ B[..., 0]
    assert np.array_equal(C8[..., 0], exact) and np.array_equal(C19, C8)
