"""Error bits of computed multi-double matrices: the measurement half of the
error reporting (not on the GEMM path; the benchmark and the tests use it).

Each p-double is a finite sum of doubles, hence a dyadic rational; scaled by
a common power of two it becomes an integer, and the dot products of such
integers are exact.  ``error_bits`` compares a computed block of C with that
exact product (Python integers: a few dozen entries at k = 8192).
``referee_error_bits`` compares a large block with a higher-precision
referee result instead (e.g. the octo-double plain GEMM of quad-double
inputs, 2^-420 accurate), exactly, entry by entry.
"""
import math

import numpy as np

_SHIFT = 1100  # every limb here lies above 2^-1100


def _limbs_to_int(x, shift):
    """sum of the limbs of x times 2^shift, exact for limbs above 2^-shift."""
    s = 0
    for v in x:
        v = float(v)
        if v == 0.0:
            continue
        m, e = math.frexp(v)
        mi = int(m * (1 << 53))
        sh = e - 53 + shift
        s += mi << sh if sh >= 0 else mi >> (-sh)
    return s



def _to_int(x):
    """sum of the limbs of x (1-D array of doubles) times 2^_SHIFT."""
    return _limbs_to_int(x, _SHIFT)


def to_ints(M):
    """(rows, cols, P) array -> nested list of exact scaled integers."""
    r, c, _ = M.shape
    return [[_to_int(M[i, j]) for j in range(c)] for i in range(r)]


def product_block(A, B, rows, cols):
    """Exact C[rows][cols] of A (m x k x P) times B (k x n x P), returned as
    (integers scaled by 2^(2*_SHIFT), and sum |a||b| scaled the same way)."""
    Ai = [[_to_int(A[i, kk]) for kk in range(A.shape[1])] for i in rows]
    Bi = [[_to_int(B[kk, j]) for kk in range(B.shape[0])] for j in cols]
    C, N = [], []
    for a in Ai:
        crow, nrow = [], []
        for b in Bi:
            crow.append(sum(x * y for x, y in zip(a, b)))
            nrow.append(sum(abs(x * y) for x, y in zip(a, b)))
        C.append(crow)
        N.append(nrow)
    return C, N


def _log2_ratio(num, den):
    """log2(|num| / |den|) for integers, den != 0; -inf for num == 0."""
    num, den = abs(num), abs(den)
    if num == 0:
        return -math.inf
    return (num.bit_length() - den.bit_length()) + math.log2(
        (num / (1 << (num.bit_length() - 1))) / (den / (1 << (den.bit_length() - 1))))


def error_bits(Cmd, A, B, rows, cols):
    """Error bits of a computed C (array of p-doubles) over a sampled block:
    (entrywise  -log2 max |C - O| / |O|,  normwise  -log2 max |C - O| / (|A||B|)).
    Capped at 1100 for an exact result."""
    O, N = product_block(A, B, rows, cols)
    worst_e, worst_n = -math.inf, -math.inf
    for a, i in enumerate(rows):
        for b, j in enumerate(cols):
            c = 0
            for v in Cmd[i, j]:
                v = float(v)
                if v != 0.0:
                    m, e = math.frexp(v)
                    mi = int(m * (1 << 53))
                    sh = e - 53 + 2 * _SHIFT
                    c += mi << sh if sh >= 0 else mi >> (-sh)
            diff = c - O[a][b]
            if N[a][b] == 0:
                continue
            if O[a][b] != 0:
                worst_e = max(worst_e, _log2_ratio(diff, O[a][b]))
            worst_n = max(worst_n, _log2_ratio(diff, N[a][b]))
    cap = lambda v: 1100.0 if v == -math.inf else min(1100.0, -v)
    return cap(worst_e), cap(worst_n)


def referee_error_bits(C, R, N):
    """(entrywise, normwise) error bits of C (r x c x P) against a referee R
    (r x c x P', more precise) with N (r x c) = sum_k |a||b| per entry:
    -log2 max |C - R| / |R| and -log2 max |C - R| / N, the differences taken
    exactly.  Capped at 1100 for identical values."""
    worst_e, worst_n = -math.inf, -math.inf
    for i in range(C.shape[0]):
        for j in range(C.shape[1]):
            r = _limbs_to_int(R[i, j], _SHIFT)
            d = _limbs_to_int(C[i, j], _SHIFT) - r
            if d == 0:
                continue
            if r != 0:
                worst_e = max(worst_e, _log2_ratio(d, r))
            n = float(N[i, j])
            if n > 0:
                worst_n = max(worst_n, math.log2(abs(d)) - _SHIFT - math.log2(n))
    cap = lambda v: 1100.0 if v == -math.inf else min(1100.0, -v)
    return cap(worst_e), cap(worst_n)
