"""Exact products of multi-double matrices with Python integers.

TEST INFRASTRUCTURE ONLY.  Each p-double is a finite sum of doubles, hence a
dyadic rational; scaled by a common power of two it becomes an integer, and
the dot products of such integers are exact.  This is the referee for the
error bits of every GEMM form, independent of any floating-point arithmetic
(the hexa-double GEMM of oracle.c is the second, slower referee).
"""
import math

import numpy as np

_SHIFT = 1100  # every limb here lies above 2^-1100


def _to_int(x):
    """sum of the limbs of x (1-D array of doubles) times 2^_SHIFT."""
    s = 0
    for v in x:
        v = float(v)
        if v == 0.0:
            continue
        m, e = math.frexp(v)
        mi = int(m * (1 << 53))
        sh = e - 53 + _SHIFT
        s += mi << sh if sh >= 0 else mi >> (-sh)  # exact for limbs > 2^-1047
    return s


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
