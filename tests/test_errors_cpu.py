"""Host-side measurement logic without a GPU: the exact referee comparison
of errors.py and the leading-dimension rule of api.gemm_ex."""
import math

import numpy as np
import torch

from conftest import pkg


def test_referee_error_bits_are_exact():
    ex = pkg("errors")
    # referee = computed value + 2^-130 exactly (a difference far below one
    # double's precision, visible only through the exact limb sums)
    C = np.array([[[1.0, 2.0 ** -60], [3.0, 0.0]]])
    R = np.array([[[1.0, 2.0 ** -60, 2.0 ** -130], [3.0, 0.0, 0.0]]])
    N = np.array([[1.0, 3.0]])
    ent, nrm = ex.referee_error_bits(C, R, N)
    assert ent == 130.0 and nrm == 130.0
    # identical values: capped
    assert ex.referee_error_bits(C[:, 1:], R[:, 1:, :2], N[:, 1:]) == (1100.0, 1100.0)
    # a relative error of 2^-100 on an entry whose norm is 2^4 larger
    C2 = np.array([[[1.0, 0.0]]])
    R2 = np.array([[[1.0, 2.0 ** -100]]])
    ent2, nrm2 = ex.referee_error_bits(C2, R2, np.array([[16.0]]))
    assert abs(ent2 - 100.0) < 1e-9 and abs(nrm2 - 104.0) < 1e-9


def test_exact_error_bits_on_known_product():
    ex = pkg("errors")
    A = np.zeros((1, 2, 2)); B = np.zeros((2, 1, 2))
    A[0, 0] = [1.0, 2.0 ** -70]; A[0, 1] = [0.5, 0.0]
    B[0, 0] = [1.0, 0.0]; B[1, 0] = [2.0, 2.0 ** -80]
    exact = 1.0 + 2.0 ** -70 + 1.0 + 2.0 ** -81       # sum_k a b
    C = np.array([[[2.0, 2.0 ** -70]]])                 # misses 2^-81
    ent, nrm = ex.error_bits(C, A, B, range(1), range(1))
    assert abs(ent - (81 + math.log2(exact))) < 1e-6


def test_gemm_ex_leading_dimension_rule():
    api = pkg("api")
    big = torch.zeros((10, 12, 4), dtype=torch.float64)
    assert api._ld(big, 4) == 12
    assert api._ld(big[:, :7], 4) == 12          # padded rows keep the row stride
    assert api._ld(big[:1, :7], 4) == 7          # one row: the logical width
    assert api._ld(torch.zeros((3, 0, 4), dtype=torch.float64), 4) == 1
