"""The counter-based input generator (mdg_generate): the oracle's C
restatement checked for the promised distributions and structure on the
CPU, the C ABI's argument checks without a GPU, and the CUDA kernel against
the oracle bit for bit on the GPU."""
import ctypes

import numpy as np
import pytest

from conftest import pkg

UNIFORM, NORMAL, REFERENCE, ROWS, COLS = 0, 1, 2, 4, 8


def ulp(x):
    e = np.frexp(np.abs(x))[1]
    return np.where(x == 0, 0.0, np.ldexp(1.0, e - 53))


@pytest.mark.parametrize("P", [2, 4, 8, 16])
def test_uniform_and_normal_distributions(orc, P):
    U = orc.generate(UNIFORM, P, 300, 200, 11)
    N = orc.generate(NORMAL, P, 300, 200, 11)
    assert np.all(np.abs(U[..., 0]) <= 1.0)
    assert abs(U[..., 0].mean()) < 0.01 and abs(U[..., 0].var() - 1 / 3) < 0.01
    assert np.all(np.abs(N[..., 0]) <= 6.0)
    assert abs(N[..., 0].mean()) < 0.01 and abs(N[..., 0].var() - 1.0) < 0.02
    for X in (U, N):
        # limbs do not overlap: each tail limb is at most half an ulp of the one above
        for i in range(1, P):
            assert np.all(np.abs(X[..., i]) <= 0.5 * ulp(X[..., i - 1]))
        assert np.count_nonzero(X[..., P - 1]) > 0.99 * X[..., 0].size


@pytest.mark.parametrize("P", [2, 4, 8, 16])
def test_reference_family_structure(orc, P):
    """random_pd (floatybits.cu:107-120): positive limbs, limb i = f 2^(e-52i)
    with f in [0.5, 1), 52 fraction bits, the first set; e in [e0, e1)."""
    e0, e1 = 3, 9
    X = orc.generate(REFERENCE, P, 40, 50, 5, e0, e1)
    _, ex = np.frexp(X[..., 0])
    assert ex.min() == e0 and ex.max() == e1 - 1
    for i in range(P):
        f = np.ldexp(X[..., i], -(ex - 52 * i))
        assert np.all((f >= 0.5) & (f < 1.0))
        k = np.ldexp(f, 52)
        assert np.array_equal(k, np.floor(k))
    X0 = orc.generate(REFERENCE, P, 4, 5, 5, -7, -7)
    assert np.all(np.frexp(X0[..., 0])[1] == -7)


def test_scales_and_determinism(orc):
    base = orc.generate(UNIFORM, 4, 30, 20, 77)
    rows = orc.generate(UNIFORM | ROWS, 4, 30, 20, 77, -32, 32)
    cols = orc.generate(UNIFORM | COLS, 4, 30, 20, 77, -32, 32)
    both = orc.generate(UNIFORM | ROWS | COLS, 4, 30, 20, 77, -5, 5)
    sr = np.log2(rows[:, :, 0] / base[:, :, 0])
    sc = np.log2(cols[:, :, 0] / base[:, :, 0])
    assert np.array_equal(sr, np.round(sr)) and np.all(sr == sr[:, :1])
    assert np.array_equal(sc, np.round(sc)) and np.all(sc == sc[:1, :])
    assert sr.min() >= -32 and sr.max() <= 32 and len(np.unique(sr)) > 10
    sb = np.log2(both[:, :, 0] / base[:, :, 0])
    assert sb.min() >= -10 and sb.max() <= 10
    assert np.array_equal(orc.generate(NORMAL, 4, 30, 20, 77), orc.generate(NORMAL, 4, 30, 20, 77))
    assert not np.array_equal(orc.generate(NORMAL, 4, 30, 20, 77),
                              orc.generate(NORMAL, 4, 30, 20, 78))
    # an entry depends on its index r * cols + c only: a sub-block of rows
    # is the prefix of the taller matrix
    assert np.array_equal(orc.generate(NORMAL, 2, 7, 20, 9), orc.generate(NORMAL, 2, 30, 20, 9)[:7])


def test_generate_argument_errors_without_gpu():
    L = pkg("_lib").lib()
    one = ctypes.c_void_p(8)
    gen = L.mdg_generate
    assert gen(UNIFORM, 3, 4, 4, 1, 0, 0, one, 4, None) == 1           # limbs
    assert gen(UNIFORM, 4, -1, 4, 1, 0, 0, one, 4, None) == 2          # size
    assert gen(UNIFORM, 4, 4, 4, 1, 0, 0, one, 3, None) == 2           # ldx < cols
    assert gen(3, 4, 4, 4, 1, 0, 0, one, 4, None) == 4                 # no such distribution
    assert gen(UNIFORM | 16, 4, 4, 4, 1, 0, 0, one, 4, None) == 4      # unknown flag
    assert gen(REFERENCE | ROWS, 4, 4, 4, 1, 0, 0, one, 4, None) == 4  # scales only for 0, 1
    assert gen(REFERENCE, 4, 4, 4, 1, 5, 4, one, 4, None) == 4         # e1 < e0
    assert gen(REFERENCE, 16, 4, 4, 1, -300, -300, one, 4, None) == 4  # last limb subnormal
    assert gen(REFERENCE, 2, 4, 4, 1, 1020, 1025, one, 4, None) == 4   # overflow
    assert gen(UNIFORM | ROWS, 4, 4, 4, 1, -65, 0, one, 4, None) == 4  # scale range
    assert gen(NORMAL, 4, 0, 4, 1, 0, 0, None, 4, None) == 0           # empty
    assert gen(NORMAL, 4, 4, 4, 1, 0, 0, None, 4, None) == 3           # NULL


@pytest.mark.gpu
@pytest.mark.parametrize("P", [2, 4, 8, 16])
@pytest.mark.parametrize("dist,e0,e1", [(UNIFORM, 0, 0), (NORMAL, 0, 0), (REFERENCE, 0, 0),
                                        (REFERENCE, -100, 50), (NORMAL | ROWS, -32, 32),
                                        (UNIFORM | COLS, -32, 32), (UNIFORM | ROWS | COLS, -3, 4)])
def test_generate_bit_exact_against_oracle(orc, P, dist, e0, e1):
    import torch
    api = pkg("api")
    rows, cols = 67, 45
    for seed in (0, 4, 2 ** 64 - 1):
        ref = orc.generate(dist, P, rows, cols, seed, e0, e1)
        kind = {0: "uniform", 1: "normal", 2: "reference"}[dist & 3]
        got = api.generate(kind, P, rows, cols, seed, e0, e1, scale_rows=bool(dist & ROWS),
                           scale_cols=bool(dist & COLS))
        assert np.array_equal(got.cpu().numpy(), ref), seed
    # leading dimension larger than cols: only the first cols entries per row change
    big = torch.full((rows, cols + 5, P), 7.0, dtype=torch.float64, device="cuda")
    api.generate("normal", P, rows, cols, 9, out=big[:, :cols])
    assert np.array_equal(big[:, :cols].cpu().numpy(), orc.generate(NORMAL, P, rows, cols, 9))
    assert torch.all(big[:, cols:] == 7.0)


@pytest.mark.gpu
def test_generate_large_matches_oracle_rows(orc):
    """A 4096 x 4096 quad-double draw (grid-stride over 16.7 M entries):
    sampled rows equal the oracle's rows of the same matrix."""
    api = pkg("api")
    X = api.generate("normal", 4, 4096, 4096, 4)
    head = orc.generate(NORMAL, 4, 3, 4096, 4)
    assert np.array_equal(X[:3].cpu().numpy(), head)
    assert abs(float(X[..., 0].mean())) < 0.01 and abs(float(X[..., 0].var()) - 1) < 0.01
