"""The CPU oracle against the golden vectors made by the reference itself.

Every comparison is bit for bit (values compared with ==, so +0 and -0 are
equal, plus an explicit sign-of-zero check for the split slices)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, pkg


def load(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.mark.parametrize("P", [2, 4, 8, 16])
@pytest.mark.parametrize("op", ["add", "mul", "sub", "div", "sqrt", "inc_d", "mul_d"])
def test_arith_matches_reference(orc, P, op):
    g = load(f"arith_P{P}.npz")
    a, b = g["a"], g["b"]
    if op == "sqrt":
        out = orc.vec_op("sqrt", P, np.abs(a))
    elif op in ("inc_d", "mul_d"):
        out = orc.vec_op(op, P, a, b[:, 0])
    else:
        out = orc.vec_op(op, P, a, b)
    assert np.array_equal(out, g[op], equal_nan=True)


@pytest.mark.parametrize("P", [2, 4, 8, 16])
def test_plain_gemm_matches_reference(orc, P):
    g = load(f"matmul_P{P}.npz")
    n = g["A"].shape[0]
    assert np.array_equal(orc.gemm_plain(P, g["A"], g["B"], n, n, n), g["C"])


def test_dd64_workload_matches_reference(orc):
    g = load("matmul_dd64.npz")
    assert np.array_equal(orc.gemm_plain(2, g["A"], g["B"], 64, 64, 64), g["C"])


def test_dd64_inputs_are_the_committed_ones(inputs):
    g = load("matmul_dd64.npz")
    P, A, B = inputs.workload("dd64")
    assert P == 2 and np.array_equal(A, g["A"]) and np.array_equal(B, g["B"])


@pytest.mark.parametrize("P", [2, 4, 8, 16])
@pytest.mark.parametrize("kind", ["split4", "split8"])
@pytest.mark.parametrize("style", ["", "_refstyle"])
def test_split_matches_reference(orc, P, kind, style):
    g = load(f"{kind}_P{P}{style}.npz")
    out = orc.split(kind, P, g["x"])
    assert np.array_equal(out, g["out"])
    assert np.array_equal(np.signbit(out), np.signbit(g["out"]))


def test_mixsplit_matches_reference(orc):
    g = load("split_mix_P2.npz")
    out = orc.split("mix", 2, g["x"])
    assert np.array_equal(out, g["out"])
    assert np.array_equal(np.signbit(out), np.signbit(g["out"]))


@pytest.mark.parametrize("P,pp", [(2, 8), (2, 12), (2, 16), (4, 16), (4, 32), (8, 32), (8, 64),
                                  (16, 64), (16, 128)])
def test_squeeze_matches_reference(orc, P, pp):
    g = load(f"squeeze_P{P}_pp{pp}.npz")
    assert np.array_equal(orc.squeeze(P, pp, g["x"]), g["y"])


def test_cpu_convolution_path_matches_reference(orc):
    g = load("cudant.npz")
    n, pp = g["A"].shape[0], g["As"].shape[2]
    Ap = np.ascontiguousarray(np.moveaxis(g["As"], 2, 0))
    Bp = np.ascontiguousarray(np.moveaxis(g["Bs"], 2, 0))
    assert np.array_equal(orc.plane_conv(n, pp, Ap, Bp), g["conv"])
    # the per-entry order of directdotconv is the k-outer, j-inner order
    direct = orc.slice_conv(pp, g["As"], g["Bs"], n, n, n)
    assert np.array_equal(np.moveaxis(direct, 2, 0), g["direct"])


def test_bigB2_layout(orc):
    """The block-Toeplitz matrix of the reference equals the truncated
    slice convolution the oracle computes without it."""
    g = load("bigB2.npz")
    n, pp, Bq = int(g["n"]), int(g["pp"]), g["Bq"]
    BB = g["out"].reshape(n * pp, n * pp).T  # column-major -> [row][col]
    rng = np.random.default_rng(0)
    Aq = rng.uniform(-1, 1, size=(2, n, pp))
    via_bigB2 = Aq.reshape(2, n * pp) @ BB
    conv = orc.slice_conv(pp, Aq, Bq, 2, n, n)
    assert np.allclose(via_bigB2.reshape(2, n, pp), conv, rtol=1e-14, atol=1e-15)


def test_slice_digit_form_is_exact_on_small_case(orc, inputs):
    """Slice digits reconstruct the inputs and the diagonal GEMM keeps
    enough bits: qd 16^3 agrees with the exact product to > 212 bits."""
    ex = pkg("errors")
    P, A, B = inputs.workload("qd1024", 16, 16, 16)
    C = orc.gemm_slices(P, 28, 28, A, B, 16, 16, 16)
    ent, nrm = ex.error_bits(C, A, B, range(16), range(16))
    Cp = orc.gemm_plain(P, A, B, 16, 16, 16)
    ent_p, nrm_p = ex.error_bits(Cp, A, B, range(16), range(16))
    assert nrm >= nrm_p - 1.0, (nrm, nrm_p)
    assert nrm > 205
