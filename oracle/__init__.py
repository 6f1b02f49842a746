"""CPU oracle for the multi-double GEMM path.

TEST INFRASTRUCTURE ONLY: this package is the checker.  tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the
library under multiple-double-arithmetic-matrix-matrix-multiplication_gb300/
never does.

* ``liboracle`` (oracle.c) restates the reference's algorithms in plain C.
* ``ref`` binds oracle/_ref/libref.so, the reference's own host functions,
  when that library has been built (only possible where the reference
  sources are present).
* ``exact`` computes exact products with Python integers, the independent
  referee for error bits.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(HERE, "_build", "liboracle.so")
_REF = os.path.join(HERE, "_ref", "libref.so")
_CUDANT = os.path.join(HERE, "_ref", "libcudant.so")
# the reference's C++ sources, staged beside the repository by `make stage`
REF_SOURCES = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "C++")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_int64)


def build(ref=None):
    """Compile oracle.c (and the reference libraries when the reference
    sources exist and ``ref`` is not False).  The sources are staged into
    REF_SOURCES first when a reference checkout is at hand."""
    targets = ["oracle"]
    if ref is not False:
        subprocess.run(["make", "-s", "-C", HERE, "stage"], check=True)
    if ref is None:
        ref = os.path.isdir(REF_SOURCES)
    if ref:
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_BUILD):
            build(ref=False)
        L = ctypes.CDLL(_BUILD)
        L.orc_gemm_plain_rows.argtypes = [ctypes.c_int] * 4 + [_dp, _dp, _dp] + [ctypes.c_int] * 3
        L.orc_vec_binop.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, _dp, _dp, _dp]
        L.orc_split.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_long, _dp, _dp]
        L.orc_squeeze.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, _dp, _dp]
        L.orc_slice_conv_rows.argtypes = [ctypes.c_int] * 4 + [_dp, _dp, _dp] + [ctypes.c_int] * 3
        L.orc_scale_exps.argtypes = [ctypes.c_int] * 4 + [_dp, _dp, _ip, _ip]
        L.orc_digits.argtypes = [ctypes.c_int] * 4 + [_dp, _ip, ctypes.c_int, _ip]
        L.orc_diag_sums.argtypes = [ctypes.c_int] * 5 + [_ip, _ip, _lp]
        L.orc_renorm_diags.argtypes = [ctypes.c_int] * 4 + [_lp, _ip, _ip, _dp]
        L.orc_gemm_slices.argtypes = [ctypes.c_int] * 6 + [_dp, _dp, _dp]
        L.orc_gemm_digits.argtypes = [ctypes.c_int] * 6 + [_dp, _dp, _dp]
        L.orc_has_openmp.restype = ctypes.c_int
        L.orc_plane_conv.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
        L.orc_generate.argtypes = [ctypes.c_int] * 4 + [ctypes.c_uint64, ctypes.c_int,
                                                        ctypes.c_int, _dp]
        _lib = L
    return _lib


# ----------------------------------------------------------------- oracle --

OPS = {"add": 0, "mul": 1, "sub": 2, "div": 3, "sqrt": 4, "inc_d": 5, "mul_d": 6}


def vec_op(op, P, a, b=None):
    a = _f64(a).reshape(-1, P)
    b = np.zeros_like(a) if b is None else _f64(b).reshape(-1, P) if np.size(b) == a.size else _f64(np.column_stack([b] + [np.zeros_like(b)] * (P - 1)))
    c = np.zeros_like(a)
    lib().orc_vec_binop(OPS[op], P, a.shape[0], _ptr(a), _ptr(b), _ptr(c))
    return c


def gemm_plain(P, A, B, m, n, k, rows=None, threads=1):
    """C = A*B with the reference's plain multi-double arithmetic
    (TCcuda.cu:320-372); A is m x k, B is k x n, row-major, limbs last."""
    A = _f64(A)
    B = _f64(B)
    C = np.zeros(m * n * P, dtype=np.float64)
    r0, r1 = (0, m) if rows is None else rows
    lib().orc_gemm_plain_rows(P, m, n, k, _ptr(A), _ptr(B), _ptr(C), r0, r1, threads)
    return C.reshape(m, n, P)


SPLIT_KINDS = {"split4": 0, "split8": 1, "mix": 2}


def split(kind, P, x, exact=False):
    x = _f64(x).reshape(-1, P)
    pp = {0: 4 * P, 1: 8 * P, 2: 12}[SPLIT_KINDS[kind]]
    out = np.zeros((x.shape[0], pp), dtype=np.float64)
    lib().orc_split(SPLIT_KINDS[kind], int(exact), P, x.shape[0], _ptr(x), _ptr(out))
    return out


def squeeze(P, pp, x):
    x = _f64(x).reshape(-1, pp)
    y = np.zeros((x.shape[0], P), dtype=np.float64)
    lib().orc_squeeze(P, pp, x.shape[0], _ptr(x), _ptr(y))
    return y


def slice_conv(pp, Aq, Bq, m, n, k, rows=None, threads=1):
    Aq = _f64(Aq)
    Bq = _f64(Bq)
    C = np.zeros(m * n * pp, dtype=np.float64)
    r0, r1 = (0, m) if rows is None else rows
    lib().orc_slice_conv_rows(pp, m, n, k, _ptr(Aq), _ptr(Bq), _ptr(C), r0, r1, threads)
    return C.reshape(m, n, pp)


def gemm_fp64split(P, A, B, m, n, k, kind="split4", exact=True):
    """The FP64 split form end to end: split, truncated slice convolution,
    squeeze (TCtest.cu:48-114)."""
    Aq = split(kind, P, A, exact)
    Bq = split(kind, P, B, exact)
    pp = Aq.shape[1]
    Cq = slice_conv(pp, Aq, Bq, m, n, k)
    return squeeze(P, pp, Cq.reshape(-1, pp)).reshape(m, n, P)


def scale_exps(P, A, B, m, n, k):
    A = _f64(A)
    B = _f64(B)
    E = np.zeros(m, dtype=np.int32)
    F = np.zeros(n, dtype=np.int32)
    lib().orc_scale_exps(P, m, n, k, _ptr(A), _ptr(B), _ptr(E, _ip), _ptr(F, _ip))
    return E, F


def digits(P, s, x, rows, cols, E, trans):
    x = _f64(x)
    E = np.ascontiguousarray(E, dtype=np.int32)
    out = np.zeros((s, rows, cols), dtype=np.int32)
    lib().orc_digits(P, s, rows, cols, _ptr(x), _ptr(E, _ip), int(trans), _ptr(out, _ip))
    return out


def diag_sums(s, D, dA, dB, m, n, k):
    dA = np.ascontiguousarray(dA, dtype=np.int32)
    dB = np.ascontiguousarray(dB, dtype=np.int32)
    Cd = np.zeros((D, m, n), dtype=np.int64)
    lib().orc_diag_sums(s, D, m, n, k, _ptr(dA, _ip), _ptr(dB, _ip), _ptr(Cd, _lp))
    return Cd


def renorm_diags(P, D, Cd, E, F, m, n):
    Cd = np.ascontiguousarray(Cd, dtype=np.int64)
    E = np.ascontiguousarray(E, dtype=np.int32)
    F = np.ascontiguousarray(F, dtype=np.int32)
    C = np.zeros((m, n, P), dtype=np.float64)
    lib().orc_renorm_diags(P, D, m, n, _ptr(Cd, _lp), _ptr(E, _ip), _ptr(F, _ip), _ptr(C))
    return C


def gemm_slices(P, s, D, A, B, m, n, k):
    A = _f64(A)
    B = _f64(B)
    C = np.zeros((m, n, P), dtype=np.float64)
    lib().orc_gemm_slices(P, s, D, m, n, k, _ptr(A), _ptr(B), _ptr(C))
    return C


def gemm_digits(P, s, D, A, B, m, n, k):
    """The FP64 digit form (19-bit digits) on the CPU, bit for bit."""
    A = _f64(A)
    B = _f64(B)
    C = np.zeros((m, n, P), dtype=np.float64)
    lib().orc_gemm_digits(P, s, D, m, n, k, _ptr(A), _ptr(B), _ptr(C))
    return C


def plane_conv(n, pp, A, B):
    """TCcudant.cpp's manualconvmult order on pp slice planes of n x n."""
    A = _f64(A)
    B = _f64(B)
    C = np.zeros((pp, n, n), dtype=np.float64)
    lib().orc_plane_conv(n, pp, _ptr(A), _ptr(B), _ptr(C))
    return C


def generate(dist, P, rows, cols, seed, e0=0, e1=0):
    """rows x cols x P float64 from the counter-based generator (dist as in
    mdg_generate: 0 uniform, 1 normal, 2 reference family, +4 / +8 scales)."""
    X = np.empty((rows, cols, P), dtype=np.float64)
    lib().orc_generate(dist, P, rows, cols, int(seed) & (2 ** 64 - 1), e0, e1, _ptr(X))
    return X


def has_openmp():
    return bool(lib().orc_has_openmp())


# ------------------------------------------------------------- reference --

_ref = None
_cudant = None


def ref_available():
    """The reference-built libraries exist and load on this machine (a copy
    built for another architecture does not count)."""
    if not (os.path.exists(_REF) and os.path.exists(_CUDANT)):
        return False
    try:
        ref()
        cudant()
    except OSError:
        return False
    return True


def ref():
    """The reference's own host functions (oracle/_ref/libref.so)."""
    global _ref
    if _ref is None:
        R = ctypes.CDLL(_REF)
        R.ref_binop.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, _dp, _dp, _dp]
        R.ref_matmul.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
        R.ref_split.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, _dp, _dp]
        R.ref_squeeze.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, _dp, _dp]
        R.ref_mat.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp]
        R.ref_bigB2.argtypes = [_dp, ctypes.c_int, ctypes.c_int, _dp]
        R.ref_host.argtypes = [ctypes.c_int] * 4 + [_dp, _dp, _dp]
        R.ref_host.restype = ctypes.c_long
        _ref = R
    return _ref


def cudant():
    global _cudant
    if _cudant is None:
        L = ctypes.CDLL(_CUDANT)
        L.cudant_split4.argtypes = [ctypes.c_long, _dp, _dp]
        L.cudant_conv.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
        _cudant = L
    return _cudant


def ref_vec_op(op, P, a, b=None):
    a = _f64(a).reshape(-1, P)
    b = np.zeros_like(a) if b is None else _f64(b).reshape(-1, P) if np.size(b) == a.size else _f64(np.column_stack([b] + [np.zeros_like(b)] * (P - 1)))
    c = np.zeros_like(a)
    rc = ref().ref_binop(OPS[op], P, a.shape[0], _ptr(a), _ptr(b), _ptr(c))
    assert rc == 0
    return c


def ref_matmul(P, A, B, n):
    A = _f64(A)
    B = _f64(B)
    C = np.zeros(n * n * P, dtype=np.float64)
    assert ref().ref_matmul(P, n, _ptr(A), _ptr(B), _ptr(C)) == 0
    return C.reshape(n, n, P)


def ref_split(kind, P, x):
    x = _f64(x).reshape(-1, P)
    pp = {0: 4 * P, 1: 8 * P, 2: 12}[SPLIT_KINDS[kind]]
    out = np.zeros((x.shape[0], pp), dtype=np.float64)
    assert ref().ref_split(SPLIT_KINDS[kind], P, x.shape[0], _ptr(x), _ptr(out)) == 0
    return out


def ref_squeeze(P, pp, x):
    x = _f64(x).reshape(-1, pp)
    y = np.zeros((x.shape[0], P), dtype=np.float64)
    assert ref().ref_squeeze(P, pp, x.shape[0], _ptr(x), _ptr(y)) == 0
    return y


def ref_mat(seed, n, P, expmin=0, expmax=0):
    out = np.zeros(n * n * P, dtype=np.float64)
    ref().ref_mat(seed, n, P, expmin, expmax, _ptr(out))
    return out.reshape(n, n, P)


def ref_bigB2(Bq, n, pp):
    Bq = _f64(Bq)
    out = np.zeros((n * pp) * (n * pp), dtype=np.float64)
    ref().ref_bigB2(_ptr(Bq), n, pp, _ptr(out))
    return out


REF_HOST = {"part": 0, "bigA": 1, "bigB": 2, "matmulhost": 3, "renormhost": 4,
            "renormhostbig": 5}


def ref_host(name, n, p, A, B=None, i=0):
    """The reference's layout helper / host function `name` (TCcuda.h:33-81)
    on n P-doubles (part) or n x n P-doubles (the others)."""
    A = _f64(A)
    B = _f64(B) if B is not None else np.zeros(1)
    out = np.zeros(max(A.size, (n * p) ** 2), dtype=np.float64)
    got = ref().ref_host(REF_HOST[name], n, p, i, _ptr(A), _ptr(B), _ptr(out))
    assert got >= 0, name
    return out[:got].copy()


def ref_cudant_conv(how, n, pp, A, B):
    A = _f64(A)
    B = _f64(B)
    C = np.zeros(pp * n * n, dtype=np.float64)
    cudant().cudant_conv(how, n, pp, _ptr(A), _ptr(B), _ptr(C))
    return C.reshape(pp, n, n)


def ref_cudant_split4(x):
    x = _f64(x).ravel()
    out = np.zeros(x.size * 4, dtype=np.float64)
    cudant().cudant_split4(x.size, _ptr(x), _ptr(out))
    return out
