"""Generates the golden vectors in this directory from the reference itself.

Every output below is computed by the reference's own functions, compiled
from its sources by oracle/Makefile into oracle/_ref (the sources must be
present, so this script runs in the build container only).  Inputs come
from the seeded generators of the library's inputs module.

    python tests/golden/make_golden.py              # every file
    python tests/golden/make_golden.py hostfuncs    # hostfuncs_P{2,4}, squeeze_P2_pp12, mat_seed_range
    python tests/golden/make_golden.py hostfuncs_wide   # hostfuncs_P{8,16}.npz only

Files (numpy .npz):
  arith_P{2,4,8,16}.npz   add/mul/sub/div/sqrt/inc_d/mul_d of 256 pairs
                          (ddf_*/qdf_*/odf_*/hdf_*, *_double_functions.cu)
  matmul_P*.npz           matmul{dd,qd,od,hd}f on n x n (TCcuda.cu:320-372)
  matmul_dd64.npz         the 64^3 double-double workload (seed 0)
  split_*.npz             split4pd/split8pd/mixsplit2 (floatybits.cu:196-342)
  squeeze_P*.npz          *_inc_d squeeze of pp partials (TCcuda.cu:876-906)
  mat_seed.npz            srand(seed); mat(n, p) (TCcuda.cu:14)
  bigB2.npz               bigB2 block-Toeplitz matrix (TCcuda.cu:79-95)
  cudant.npz              TCcudant.cpp split4pd + manualconvmult/directdotconv
  hostfuncs_P{2,4,8,16}.npz  part, bigA, bigB, matmulhost, renormhost, renormhostbig
                          (TCcuda.cu host functions, TCcuda.h:33-81)
  mat_seed_range.npz      srand(seed); mat(n, p, expmin, expmax) with expmin < expmax
  squeeze_P2_pp12.npz     dd squeeze of the 12 partials of mixsplit2
"""
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

inputs = importlib.import_module(
    "multiple-double-arithmetic-matrix-matrix-multiplication_gb300.inputs")


def mixed(rng, count, P):
    """Half signed uniform p-doubles, half reference-style positive ones,
    with zeros, exact powers of two and a negative tail limb planted."""
    a = inputs.uniform_pd(rng, (count // 2,), P)
    b = inputs.reference_pd(rng, (count - count // 2,), P)
    x = np.concatenate([a, b])
    x[5] = 0.0
    x[6, 0] = 1.0
    x[6, 1:] = 0.0
    x[7, 0] = -0.5
    x[9, 1] = -abs(x[9, 1])
    return x


def main():
    oracle.build(ref=True)
    rng = np.random.default_rng(20240601)
    for P in (2, 4, 8, 16):
        a = mixed(rng, 256, P)
        b = mixed(rng, 256, P) * 0.625
        d = {"a": a, "b": b}
        for op in ("add", "mul", "sub", "div", "inc_d", "mul_d"):
            bb = b[:, 0] if op in ("inc_d", "mul_d") else b
            d[op] = oracle.ref_vec_op(op, P, a, bb)
        d["sqrt"] = oracle.ref_vec_op("sqrt", P, np.abs(a))
        np.savez_compressed(os.path.join(HERE, f"arith_P{P}.npz"), **d)

        n = {2: 12, 4: 10, 8: 8, 16: 4}[P]
        A = mixed(rng, n * n, P).reshape(n, n, P)
        B = mixed(rng, n * n, P).reshape(n, n, P)
        np.savez_compressed(os.path.join(HERE, f"matmul_P{P}.npz"), A=A, B=B,
                            C=oracle.ref_matmul(P, A, B, n))

        for pp_mul, kind in ((4, "split4"), (8, "split8")):
            x = mixed(rng, 64, P)
            np.savez_compressed(os.path.join(HERE, f"{kind}_P{P}.npz"), x=x,
                                out=oracle.ref_split(kind, P, x))
            xr = inputs.reference_pd(rng, (64,), P)
            np.savez_compressed(os.path.join(HERE, f"{kind}_P{P}_refstyle.npz"), x=xr,
                                out=oracle.ref_split(kind, P, xr))
            pp = pp_mul * P
            parts = oracle.ref_split(kind, P, xr) * 3.0
            np.savez_compressed(os.path.join(HERE, f"squeeze_P{P}_pp{pp}.npz"), x=parts,
                                y=oracle.ref_squeeze(P, pp, parts))
    x = mixed(rng, 64, 2)
    np.savez_compressed(os.path.join(HERE, "split_mix_P2.npz"), x=x,
                        out=oracle.ref_split("mix", 2, x))

    _, A, B = inputs.workload("dd64")
    np.savez_compressed(os.path.join(HERE, "matmul_dd64.npz"), A=A, B=B,
                        C=oracle.ref_matmul(2, A, B, 64))

    np.savez_compressed(os.path.join(HERE, "mat_seed.npz"), seed=7, n=3, P=4,
                        out=oracle.ref_mat(7, 3, 4))

    n, pp = 3, 8
    Bq = rng.uniform(-1, 1, size=(n, n, pp))
    np.savez_compressed(os.path.join(HERE, "bigB2.npz"), Bq=Bq, n=n, pp=pp,
                        out=oracle.ref_bigB2(Bq, n, pp))

    n, P = 8, 4
    A = inputs.reference_pd(rng, (n, n), P)
    B = inputs.reference_pd(rng, (n, n), P)
    As = oracle.ref_cudant_split4(A).reshape(n, n, 4 * P)
    Bs = oracle.ref_cudant_split4(B).reshape(n, n, 4 * P)
    Ap = np.ascontiguousarray(np.moveaxis(As, 2, 0))
    Bp = np.ascontiguousarray(np.moveaxis(Bs, 2, 0))
    np.savez_compressed(os.path.join(HERE, "cudant.npz"), A=A, B=B, As=As, Bs=Bs,
                        conv=oracle.ref_cudant_conv(0, n, 4 * P, Ap, Bp),
                        direct=oracle.ref_cudant_conv(1, n, 4 * P, Ap, Bp))


def hostfuncs():
    """The reference's layout helpers and host-side functions on small
    signed inputs (own seed, so the other files stay as they are)."""
    oracle.build(ref=True)
    rng = np.random.default_rng(20241203)
    for P, n in ((2, 5), (4, 4)):
        A = mixed(rng, n * n, P).reshape(n, n, P)
        B = mixed(rng, n * n, P).reshape(n, n, P)
        d = {"A": A, "B": B, "n": n, "P": P,
             "part1": oracle.ref_host("part", n * n, P, A, i=1),
             "bigA": oracle.ref_host("bigA", n, P, A),
             "bigB": oracle.ref_host("bigB", n, P, B),
             "matmulhost": oracle.ref_host("matmulhost", n, P, A, B),
             "renormhost": oracle.ref_host("renormhost", n, P, A),
             "renormhostbig": oracle.ref_host("renormhostbig", n, P, A)}
        np.savez_compressed(os.path.join(HERE, f"hostfuncs_P{P}.npz"), **d)
    # the double-double squeeze of the mixed split (12 partials per entry)
    parts = oracle.ref_split("mix", 2, mixed(rng, 48, 2)) * 3.0
    np.savez_compressed(os.path.join(HERE, "squeeze_P2_pp12.npz"), x=parts,
                        y=oracle.ref_squeeze(2, 12, parts))
    # mat / random_pd with an exponent range: rand() % (expmax - expmin) drawn per entry
    np.savez_compressed(os.path.join(HERE, "mat_seed_range.npz"), seed=11, n=4, P=4,
                        expmin=-6, expmax=5, out=oracle.ref_mat(11, 4, 4, -6, 5))


def hostfuncs_wide():
    """The same host functions at P = 8 and 16 (own seed, so the files of
    ``hostfuncs`` stay as they are)."""
    oracle.build(ref=True)
    rng = np.random.default_rng(20241204)
    for P in (8, 16):
        n = 4
        A = mixed(rng, n * n, P).reshape(n, n, P)
        B = mixed(rng, n * n, P).reshape(n, n, P)
        d = {"A": A, "B": B, "n": n, "P": P,
             "part1": oracle.ref_host("part", n * n, P, A, i=1),
             "bigA": oracle.ref_host("bigA", n, P, A),
             "bigB": oracle.ref_host("bigB", n, P, B),
             "matmulhost": oracle.ref_host("matmulhost", n, P, A, B),
             "renormhost": oracle.ref_host("renormhost", n, P, A),
             "renormhostbig": oracle.ref_host("renormhostbig", n, P, A)}
        np.savez_compressed(os.path.join(HERE, f"hostfuncs_P{P}.npz"), **d)


if __name__ == "__main__":
    if sys.argv[1:] == ["hostfuncs"]:
        hostfuncs()
    elif sys.argv[1:] == ["hostfuncs_wide"]:
        hostfuncs_wide()
    else:
        main()
        hostfuncs()
        hostfuncs_wide()
