"""The CPU convolution driver's functions (include/TCcudant.h) against the
golden vectors the reference's own TCcudant.cpp produced (tests/golden/
cudant.npz): the unbalanced split and its planes bit for bit, the FP64
plane convolutions within the summation-order bound.  The driver program is
built with the host compiler only (the header needs no nvcc)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, pkg

CXX = shutil.which("g++") or "g++"


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    lib = pkg("_lib").LIB_PATH
    if not os.path.exists(lib):
        pkg("build").build()
    out = str(tmp_path_factory.mktemp("cudant") / "test_cudant")
    libdir = os.path.dirname(lib)
    subprocess.run([CXX, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    "-I", "/usr/local/cuda/include",
                    os.path.join(ROOT, "tests", "cpp", "test_cudant.cpp"),
                    "-L", libdir, "-lmdgemm", "-Wl,-rpath," + libdir, "-o", out],
                   check=True, capture_output=True)
    return out


def test_driver_builds_with_host_compiler(prog):
    assert os.path.exists(prog)


def test_short_operands_leave_outputs_alone(prog):
    """Plane operands one entry shorter than n x n x p: nothing is read or
    written past their end; convmult2 / convadd2 leave their outputs as they
    are and the one-step products return zeros before any device copy."""
    r = subprocess.run([prog, "short"], check=True, capture_output=True, text=True, timeout=60)
    assert r.stdout.strip() == "short 0"


def bound(Ap, Bp):
    """Per-entry bound on the difference of two FP64 summation orders of the
    truncated convolution: 2^-50 * sum_{j<=i} |A_j| |B_{i-j}|."""
    pp = Ap.shape[0]
    aA, aB = np.abs(Ap), np.abs(Bp)
    S = np.zeros((pp,) + (Ap.shape[1], Bp.shape[2]))
    for i in range(pp):
        for j in range(i + 1):
            S[i] += aA[j] @ aB[i - j]
    return 2.0 ** -50 * S + 1e-300


@pytest.mark.gpu
def test_cudant_functions_match_reference(prog, tmp_path):
    g = np.load(os.path.join(GOLDEN, "cudant.npz"))
    n, pp = g["A"].shape[0], g["As"].shape[2]
    P = pp // 4
    g["A"].tofile(tmp_path / "A.bin")
    g["B"].tofile(tmp_path / "B.bin")
    subprocess.run([prog, str(P), str(n), str(tmp_path / "A.bin"), str(tmp_path / "B.bin"),
                    str(tmp_path)], check=True, capture_output=True, timeout=120)
    rd = lambda name: np.fromfile(tmp_path / name)
    split = rd("split.bin").reshape(g["As"].shape)
    assert np.array_equal(split, g["As"]) and np.array_equal(np.signbit(split), np.signbit(g["As"]))
    Ap = np.ascontiguousarray(np.moveaxis(g["As"], 2, 0))
    Bp = np.ascontiguousarray(np.moveaxis(g["Bs"], 2, 0))
    assert np.array_equal(rd("planes.bin").reshape(Ap.shape), Ap)
    tol = bound(Ap, Bp)
    for name, ref in (("manual.bin", g["conv"]), ("direct.bin", g["direct"]),
                      ("twostep.bin", g["conv"]), ("accum.bin", g["direct"] + 1.0)):
        got = rd(name).reshape(ref.shape)
        assert np.all(np.abs(got - ref) <= tol + (2.0 ** -52 if name == "accum.bin" else 0)), name
    M = rd("matmul.bin").reshape(n, n)
    assert np.allclose(M, 1.0 + Ap[0] @ Bp[0], rtol=0, atol=2.0 ** -50 * float(np.abs(Ap[0]).sum()
                                                                               * np.abs(Bp[0]).max() + 1))


@pytest.mark.gpu
@pytest.mark.parametrize("P", [2, 4])
def test_split_planes_and_plane_conv_against_oracle(orc, inputs, P):
    """mdg_split kind 3 / mdg_split_planes against the oracle's unbalanced
    split (the reference's TCcudant split4pd), and mdg_plane_conv on
    rectangular planes against the oracle's slice convolution."""
    api = pkg("api")
    rng = np.random.default_rng(P)
    x = inputs.reference_pd(rng, (37, 5), P)
    planes = api.split_planes(3, x, P).cpu().numpy()
    aos = api.split4pd_unbalanced(x, P).cpu().numpy()
    assert np.array_equal(planes, aos.T)
    if orc.ref_available():
        assert np.array_equal(aos.reshape(-1), orc.ref_cudant_split4(x.reshape(-1)))
    m, n, k, pp = 70, 45, 33, 4 * P
    Aq = rng.standard_normal((m, k, pp))
    Bq = rng.standard_normal((k, n, pp))
    ref = orc.slice_conv(pp, Aq, Bq, m, n, k)
    import torch
    Ap = torch.from_numpy(np.ascontiguousarray(np.moveaxis(Aq, 2, 0))).cuda()
    Bp = torch.from_numpy(np.ascontiguousarray(np.moveaxis(Bq, 2, 0))).cuda()
    got = np.moveaxis(api.plane_conv(Ap, Bp).cpu().numpy(), 0, 2)
    tol = np.moveaxis(bound(np.moveaxis(Aq, 2, 0), np.moveaxis(Bq, 2, 0)), 0, 2)
    assert np.all(np.abs(got - ref) <= tol)
    # AoS and plane layouts give the same bits (same DMMA order)
    aos_conv = api.slice_conv(torch.from_numpy(Aq).cuda(), torch.from_numpy(Bq).cuda()).cpu().numpy()
    assert np.array_equal(got, aos_conv)


def test_plane_entries_reject_bad_arguments():
    import ctypes
    L = pkg("_lib").lib()
    one = ctypes.c_void_p(8)
    assert L.mdg_split_planes(3, 0, 4, 10, one, one, 9, None) == 2      # plane stride < count
    assert L.mdg_split_planes(4, 0, 4, 10, one, one, 10, None) == 4     # no kind 4
    assert L.mdg_split_planes(2, 0, 4, 10, one, one, 10, None) == 1     # mixed split needs P = 2
    assert L.mdg_split(3, 2, 4, 10, one, one, None) == 4                # exact must be 0 or 1
    assert L.mdg_plane_conv(0, 4, 4, 4, one, one, one, None) == 2
    assert L.mdg_plane_conv(4, 4, 4, 4, None, one, one, None) == 3
    assert L.mdg_plane_conv(4, 0, 4, 4, None, None, None, None) == 0
