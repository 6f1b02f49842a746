"""The drop-in C++ surface on the host (no GPU): a small C++ program linked
against libmdgemm.so runs the reference-named host functions and the
results are compared with the golden vectors made by the reference itself.
Also checks that the reference's own driver compiles against the drop-in
headers when the reference sources are present."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, pkg

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    lib = pkg("_lib").LIB_PATH
    if not os.path.exists(lib):
        pkg("build").build()
    out = str(tmp_path_factory.mktemp("dropin") / "test_dropin")
    libdir = os.path.dirname(lib)
    subprocess.run([NVCC, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    "-x", "cu", os.path.join(ROOT, "tests", "cpp", "test_dropin.cpp"),
                    "-gencode", "arch=compute_103a,code=sm_103a",
                    "-L", libdir, "-lmdgemm", "-Xlinker", "-rpath," + libdir, "-o", out],
                   check=True, capture_output=True)
    return out


def run(prog, *args):
    subprocess.run([prog] + [str(a) for a in args], check=True, capture_output=True, timeout=120)


def test_mat_reproduces_reference_rand_sequence(prog, tmp_path):
    g = np.load(os.path.join(GOLDEN, "mat_seed.npz"))
    out = tmp_path / "mat.bin"
    run(prog, "mat", int(g["n"]), int(g["P"]), int(g["seed"]), out)
    assert np.array_equal(np.fromfile(out).reshape(g["out"].shape), g["out"])


def test_mat_with_exponent_range_reproduces_reference(prog, tmp_path):
    g = np.load(os.path.join(GOLDEN, "mat_seed_range.npz"))
    out = tmp_path / "mat.bin"
    run(prog, "mat", int(g["n"]), int(g["P"]), int(g["seed"]), out, int(g["expmin"]),
        int(g["expmax"]))
    got = np.fromfile(out).reshape(g["out"].shape)
    assert np.array_equal(got, g["out"])
    e = np.frexp(got[..., 0])[1]
    assert e.min() >= int(g["expmin"]) and e.max() < int(g["expmax"])


@pytest.mark.parametrize("P", [2, 4, 8, 16])
def test_host_matmul_matches_reference(prog, tmp_path, P):
    g = np.load(os.path.join(GOLDEN, f"matmul_P{P}.npz"))
    n = g["A"].shape[0]
    g["A"].tofile(tmp_path / "A.bin")
    g["B"].tofile(tmp_path / "B.bin")
    run(prog, "matmul", P, n, tmp_path / "A.bin", tmp_path / "B.bin", tmp_path / "C.bin")
    assert np.array_equal(np.fromfile(tmp_path / "C.bin").reshape(g["C"].shape), g["C"],
                          equal_nan=True)


def test_bigB2_matches_reference(prog, tmp_path):
    g = np.load(os.path.join(GOLDEN, "bigB2.npz"))
    g["Bq"].tofile(tmp_path / "Bq.bin")
    run(prog, "bigB2", int(g["n"]), int(g["pp"]), tmp_path / "Bq.bin", tmp_path / "o.bin")
    assert np.array_equal(np.fromfile(tmp_path / "o.bin"), g["out"])


@pytest.mark.parametrize("P,pp", [(2, 8), (2, 12), (4, 32), (8, 64), (16, 128)])
def test_host_squeeze_matches_reference(prog, tmp_path, P, pp):
    g = np.load(os.path.join(GOLDEN, f"squeeze_P{P}_pp{pp}.npz"))
    g["x"].tofile(tmp_path / "x.bin")
    run(prog, "squeeze", P, pp, tmp_path / "x.bin", tmp_path / "y.bin")
    assert np.array_equal(np.fromfile(tmp_path / "y.bin").reshape(g["y"].shape), g["y"])


@pytest.mark.parametrize("P", [2, 4, 8, 16])
@pytest.mark.parametrize("name", ["part1", "bigA", "bigB", "matmulhost", "renormhost",
                                  "renormhostbig"])
def test_host_layout_and_renorm_functions_match_reference(prog, tmp_path, P, name):
    """part, bigA, bigB, matmulhost, renormhost and renormhostbig of the
    drop-in against the reference's own functions (TCcuda.h:33-81)."""
    g = np.load(os.path.join(GOLDEN, f"hostfuncs_P{P}.npz"))
    g["A"].tofile(tmp_path / "A.bin")
    g["B"].tofile(tmp_path / "B.bin")
    run(prog, "host", name, P, int(g["n"]), tmp_path / "A.bin", tmp_path / "B.bin",
        tmp_path / "o.bin")
    got = np.fromfile(tmp_path / "o.bin")
    assert np.array_equal(got, g[name])
    assert np.array_equal(np.signbit(got), np.signbit(g[name]))


@pytest.mark.parametrize("P", [2, 4])
def test_short_operands_give_empty_or_zero_results(prog, P):
    """Vectors one double shorter than their n x n x p shape (the reference
    reads past their end): the layout builders return empty vectors, the
    products zeros, the in-place renormalisations leave the vector as it is,
    and the GPU product returns before any device copy."""
    n = 3
    full = n * n * P
    r = subprocess.run([prog, "short", str(P), str(n)], check=True, capture_output=True,
                       text=True, timeout=60)
    got = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())
    assert got["bigA"] == got["bigB"] == got["bigB2"] == "0"
    assert got["matmulhost"] == f"{full} 0 {full} 0"
    assert float(got["renormhost"]) == float(got["renormhostbig"]) == full - 1  # all ones kept
    assert got["matmulTCnt"] == f"{full} 0 0"
    assert got["matmulddf" if P == 2 else "matmulqdf"] == "0"
    assert got["pllntsqueeze"] == "0"


def test_every_declared_kernel_links(prog):
    """The __global__ functions TCcuda.h declares (TCcuda.h:56-102) resolve
    to libmdgemm.so: renormbigA, renormA, ddmm..hdmm, the three separate-plane
    double-double squeezes and the four pllsqueeze_*_pp_old kernels."""
    r = subprocess.run([prog, "kernels"], check=True, capture_output=True, text=True,
                       timeout=60)
    assert r.stdout.strip() == "13"


REF_DRIVER = "/root/reference/C++/TCtest.cu"


@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference sources not present")
def test_reference_driver_compiles_against_dropin_headers(tmp_path):
    """The reference's own driver (unmodified) compiles and links against the
    drop-in headers and libmdgemm.so: the integration a maintainer makes."""
    lib = pkg("_lib").LIB_PATH
    libdir = os.path.dirname(lib)
    r = subprocess.run([NVCC, "-std=c++17", "-w", "-I", os.path.join(ROOT, "include"),
                        REF_DRIVER, "-gencode", "arch=compute_103a,code=sm_103a",
                        "-L", libdir, "-lmdgemm", "-o", str(tmp_path / "mytest")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
