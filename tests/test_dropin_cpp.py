"""The drop-in C++ surface: a small C++ program linked against libmdgemm.so
runs the reference-named functions and the results are compared with the
golden vectors made by the reference itself.  The host functions are tested
without a GPU; the tests marked gpu run the std::vector wrappers
(matmulTCnt, matmulTC, split4pd / split8pd / mixsplit2, pllsqueeze_old,
pllsqueeze, pllsqueeze_2_{8,12,16}) and launch every kernel TCcuda.h
exports (ddmm..hdmm, renormA, renormbigA, pllsqueeze_{2,4,8,16}_pp_old,
pllsqueeze_kernel_2_{8,12,16}) the way the reference's code does.
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
                    "-gencode", "arch=compute_103a,code=sm_103a", "-cudart", "shared",
                    "-L", libdir, "-lmdgemm", "-Xlinker", "-rpath," + libdir, "-o", out],
                   check=True, capture_output=True)
    return out


def run(prog, *args):
    r = subprocess.run([prog] + [str(a) for a in args], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, (args[:3], r.returncode, r.stderr[-2000:])
    return r.stdout


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


# the reference's driver, from the sources staged beside the repository
REF_DRIVER = os.path.join(ROOT, "baseline", "_ref", "C++", "TCtest.cu")


@pytest.mark.gpu
@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference sources not present")
def test_reference_driver_runs_against_the_library(tmp_path):
    """The reference's driver, unmodified (TCtest.cu:48-208: p = 8, n = 64,
    q = 4), built against the drop-in headers and libmdgemm.so and run on the
    GPU: mat, split4pd and bigB2 from the library feed the driver's own wmma
    DMMA kernel, pllsqueeze_old squeezes its 32 partials per entry and
    matmulTCnt computes the plain octo-double product.  The driver prints
    the largest difference of the two results; with its positive inputs of
    magnitude about 36 both forms are accurate to about 2^-410, so the
    difference is far below 1e-100."""
    lib = pkg("_lib").LIB_PATH
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "mytest")
    r = subprocess.run([NVCC, "-std=c++17", "-w", "-I", os.path.join(ROOT, "include"),
                        REF_DRIVER, "-gencode", "arch=compute_103a,code=sm_103a",
                        "-cudart", "shared", "-L", libdir, "-lmdgemm",
                        "-Xlinker", "-rpath," + libdir, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    print(r.stdout)
    lines = dict(line.split("? ", 1) for line in r.stdout.splitlines() if "? " in line)
    max_err = float(lines["Max error"].split()[0])
    assert 0.0 <= max_err < 1e-100, r.stdout
    tc = [float(v) for v in lines["TC C[1,1]"].strip("()").split(",")]
    plain = [float(v) for v in lines["CUDA C[1,1]"].strip("()").split(",")]
    assert len(tc) == len(plain) == 8 and 1.0 < tc[0] < 64.0
    assert abs(tc[0] - plain[0]) <= 1e-13 * plain[0]


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


# ------------------------------------------------------------------ GPU --

def _roundtrip(prog, tmp_path, args, inputs, out_shape=None):
    """Write the inputs, run the command with their paths, read the output."""
    paths = []
    for i, x in enumerate(inputs):
        path = tmp_path / f"in{i}.bin"
        np.ascontiguousarray(x, dtype=np.float64).tofile(path)
        paths.append(path)
    out = tmp_path / "out.bin"
    run(prog, *args, *paths, out)
    got = np.fromfile(out)
    return got.reshape(out_shape) if out_shape is not None else got


GOLDEN_MATMUL = [(2, "matmul_P2"), (4, "matmul_P4"), (8, "matmul_P8"), (16, "matmul_P16"),
                 (2, "matmul_dd64")]


@pytest.mark.gpu
@pytest.mark.parametrize("P,name", GOLDEN_MATMUL)
def test_gpu_matmulTCnt_wrapper_matches_reference(prog, tmp_path, P, name):
    """matmulTCnt (TCcuda.cu:248-302) through the std::vector wrapper:
    the reference's host product bit for bit, two timed launches."""
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    n = g["A"].shape[0]
    got = _roundtrip(prog, tmp_path, ["tcnt", P, n, min(32, n)], [g["A"], g["B"]],
                     g["C"].shape)
    assert np.array_equal(got, g["C"], equal_nan=True)


@pytest.mark.gpu
@pytest.mark.parametrize("P,name", GOLDEN_MATMUL)
def test_gpu_exported_plain_kernels_match_reference(prog, tmp_path, P, name):
    """ddmm / qdmm / odmm / hdmm launched by the caller as matmulTCnt does in
    the reference (grid (n/nfrag)^2, block nfrag^2, TCcuda.cu:262-297)."""
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    n = g["A"].shape[0]
    nfrag = 32 if n % 32 == 0 else n
    got = _roundtrip(prog, tmp_path, ["kmm", P, n, nfrag], [g["A"], g["B"]], g["C"].shape)
    assert np.array_equal(got, g["C"], equal_nan=True)


@pytest.mark.gpu
@pytest.mark.parametrize("P", [2, 4, 8])
def test_gpu_matmulTC_wrapper_all_forms(prog, tmp_path, orc, inputs, P):
    """matmulTC in the plain (bit for bit), FP64-split (oracle error bits
    within 2), BF16 slice and FP64 digit (bit for bit vs the oracle) forms."""
    ex = pkg("errors")
    n = 24
    rng = np.random.default_rng(P + 40)
    A = inputs.uniform_pd(rng, (n, n), P)
    B = inputs.uniform_pd(rng, (n, n), P)
    plain = _roundtrip(prog, tmp_path, ["tc", 0, P, n], [A, B], (n, n, P))
    assert np.array_equal(plain, orc.gemm_plain(P, A, B, n, n, n))
    s = pkg("api").default_slices(P)
    sl = _roundtrip(prog, tmp_path, ["tc", 2, P, n], [A, B], (n, n, P))
    assert np.array_equal(sl, orc.gemm_slices(P, s, s, A, B, n, n, n))
    s19 = pkg("api").default_slices(P, "fp64_digits")
    fd = _roundtrip(prog, tmp_path, ["tc", 3, P, n], [A, B], (n, n, P))
    assert np.array_equal(fd, orc.gemm_digits(P, s19, s19, A, B, n, n, n))
    sp = _roundtrip(prog, tmp_path, ["tc", 1, P, n], [A, B], (n, n, P))
    ref = orc.gemm_fp64split(P, A, B, n, n, n)
    bits = ex.error_bits(sp, A, B, range(n), range(n))
    bits_ref = ex.error_bits(ref, A, B, range(n), range(n))
    assert bits[1] >= bits_ref[1] - 2.0, (bits, bits_ref)


@pytest.mark.gpu
@pytest.mark.parametrize("P", [2, 4, 8, 16])
@pytest.mark.parametrize("kind", ["split4", "split8"])
@pytest.mark.parametrize("style", ["", "_refstyle"])
def test_gpu_split_wrappers_match_reference(prog, tmp_path, P, kind, style):
    """split4pd / split8pd (floatybits.cu:515,622) through the wrapper."""
    g = np.load(os.path.join(GOLDEN, f"{kind}_P{P}{style}.npz"))
    got = _roundtrip(prog, tmp_path, ["gsplit", kind, P], [g["x"]], g["out"].shape)
    assert np.array_equal(got, g["out"])
    assert np.array_equal(np.signbit(got), np.signbit(g["out"]))


@pytest.mark.gpu
def test_gpu_mixsplit2_wrapper_matches_reference(prog, tmp_path):
    g = np.load(os.path.join(GOLDEN, "split_mix_P2.npz"))
    got = _roundtrip(prog, tmp_path, ["gsplit", "mix", 2], [g["x"]], g["out"].shape)
    assert np.array_equal(got, g["out"])
    assert np.array_equal(np.signbit(got), np.signbit(g["out"]))


SQUEEZES = [(2, 8), (2, 12), (2, 16), (4, 16), (4, 32), (8, 32), (8, 64), (16, 64), (16, 128)]


@pytest.mark.gpu
@pytest.mark.parametrize("P,pp", SQUEEZES)
def test_gpu_squeeze_wrappers_match_reference(prog, tmp_path, P, pp):
    """pllsqueeze_old and pllsqueeze (TCcuda.cu:908, 810) through the
    wrappers; for double-double also pllsqueeze_2_{8,12,16} (TCcuda.cu:412)."""
    g = np.load(os.path.join(GOLDEN, f"squeeze_P{P}_pp{pp}.npz"))
    hows = ["old", "any"] + (["dd"] if P == 2 else [])
    for how in hows:
        got = _roundtrip(prog, tmp_path, ["gsqueeze", how, P, pp], [g["x"]], g["y"].shape)
        assert np.array_equal(got, g["y"]), how


@pytest.mark.gpu
@pytest.mark.parametrize("P,pp", SQUEEZES)
def test_gpu_exported_squeeze_kernels_match_reference(prog, tmp_path, P, pp):
    """pllsqueeze_{2,4,8,16}_pp_old (TCcuda.cu:876-906) launched by the caller
    with exactly one thread per entry."""
    g = np.load(os.path.join(GOLDEN, f"squeeze_P{P}_pp{pp}.npz"))
    count = g["x"].shape[0]
    got = _roundtrip(prog, tmp_path, ["ksqpp", P, pp, count // 16, 16], [g["x"]], g["y"].shape)
    assert np.array_equal(got, g["y"])


@pytest.mark.gpu
@pytest.mark.parametrize("pp", [8, 12, 16])
def test_gpu_separate_plane_squeeze_kernels(prog, tmp_path, orc, pp):
    """pllsqueeze_kernel_2_{8,12,16} (TCcuda.cu:400, 508, 646) on the
    reference's golden partials, and on 1000 entries launched as <<<8, 125>>>
    (a count that is not a multiple of a power-of-two block), against the
    oracle's squeeze; these kernels have no bounds check, so the launch
    covers exactly the entries."""
    g = np.load(os.path.join(GOLDEN, f"squeeze_P2_pp{pp}.npz"))
    count = g["x"].shape[0]
    got = _roundtrip(prog, tmp_path, ["ksq2", pp, count // 16, 16], [g["x"]], g["y"].shape)
    assert np.array_equal(got, g["y"])
    rng = np.random.default_rng(pp)
    x = np.ldexp(rng.uniform(-1, 1, size=(1000, pp)), -13 * np.arange(pp))
    got = _roundtrip(prog, tmp_path, ["ksq2", pp, 8, 125], [x], (1000, 2))
    assert np.array_equal(got, orc.squeeze(2, pp, x))


@pytest.mark.gpu
@pytest.mark.parametrize("P", [2, 4, 8, 16])
@pytest.mark.parametrize("which,golden", [("A", "renormhost"), ("bigA", "renormhostbig")])
def test_gpu_exported_renorm_kernels_match_reference(prog, tmp_path, P, which, golden):
    """renormA / renormbigA (TCcuda.cu:97-117), one block of n x n threads,
    against the reference's host renormhost / renormhostbig of the same
    pass (not an error-free transform; kept as the reference defines it)."""
    g = np.load(os.path.join(GOLDEN, f"hostfuncs_P{P}.npz"))
    n = int(g["n"])
    got = _roundtrip(prog, tmp_path, ["krenorm", which, P, n], [g["A"]])
    assert np.array_equal(got, g[golden])
    assert np.array_equal(np.signbit(got), np.signbit(g[golden]))
