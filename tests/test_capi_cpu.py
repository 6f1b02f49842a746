"""C ABI checks that need no GPU: the library loads, exports every function
include/mdgemm.h declares, and rejects bad arguments before any CUDA call."""
import ctypes
import re

import pytest

from conftest import pkg


@pytest.fixture(scope="module")
def L():
    return pkg("_lib").lib()


def declared_functions():
    src = open(pkg("_lib").HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mdg_[a-z_0-9]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(L):
    names = declared_functions()
    assert len(names) >= 17
    for name in names:
        assert hasattr(L, name), name
    assert set(names) == set(pkg("_lib").SIGNATURES), "ctypes table out of sync with header"


def test_status_strings(L):
    assert L.mdg_status_string(0) == b"success"
    assert b"limb" in L.mdg_status_string(1)
    assert L.mdg_status_string(12345) == b"unknown status"
    assert L.mdg_version() >= 100


def test_default_slices(L):
    assert [L.mdg_default_slices(p) for p in (2, 4, 8, 16)] == [14, 28, 55, 110]
    assert L.mdg_default_slices(3) == 0
    assert [L.mdg_default_fp64_digits(p) for p in (2, 4, 8, 16)] == [6, 12, 24, 47]
    # the FP64 digit form's workspace: digit planes (8 B a digit), int64
    # diagonal sums, exponents
    ws = L.mdg_gemm_workspace_size(3, 4, 100, 80, 60, None)
    assert ws >= 12 * (100 + 80) * 60 * 8 + 12 * 100 * 80 * 8


@pytest.mark.parametrize("p", [0, 1, 3, 5, 32, -2])
def test_bad_limb_count_rejected(L, p):
    assert L.mdg_gemm(0, p, 4, 4, 4, None, 4, None, 4, None, 4, None, None, 0, None) == 1
    assert L.mdg_split(0, 0, p, 4, None, None, None) == 1
    assert L.mdg_squeeze(p, 8, 4, None, None, None) == 1


def test_bad_sizes_and_pointers_rejected(L):
    one = ctypes.c_void_p(1)
    assert L.mdg_gemm(0, 4, -1, 4, 4, one, 4, one, 4, one, 4, None, None, 0, None) == 2
    assert L.mdg_gemm(0, 4, 4, 4, 8, one, 4, one, 4, one, 4, None, None, 0, None) == 2  # lda < k
    assert L.mdg_gemm(0, 4, 4, 4, 4, None, 4, one, 4, one, 4, None, None, 0, None) == 3
    assert L.mdg_gemm(7, 4, 4, 4, 4, one, 4, one, 4, one, 4, None, None, 0, None) == 4
    assert L.mdg_gemm(1, 4, 4, 4, 4, one, 4, one, 4, one, 4, None, None, 0, None) == 5  # no workspace
    assert L.mdg_gemm(2, 4, 4, 4, 4, one, 4, one, 4, one, 4, None, None, 0, None) == 5
    assert L.mdg_split(2, 0, 4, 4, one, one, None) == 1   # mixed split needs P = 2
    assert L.mdg_split(0, 3, 4, 4, one, one, None) == 4
    assert L.mdg_squeeze(4, 0, 4, one, one, None) == 2
    assert L.mdg_slice_diagonals(4, 4, 100, 128, 64, one, one, 64, 1, 1, one, None) == 2
    # digit planes that would overlap (plane stride below rows x ld)
    assert L.mdg_slice_diagonals(4, 4, 128, 256, 64, one, one, 64, 128 * 64 - 1, 256 * 64,
                                 one, None) == 2
    assert L.mdg_slice_diagonals(4, 4, 128, 256, 64, one, one, 64, 128 * 64, 256 * 64 - 64,
                                 one, None) == 2


def test_empty_problems_succeed_without_gpu(L):
    assert L.mdg_gemm(0, 4, 0, 5, 5, None, 5, None, 5, None, 5, None, None, 0, None) == 0
    assert L.mdg_split(0, 0, 4, 0, None, None, None) == 0
    assert L.mdg_squeeze(4, 16, 0, None, None, None) == 0


def test_workspace_sizes(L):
    api = pkg("api")
    assert api.workspace_size("plain", 4, 64, 64, 64) == 0
    ws_split = api.workspace_size("fp64split", 4, 64, 64, 64)
    assert ws_split >= 16 * 3 * 64 * 64 * 8
    ws_tc = api.workspace_size("slice_bf16", 4, 64, 64, 64)
    # digits of A and B (28 planes of 128 x 64 BF16) + 28 diagonal planes
    assert ws_tc >= 2 * 28 * 128 * 64 * 2 + 28 * 128 * 128 * 8
    assert api.workspace_size("slice_bf16", 4, 64, 64, 64, slices=200) == 0


def test_chunk_counts(L):
    """Diagonal d (pairs_d digit pairs, k/64 steps each) is cut into int32
    chunks of at most 2032 steps: quad-double at k = 8192 has 15 diagonals
    of one chunk and 13 of two."""
    count = L.mdg_slice_chunk_count
    assert count(1, 1, 2032 * 64) == 1 and count(1, 1, 2032 * 64 + 1) == 2
    assert count(1, 1, 2 * 2032 * 64 + 640) == 3
    assert count(28, 28, 8192) == 15 + 2 * 13
    assert count(28, 28, 0) == 28  # k = 0: one (empty) step per pair
    assert count(28, 56, 64) == 0 and count(0, 1, 64) == 0


@pytest.mark.parametrize("field,value", [("engine", 4), ("engine", -1), ("parts", 9), ("parts", -1),
                                         ("raster", -1), ("split_exact", 3), ("pace", -2),
                                         ("pace", 65537)])
def test_bad_options_rejected(L, field, value):
    """Out-of-range mdg_options fields: no workspace size, and mdg_gemm
    returns MDG_ERROR_INVALID_FORM before touching the device."""
    api = pkg("api")
    o = api._opts()
    setattr(o, field, value)
    assert L.mdg_gemm_workspace_size(2, 4, 64, 64, 64, ctypes.byref(o)) == 0
    one = ctypes.c_void_p(1)
    assert L.mdg_gemm(2, 4, 4, 4, 4, one, 4, one, 4, one, 4, ctypes.byref(o), None, 0, None) == 4


def test_schedule_options_accepted(L):
    """parts, raster and engine choices inside their ranges resolve."""
    api = pkg("api")
    base = api.workspace_size("slice_bf16", 4, 512, 512, 512)
    for kw in ({"engine": "tc_pair", "parts": 8, "raster": 1000}, {"engine": "mma_sync"},
               {"engine": "tc", "parts": 1, "raster": 1}, {"pace": -1}, {"pace": 128}):
        assert api.workspace_size("slice_bf16", 4, 512, 512, 512, **kw) == base


def test_allocation_cap_simulates_out_of_memory(L, monkeypatch):
    """Host-side fault injection: MDG_ALLOC_LIMIT_BYTES makes the library's
    own allocations (the host entry's buffers, plan workspaces, page-locked
    host buffers) fail with MDG_ERROR_ALLOCATION before any CUDA call."""
    import numpy as np
    monkeypatch.setenv("MDG_ALLOC_LIMIT_BYTES", "1024")
    A = np.zeros((64, 64, 4))
    C = np.zeros((64, 64, 4))
    ptr = lambda a: ctypes.c_void_p(a.ctypes.data)
    for form in (0, 1, 2):
        assert L.mdg_gemm_host(form, 4, 64, 64, 64, ptr(A), ptr(A), ptr(C), None) == 9
    h = ctypes.c_void_p()
    assert L.mdg_plan_create(2, 4, 64, 64, 64, None, ctypes.byref(h)) == 9
    # page-locked host buffers count too
    p = ctypes.c_void_p(1)
    assert L.mdg_host_alloc(4096, ctypes.byref(p)) == 9 and p.value is None
    assert L.mdg_host_alloc(8, None) == 3
    assert L.mdg_status_string(9) == b"allocation failed"


def test_plain_c_program_builds_and_links(tmp_path):
    """The C ABI from C99: the header compiles with -pedantic, and a C
    program linked against libmdgemm.so calls entries that need no GPU."""
    import os
    import shutil
    import subprocess
    from conftest import ROOT
    cc = shutil.which("gcc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    lib = pkg("_lib").LIB_PATH
    src = tmp_path / "abi.c"
    src.write_text(
        '#include <stdio.h>\n#include <string.h>\n#include "mdgemm.h"\n'
        "int main(void) {\n"
        "  mdg_options o;\n  memset(&o, 0, sizeof o);\n"
        "  if (mdg_version() < 100) return 1;\n"
        "  if (mdg_default_slices(4) != 28) return 2;\n"
        "  if (mdg_gemm(MDG_FORM_PLAIN, 3, 4, 4, 4, NULL, 4, NULL, 4, NULL, 4, &o, NULL, 0, NULL)\n"
        "      != MDG_ERROR_INVALID_LIMBS) return 3;\n"
        '  printf("%s\\n", mdg_status_string(MDG_ERROR_WORKSPACE));\n'
        "  return 0;\n}\n")
    exe = tmp_path / "abi"
    libdir = os.path.dirname(lib)
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                    "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
                    str(src), "-L", libdir, "-lmdgemm", "-Wl,-rpath," + libdir, "-o", str(exe)],
                   check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert "workspace" in r.stdout


def _table(probs):
    Problem = pkg("_lib").Problem
    t = (Problem * len(probs))()
    for i, (p, m, n, k) in enumerate(probs):
        # stand-in pointers: every call below returns before touching them
        t[i] = Problem(p, m, n, k, 16, 16, 16, max(k, 1), max(n, 1), max(n, 1))
    return t


def test_batch_plan_sizes_and_arguments(L):
    """The batched plan (mdg_batch_*) and the one-call batched entry size
    their workspace and check every problem on the host; mixed P including
    hexa-double is accepted."""
    t = _table([(16, 40, 50, 70), (2, 32, 32, 32), (8, 100, 300, 64), (4, 1, 1, 1)])
    full = L.mdg_batch_workspace_size(t, 4)
    assert full > 0
    sizes = [L.mdg_batch_workspace_size(t, c) for c in range(1, 5)]
    assert sizes == sorted(set(sizes)) and sizes[-1] == full  # each problem adds its planes
    assert L.mdg_gemm_batched_workspace_size(2, t, 4, None) == full
    assert L.mdg_batch_workspace_size(t, 0) == 0
    assert L.mdg_batch_workspace_size(None, 2) == 0
    assert L.mdg_batch_workspace_size(_table([(3, 8, 8, 8)]), 1) == 0
    assert L.mdg_batch_workspace_size(_table([(4, 0, 8, 8)]), 1) == 0
    h = ctypes.c_void_p()
    assert L.mdg_batch_create(t, 4, None, 0, None, None) == 3
    assert L.mdg_batch_create(t, 0, None, 0, None, ctypes.byref(h)) == 2
    assert L.mdg_batch_create(_table([(3, 8, 8, 8)]), 1, None, 0, None, ctypes.byref(h)) == 1
    assert L.mdg_batch_create(t, 4, None, full, None, ctypes.byref(h)) == 5
    assert L.mdg_batch_create(t, 4, ctypes.c_void_p(256), full - 1, None, ctypes.byref(h)) == 5
    assert not h.value
    assert L.mdg_batch_run(None, None) == 3
    assert L.mdg_batch_set_split(None, 1, None) == 3 and L.mdg_batch_split(None) == -1
    assert L.mdg_batch_set_tiles(None, 1, None) == 3 and L.mdg_batch_tiles(None) == -1
    L.mdg_batch_destroy(None)
    assert L.mdg_gemm_batched(2, t, -1, None, None, 0, None) == 2
    assert L.mdg_gemm_batched(2, t, 0, None, None, 0, None) == 0
    assert L.mdg_gemm_batched(2, None, 3, None, None, 0, None) == 3
    assert L.mdg_gemm_batched(2, _table([(3, 8, 8, 8)]), 1, None, None, 0, None) == 1
    assert L.mdg_gemm_batched(7, t, 4, None, None, 0, None) == 4
    assert L.mdg_gemm_batched(2, t, 4, None, None, 0, None) == 5
