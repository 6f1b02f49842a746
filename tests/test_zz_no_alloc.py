"""The allocation-free entry point, mdg_gemm_slice_static, through the C ABI.

It exists for callers that may not allocate device memory (a stream capture
owned by another component, hosts that own all device allocations); it
computes the BF16 slice-digit GEMM in a fixed scratch array inside the
library.  Its result must equal the workspace entry's (mdg_gemm, BF16
form) bit for bit -- the tolerance every slice-form test here uses -- on
two calls in a row with different problems, so that contents the first
call leaves in the shared scratch cannot leak into the second.  This file
sorts last so that a run stopping at the first failure has run the rest.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import pkg


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _static(L, P, m, n, k, A, lda, B, ldb, C, ldc):
    return L.mdg_gemm_slice_static(P, m, n, k, _vp(A), lda, _vp(B), ldb, _vp(C), ldc,
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


@pytest.mark.gpu
def test_static_scratch_entry_matches_workspace_entry():
    assert torch.cuda.is_available(), "a GPU test ran without a GPU"
    L = pkg("_lib").lib()
    api, inputs = pkg("api"), pkg("inputs")
    cases = [("qd1024", 200, 300, 250), ("dd64", 131, 97, 513)]
    for name, m, n, k in cases:
        P, A, B = inputs.workload(name, m, n, k)
        dA = torch.from_numpy(A).cuda()
        dB = torch.from_numpy(B).cuda()
        ref = api.gemm(dA, dB, "slice_bf16")
        C = torch.full((m, n, P), np.nan, dtype=torch.float64, device="cuda")
        st = _static(L, P, m, n, k, dA, k, dB, n, C, n)
        assert st == 0, L.mdg_status_string(st)
        torch.cuda.synchronize()
        assert torch.equal(C, ref), name


@pytest.mark.gpu
def test_static_scratch_entry_leading_dimensions_and_empty_sum():
    """Padded rows (lda > k, ldb > n, ldc > n) against mdg_gemm at the same
    leading dimensions, bit for bit, with the padding of C left alone; then
    k = 0, which clears C in place."""
    L = pkg("_lib").lib()
    inputs = pkg("inputs")
    P, A, B = inputs.workload("od2048_spread", 90, 70, 130)
    m, k = A.shape[:2]
    n = B.shape[1]
    lda, ldb, ldc = k + 7, n + 3, n + 5
    Aw = torch.zeros((m, lda, P), dtype=torch.float64, device="cuda")
    Bw = torch.zeros((k, ldb, P), dtype=torch.float64, device="cuda")
    Aw[:, :k] = torch.from_numpy(A).cuda()
    Bw[:, :n] = torch.from_numpy(B).cuda()
    ref = torch.full((m, ldc, P), 5.0, dtype=torch.float64, device="cuda")
    need = L.mdg_gemm_workspace_size(2, P, m, n, k, None)
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    st = L.mdg_gemm(2, P, m, n, k, _vp(Aw), lda, _vp(Bw), ldb, _vp(ref), ldc, None, _vp(ws),
                    need, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, L.mdg_status_string(st)
    C = torch.full((m, ldc, P), 5.0, dtype=torch.float64, device="cuda")
    assert _static(L, P, m, n, k, Aw, lda, Bw, ldb, C, ldc) == 0
    torch.cuda.synchronize()
    assert torch.equal(C, ref)
    assert torch.all(C[:, n:] == 5.0)
    # k = 0: the empty sum, C = 0 on the m x n entries only
    assert _static(L, P, m, n, 0, Aw, 1, Bw, ldb, C, ldc) == 0
    torch.cuda.synchronize()
    assert torch.all(C[:, :n] == 0) and torch.all(C[:, n:] == 5.0)


def test_static_scratch_entry_rejects_oversize():
    """The size check runs on the host before any device access, so this
    runs without a GPU: the fixed scratch is 64 MiB, quad-double fits up to
    512^3, octo- and hexa-double up to 256^3; larger problems are refused."""
    L = pkg("_lib").lib()
    cap = L.mdg_static_scratch_bytes()
    assert cap == 64 << 20
    ws = L.mdg_gemm_workspace_size
    assert ws(2, 4, 512, 512, 512, None) <= cap < ws(2, 4, 513, 513, 513, None)
    assert ws(2, 8, 256, 256, 256, None) <= cap < ws(2, 8, 257, 257, 257, None)
    assert ws(2, 16, 256, 256, 256, None) <= cap
    one = ctypes.c_void_p(256)
    # quad-double 1024^3 and 513^3 need more than the fixed scratch: refused up front
    for size in (1024, 513):
        assert L.mdg_gemm_slice_static(4, size, size, size, one, size, one, size, one, size,
                                       None) == 10
    assert L.mdg_gemm_slice_static(8, 257, 257, 257, one, 257, one, 257, one, 257, None) == 10
    assert b"scratch" in L.mdg_status_string(10)
    # argument checks mirror mdg_gemm's
    assert L.mdg_gemm_slice_static(3, 4, 4, 4, one, 4, one, 4, one, 4, None) == 1
    assert L.mdg_gemm_slice_static(4, 4, 4, 4, one, 3, one, 4, one, 4, None) == 2
    assert L.mdg_gemm_slice_static(4, 4, 4, 4, None, 4, one, 4, one, 4, None) == 3
