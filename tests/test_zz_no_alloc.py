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
        st = L.mdg_gemm_slice_static(P, m, n, k, ctypes.c_void_p(dA.data_ptr()), k,
                                     ctypes.c_void_p(dB.data_ptr()), n,
                                     ctypes.c_void_p(C.data_ptr()), n,
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == 0, L.mdg_status_string(st)
        torch.cuda.synchronize()
        assert torch.equal(C, ref), name


@pytest.mark.gpu
def test_static_scratch_entry_rejects_oversize():
    L = pkg("_lib").lib()
    assert L.mdg_static_scratch_bytes() == 64 << 20
    one = ctypes.c_void_p(256)
    # quad-double 1024^3 needs more than the fixed scratch: refused up front
    assert L.mdg_gemm_slice_static(4, 1024, 1024, 1024, one, 1024, one, 1024, one, 1024,
                                   None) == 10
    assert b"scratch" in L.mdg_status_string(10)
