"""mdg_gemm_ex: transposed operands and C (+)= op(A) op(B).  The result must
equal mdg_gemm of the same form on explicitly transposed operands (bit for
bit: the transposes are exact copies), followed by the oracle's P-double
addition (the reference's *_add) when accumulating."""
import ctypes

import numpy as np
import pytest

from conftest import pkg


def test_gemm_ex_arguments_without_gpu():
    L = pkg("_lib").lib()
    one = ctypes.c_void_p(8)
    ex = L.mdg_gemm_ex
    # trans_a: A is stored k x m, so lda >= m (here m = 6 > k = 4)
    assert ex(0, 1, 0, 0, 4, 6, 5, 4, one, 4, one, 5, one, 5, None, None, 0, None) == 2
    # trans_b: B is stored n x k, so ldb >= k
    assert ex(0, 0, 1, 0, 4, 6, 5, 4, one, 4, one, 3, one, 5, None, None, 0, None) == 2
    assert ex(0, 2, 0, 0, 4, 6, 5, 4, one, 6, one, 5, one, 5, None, None, 0, None) == 4
    assert ex(0, 0, 0, 3, 4, 6, 5, 4, one, 4, one, 5, one, 5, None, None, 0, None) == 4
    assert ex(5, 0, 0, 0, 4, 6, 5, 4, one, 4, one, 5, one, 5, None, None, 0, None) == 4
    assert ex(0, 0, 0, 0, 3, 6, 5, 4, one, 4, one, 5, one, 5, None, None, 0, None) == 1
    assert ex(0, 0, 0, 0, 4, 0, 5, 4, None, 4, None, 5, None, 5, None, None, 0, None) == 0
    assert ex(0, 0, 0, 1, 4, 6, 5, 4, one, 4, one, 5, None, 5, None, None, 0, None) == 3
    # plain form: workspace only for the copies and the product
    assert ex(0, 1, 0, 0, 4, 6, 5, 4, one, 6, one, 5, one, 5, None, None, 0, None) == 5
    size = L.mdg_gemm_ex_workspace_size
    assert size(0, 0, 0, 0, 4, 64, 32, 16, None) == 0
    assert size(0, 1, 0, 0, 4, 64, 32, 16, None) == 64 * 16 * 4 * 8
    assert size(0, 1, 1, 1, 4, 64, 32, 16, None) == (64 * 16 + 16 * 32 + 64 * 32) * 4 * 8
    inner = L.mdg_gemm_workspace_size(2, 4, 64, 32, 16, None)
    assert size(2, 0, 0, 1, 4, 64, 32, 16, None) >= inner + 64 * 32 * 4 * 8


def host(t):
    return t.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["plain", "fp64split", "slice_bf16"])
@pytest.mark.parametrize("P", [2, 4])
@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("acc", [0, 1])
def test_gemm_ex_matches_gemm_on_transposed_operands(orc, inputs, form, P, ta, tb, acc):
    import torch
    api = pkg("api")
    m, n, k = 37, 29, 45
    rng = np.random.default_rng(P * 10 + ta * 4 + tb * 2 + acc)
    A = inputs.uniform_pd(rng, (m, k), P)
    B = inputs.uniform_pd(rng, (k, n), P)
    C0 = inputs.uniform_pd(rng, (m, n), P)
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    ref = host(api.gemm(dev(A), dev(B), form))
    if acc:
        ref = orc.vec_op("add", P, C0, ref).reshape(m, n, P)
    # stored operands, with padded rows (leading dimension > minimum)
    As = np.swapaxes(A, 0, 1) if ta else A
    Bs = np.swapaxes(B, 0, 1) if tb else B
    padA = torch.full((As.shape[0], As.shape[1] + 3, P), 5.0, dtype=torch.float64, device="cuda")
    padB = torch.full((Bs.shape[0], Bs.shape[1] + 1, P), 5.0, dtype=torch.float64, device="cuda")
    padA[:, :As.shape[1]] = dev(As)
    padB[:, :Bs.shape[1]] = dev(Bs)
    padC = torch.full((m, n + 2, P), 9.0, dtype=torch.float64, device="cuda")
    padC[:, :n] = dev(C0)
    got = api.gemm_ex(padA[:, :As.shape[1]], padB[:, :Bs.shape[1]], form, trans_a=bool(ta),
                      trans_b=bool(tb), C=padC[:, :n], accumulate=bool(acc))
    assert np.array_equal(host(got), ref)
    assert torch.all(padC[:, n:] == 9.0)
    assert api.device_status() == 0


@pytest.mark.gpu
def test_gemm_ex_large_slice_accumulate_twice(orc, inputs):
    """C = 0, then C (+)= A B twice with A transposed: equals the oracle's
    add of the two (identical) products."""
    import torch
    api = pkg("api")
    P, m, n, k = 4, 300, 260, 130
    rng = np.random.default_rng(300)
    A = inputs.normal_pd(rng, (m, k), P)
    B = inputs.uniform_pd(rng, (k, n), P)
    dA = torch.from_numpy(np.ascontiguousarray(np.swapaxes(A, 0, 1))).cuda()
    dB = torch.from_numpy(B).cuda()
    prod = host(api.gemm(torch.from_numpy(A).cuda(), dB, "slice_bf16"))
    C = torch.zeros((m, n, P), dtype=torch.float64, device="cuda")
    api.gemm_ex(dA, dB, "slice_bf16", trans_a=True, C=C, accumulate=True)
    assert np.array_equal(host(C), orc.vec_op("add", P, np.zeros_like(prod), prod).reshape(m, n, P))
    api.gemm_ex(dA, dB, "slice_bf16", trans_a=True, C=C, accumulate=True)
    once = orc.vec_op("add", P, np.zeros_like(prod), prod)
    assert np.array_equal(host(C), orc.vec_op("add", P, once, prod).reshape(m, n, P))
