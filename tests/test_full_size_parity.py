"""Parity at the benchmark sizes: every form run on the whole matrices of
the named workloads, a sampled block of C compared with the oracle.

The slice-digit form scales row r of A by 2^-E[r] (E from that row alone)
and column c of B by 2^-F[c]; each entry of C depends only on its row of A
and its column of B.  The oracle run on A[rows] and B[:, cols] therefore
computes exactly the sampled block of the full-size product, so the block
is compared bit for bit.  The plain form is per entry as well (bit for
bit).  The FP64 split form sums its slice products in the DMMA unit's
order; its block must reach the oracle's error bits within 2 bits, the
tolerance of the small-size test.

Workloads (quad-double 1024^3 seed 1, octo-double 2048^3 seed 2 with row
and column scales 2^U{-32..32}, quad-double 8192^3 seed 4 with N(0, 1) hi
limbs, double-double 64^3 seed 0, and the 256 mixed problems of seed 3):
synthetic seeded inputs with the benchmark's shapes and distributions.
"""
import numpy as np
import pytest
import torch

from conftest import pkg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a GPU")
    return pkg("api")


def sample(count, size, seed):
    """`count` sorted indices in [0, size): the first, the last (in the
    tail tile) and the rest drawn without repetition."""
    rng = np.random.default_rng(seed)
    pick = {0, size - 1}
    for v in rng.permutation(size):
        if len(pick) >= min(count, size):
            break
        pick.add(int(v))
    return np.array(sorted(pick))


def block_inputs(A, B, rows, cols):
    return np.ascontiguousarray(A[rows]), np.ascontiguousarray(B[:, cols])


@pytest.mark.parametrize("name", ["dd64", "qd1024", "od2048_spread", "qd8192_normal"])
def test_slice_form_full_size_block_bit_exact(api, orc, inputs, name):
    P, A, B = inputs.workload(name)
    m, k = A.shape[:2]
    n = B.shape[1]
    s = api.default_slices(P)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    C = api.gemm(dA, dB, "slice_bf16")
    assert api.device_status() == 0
    rows, cols = sample(16, m, 11), sample(16, n, 13)
    got = C[torch.from_numpy(rows).cuda()][:, torch.from_numpy(cols).cuda()].cpu().numpy()
    del C, dA, dB
    torch.cuda.empty_cache()
    Ab, Bb = block_inputs(A, B, rows, cols)
    want = orc.gemm_slices(P, s, s, Ab, Bb, len(rows), len(cols), k)
    assert np.array_equal(got, want), name
    assert np.array_equal(np.signbit(got), np.signbit(want))


@pytest.mark.parametrize("name", ["dd64", "qd1024", "od2048_spread"])
def test_fp64_digit_form_full_size_block_bit_exact(api, orc, inputs, name):
    """The FP64 DMMA digit form on the whole workload; its exponents and
    digits are per row / column like the BF16 form's, so the sampled block
    equals the oracle on the block's rows and columns bit for bit."""
    P, A, B = inputs.workload(name)
    m, k = A.shape[:2]
    n = B.shape[1]
    s = api.default_slices(P, "fp64_digits")
    C = api.gemm(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), "fp64_digits")
    rows, cols = sample(8, m, 41), sample(8, n, 43)
    got = C.cpu().numpy()[np.ix_(rows, cols)]
    del C
    torch.cuda.empty_cache()
    Ab, Bb = block_inputs(A, B, rows, cols)
    assert np.array_equal(got, orc.gemm_digits(P, s, s, Ab, Bb, len(rows), len(cols), k)), name


@pytest.mark.parametrize("name", ["dd64", "qd1024"])
def test_plain_form_full_size_block_bit_exact(api, orc, inputs, name):
    P, A, B = inputs.workload(name)
    m, k = A.shape[:2]
    n = B.shape[1]
    C = api.gemm(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), "plain").cpu().numpy()
    rows, cols = sample(12, m, 17), sample(12, n, 19)
    Ab, Bb = block_inputs(A, B, rows, cols)
    want = orc.gemm_plain(P, Ab, Bb, len(rows), len(cols), k)
    assert np.array_equal(C[np.ix_(rows, cols)], want), name


@pytest.mark.parametrize("name", ["qd1024", "od2048_spread"])
def test_fp64split_form_full_size_block_error_bits(api, orc, inputs, name):
    ex = pkg("errors")
    P, A, B = inputs.workload(name)
    m, k = A.shape[:2]
    n = B.shape[1]
    C = api.gemm(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), "fp64split")
    rows, cols = sample(6, m, 23), sample(6, n, 29)
    got = C.cpu().numpy()[np.ix_(rows, cols)]
    del C
    torch.cuda.empty_cache()
    Ab, Bb = block_inputs(A, B, rows, cols)
    want = orc.gemm_fp64split(P, Ab, Bb, len(rows), len(cols), k)
    r, c = range(len(rows)), range(len(cols))
    bits = ex.error_bits(got, Ab, Bb, r, c)
    bits_ref = ex.error_bits(want, Ab, Bb, r, c)
    print(name, "fp64split", bits, "oracle", bits_ref)
    assert bits[1] >= bits_ref[1] - 2.0, (bits, bits_ref)


def test_batched_workload_equals_single_problem_gemms(api, orc, inputs):
    """The whole 256-problem batched workload (seed 3) as one plan, tuned
    (tile policy and split mode) and replayed: every problem's C equals its
    single-problem BF16 GEMM bit for bit, and a sampled block of one
    octo-double problem equals the oracle."""
    probs, rng = inputs.batched_problems(256, seed=3)
    ops = [(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda())
           for A, B in inputs.batched_operands(probs, rng)]
    plan = api.BatchPlan(ops)
    api.tune_cache_clear()
    plan.tune()
    api.tune_cache_clear()
    for C in plan.Cs:
        C.fill_(float("nan"))
    plan.run()
    torch.cuda.synchronize()
    assert api.device_status() == 0
    for i, ((A, B), C) in enumerate(zip(ops, plan.Cs)):
        assert torch.equal(C, api.gemm(A, B, "slice_bf16")), (i, probs[i])
    i = next(j for j, pr in enumerate(probs) if pr[0] == 8)
    P, m, n, k = probs[i]
    rows, cols = sample(6, m, 47), sample(6, n, 53)
    Ab, Bb = block_inputs(ops[i][0].cpu().numpy(), ops[i][1].cpu().numpy(), rows, cols)
    s = api.default_slices(P)
    got = plan.Cs[i].cpu().numpy()[np.ix_(rows, cols)]
    assert np.array_equal(got, orc.gemm_slices(P, s, s, Ab, Bb, len(rows), len(cols), k))
