"""GPU parity: every stage and every form through the C ABI against the
oracle (and, through the golden files, against the reference itself).

Tolerances: the plain form, the floatybits split, the squeeze and every
stage of the slice-digit form are bit-exact (compared with ==, NaN-free
inputs).  The FP64 DMMA slice convolution rounds its FP64 sums in the
tensor core's own order; it must agree with the oracle's sequential sum to
2^-50 relative to sum |a||b| per entry, and the whole FP64-split GEMM must
reach the oracle's error bits within 2 bits.  The slice-digit form must
reach at least the plain form's normwise error bits minus 1 against the
exact product.
"""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN, pkg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a GPU")
    return pkg("api")


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.cpu().numpy()


SHAPES = [(1, 1, 1), (7, 5, 3), (31, 33, 17), (33, 31, 64), (64, 64, 64), (16, 48, 129)]


# ------------------------------------------------------------------ plain --

@pytest.mark.parametrize("P", [2, 4, 8, 16])
@pytest.mark.parametrize("shape", SHAPES)
def test_plain_bit_exact(api, orc, inputs, P, shape):
    m, n, k = shape
    if P == 16 and m * n * k > 40000:
        pytest.skip("hd oracle cost")
    rng = np.random.default_rng(m * 1000 + n * 10 + k + P)
    A = inputs.uniform_pd(rng, (m, k), P)
    B = inputs.uniform_pd(rng, (k, n), P)
    C = host(api.gemm(dev(A), dev(B), "plain"))
    assert np.array_equal(C, orc.gemm_plain(P, A, B, m, n, k))


@pytest.mark.parametrize("P", [2, 4, 8, 16])
def test_plain_matches_reference_golden(api, P):
    g = np.load(os.path.join(GOLDEN, f"matmul_P{P}.npz"))
    C = host(api.gemm(dev(g["A"]), dev(g["B"]), "plain"))
    assert np.array_equal(C, g["C"], equal_nan=True)


def test_plain_dd64_workload_matches_reference(api):
    g = np.load(os.path.join(GOLDEN, "matmul_dd64.npz"))
    C = host(api.gemm(dev(g["A"]), dev(g["B"]), "plain"))
    assert np.array_equal(C, g["C"])


def test_matmulTCnt_mirror(api, inputs, orc):
    P, A, B = inputs.workload("qd1024", 40, 40, 40)
    C, t = api.matmulTCnt(A.ravel(), B.ravel(), 40, 32, P, loop_ct=2)
    assert t > 0
    assert np.array_equal(C.reshape(40, 40, P), orc.gemm_plain(P, A, B, 40, 40, 40))


def test_plain_batched_mixed(api, orc, inputs):
    probs, rng = inputs.batched_problems(12, seed=5)
    probs = [(P, m // 8, n // 8, k // 8) for P, m, n, k in probs]
    ops = inputs.batched_operands(probs, rng)
    Cs = api.gemm_batched([(dev(A), dev(B)) for A, B in ops], "plain")
    for (P, m, n, k), (A, B), C in zip(probs, ops, Cs):
        assert np.array_equal(host(C), orc.gemm_plain(P, A, B, m, n, k))


# ---------------------------------------------------------- FP64 split --

@pytest.mark.parametrize("P", [2, 4, 8, 16])
@pytest.mark.parametrize("kind", ["split4", "split8"])
@pytest.mark.parametrize("style", ["", "_refstyle"])
def test_split_matches_reference_golden(api, P, kind, style):
    g = np.load(os.path.join(GOLDEN, f"{kind}_P{P}{style}.npz"))
    fn = api.split4pd if kind == "split4" else api.split8pd
    out = host(fn(g["x"], P))
    assert np.array_equal(out, g["out"])
    assert np.array_equal(np.signbit(out), np.signbit(g["out"]))


def test_mixsplit_matches_reference_golden(api):
    g = np.load(os.path.join(GOLDEN, "split_mix_P2.npz"))
    out = host(api.mixsplit2(g["x"]))
    assert np.array_equal(out, g["out"]) and np.array_equal(np.signbit(out), np.signbit(g["out"]))


@pytest.mark.parametrize("P", [2, 4, 8])
@pytest.mark.parametrize("kind", ["split4", "split8"])
def test_exact_split_matches_oracle(api, orc, inputs, P, kind):
    rng = np.random.default_rng(P)
    x = inputs.uniform_pd(rng, (300,), P)
    fn = api.split4pd if kind == "split4" else api.split8pd
    out = host(fn(x, P, exact=True))
    ref = orc.split(kind, P, x, exact=True)
    assert np.array_equal(out, ref) and np.array_equal(np.signbit(out), np.signbit(ref))
    # exact slices sum back to the value (balancing moves units between
    # neighbouring slices, also across limbs, so only the total is kept)
    from fractions import Fraction
    for i in range(0, 300, 37):
        assert sum(map(Fraction, out[i])) == sum(map(Fraction, x[i]))


@pytest.mark.parametrize("P,pp", [(2, 8), (2, 16), (4, 16), (4, 32), (8, 32), (8, 64),
                                  (16, 64), (16, 128)])
def test_squeeze_matches_reference_golden(api, P, pp):
    g = np.load(os.path.join(GOLDEN, f"squeeze_P{P}_pp{pp}.npz"))
    assert np.array_equal(host(api.pllsqueeze_old(g["x"], P, pp)), g["y"])


@pytest.mark.parametrize("pp,shape", [(16, (8, 8, 8)), (16, (33, 17, 40)), (8, (64, 64, 64)),
                                      (12, (20, 9, 31))])
def test_slice_conv_against_oracle(api, orc, inputs, pp, shape):
    m, n, k = shape
    P = {16: 4, 8: 2, 12: 2}[pp]
    kind = {16: "split4", 8: "split4", 12: "mix"}[pp]
    rng = np.random.default_rng(pp + m)
    A = inputs.uniform_pd(rng, (m, k), P)
    B = inputs.uniform_pd(rng, (k, n), P)
    Aq = orc.split(kind, P, A.reshape(-1, P), exact=True).reshape(m, k, pp)
    Bq = orc.split(kind, P, B.reshape(-1, P), exact=True).reshape(k, n, pp)
    got = host(api.slice_conv(dev(Aq), dev(Bq)))
    ref = orc.slice_conv(pp, Aq, Bq, m, n, k)
    # |a||b| bound per entry and diagonal
    absC = orc.slice_conv(pp, np.abs(Aq), np.abs(Bq), m, n, k)
    assert np.all(np.abs(got - ref) <= 2.0 ** -50 * absC + 1e-300)
    frac_exact = np.mean(got == ref)
    print(f"slice_conv pp={pp} {shape}: {frac_exact:.4f} of entries bit-exact")


@pytest.mark.parametrize("name,P", [("dd64", 2), ("qd1024", 4)])
def test_fp64split_error_bits(api, orc, inputs, name, P):
    ex = pkg("errors")
    _, A, B = inputs.workload(name, 24, 24, 24)
    C = host(api.gemm(dev(A), dev(B), "fp64split"))
    ref = orc.gemm_fp64split(P, A, B, 24, 24, 24)
    bits = ex.error_bits(C, A, B, range(24), range(24))
    bits_ref = ex.error_bits(ref, A, B, range(24), range(24))
    assert bits[1] >= bits_ref[1] - 2.0, (bits, bits_ref)


@pytest.mark.parametrize("kind,P", [("split8", 2), ("split8", 4), ("split8", 8), ("mix", 2)])
def test_fp64split_gemm_other_split_kinds(api, orc, inputs, kind, P):
    """The split GEMM with the 8-slice split (split8pd, pp = 8P,
    floatybits.cu:622) and the mixed double-double split (mixsplit2, pp = 12,
    floatybits.cu:646), the choices of TCtest.cu:53-62: the same bound as
    the 4-slice form against the oracle's end-to-end split GEMM."""
    ex = pkg("errors")
    m, n, k = 20, 18, 33
    rng = np.random.default_rng(len(kind) * 10 + P)
    A = inputs.uniform_pd(rng, (m, k), P)
    B = inputs.uniform_pd(rng, (k, n), P)
    C = host(api.gemm(dev(A), dev(B), "fp64split", split_kind=kind))
    ref = orc.gemm_fp64split(P, A, B, m, n, k, kind=kind)
    bits = ex.error_bits(C, A, B, range(m), range(n))
    bits_ref = ex.error_bits(ref, A, B, range(m), range(n))
    assert bits[1] >= bits_ref[1] - 2.0, (bits, bits_ref)
    norms = np.abs(A[..., 0]) @ np.abs(B[..., 0])
    assert np.all(np.abs(C[..., 0] - ref[..., 0]) <= 2.0 ** -48 * norms)


def test_fp64split_reference_compatible_mode(api, orc, inputs):
    rng = np.random.default_rng(9)
    A = inputs.reference_pd(rng, (16, 16), 4)
    B = inputs.reference_pd(rng, (16, 16), 4)
    C = host(api.gemm(dev(A), dev(B), "fp64split", split_exact=False))
    ref = orc.gemm_fp64split(4, A, B, 16, 16, 16, exact=False)
    assert np.allclose(C[..., 0], ref[..., 0], rtol=2.0 ** -50, atol=0)


# --------------------------------------------------------- slice digits --

@pytest.mark.parametrize("P,s", [(2, 14), (4, 28), (8, 55), (16, 110)])
def test_digit_stages_bit_exact(api, orc, inputs, P, s):
    rng = np.random.default_rng(s)
    m, n, k = 20, 13, 37
    A = inputs.uniform_pd(rng, (m, k), P)
    B = inputs.uniform_pd(rng, (k, n), P)
    A, _ = inputs.scale_rows(rng, A, -8, 8)
    A[3] = 0.0
    dA, dB = dev(A), dev(B)
    E, F = api.scale_exponents(dA, dB)
    Eo, Fo = orc.scale_exps(P, A, B, m, n, k)
    assert np.array_equal(host(E), Eo) and np.array_equal(host(F), Fo)
    pa = host(api.slice_digits(dA, E, s).float()).astype(np.int32)
    pb = host(api.slice_digits(dB, F, s, trans=True).float()).astype(np.int32)
    assert np.array_equal(pa, orc.digits(P, s, A, m, k, Eo, 0))
    assert np.array_equal(pb, orc.digits(P, s, B, n, k, Fo, 1))
    assert np.abs(pa).max() <= 128 and np.abs(pb).max() <= 128


@pytest.mark.parametrize("engine", ["0", "1"])
@pytest.mark.parametrize("s,D,k", [(6, 9, 640), (3, 5, 64 * 1100)])
@pytest.mark.parametrize("m,n", [(128, 256), (256, 512)])
def test_diagonal_gemm_exact(api, orc, engine, s, D, k, m, n, monkeypatch):
    """Digit planes at the extremes the flush interval allows (runs of
    +-128 x -+128 products) through both engines; the second case cuts
    each diagonal into several int32 chunks.  m = 128 runs the single-CTA
    tcgen05 kernel, m = 256 the CTA-pair kernel."""
    monkeypatch.setenv("MDG_SLICE_ENGINE", engine)
    rng = np.random.default_rng(int(engine) + 7 + k + m)
    dA = rng.integers(-128, 129, size=(s, m, k)).astype(np.int32)
    dB = rng.integers(-128, 129, size=(s, n, k)).astype(np.int32)
    # a run of 1100 products of -2^14 fills one FP32 flush group of 1024
    # products to exactly -2^24 (the bound of the tcgen05 engines)
    run = min(k, 1100)
    dA[:, :, :run] = 128
    dB[:, :, :run] = -128
    ref = orc.diag_sums(s, D, dA, dB, m, n, k)
    Cd = api.slice_diagonals(dev(dA).to(torch.bfloat16), dev(dB).to(torch.bfloat16), D)
    assert np.array_equal(api.chunks_to_diagonals(Cd, s, D, k), ref)
    assert api.device_status() == 0


@pytest.mark.parametrize("engine", ["0", "1"])
@pytest.mark.parametrize("m,n", [(128, 256), (256, 512)])
def test_diagonal_gemm_full_chunk_at_the_int32_bound(api, engine, m, n, monkeypatch):
    """One digit pair (s = D = 1) with every product -2^14 over two whole
    int32 chunks and a partial third: each whole chunk sums to -2032 * 64 *
    2^14 = -2130706432, the largest magnitude the chunk length allows; the
    diagonal must come back as -2^14 k exactly.  Both engines; m = 128 runs
    the single-CTA tcgen05 kernel, m = 256 the CTA-pair kernel."""
    monkeypatch.setenv("MDG_SLICE_ENGINE", engine)
    k = 2 * 2032 * 64 + 640
    assert api.lib().mdg_slice_chunk_count(1, 1, k) == 3
    dA = torch.full((1, m, k), 128.0, dtype=torch.bfloat16, device="cuda")
    dB = torch.full((1, n, k), -128.0, dtype=torch.bfloat16, device="cuda")
    Cd = api.slice_diagonals(dA, dB, 1)
    assert int(Cd[0].min()) == int(Cd[0].max()) == -2032 * 64 * 2 ** 14
    diag = api.chunks_to_diagonals(Cd, 1, 1, k)
    assert np.all(diag == -(2 ** 14) * k)
    assert api.device_status() == 0


@pytest.mark.parametrize("P,D", [(2, 14), (4, 28), (8, 55), (16, 110)])
@pytest.mark.parametrize("k", [64, 64 * 4096])
def test_renorm_bit_exact(api, orc, P, D, k):
    rng = np.random.default_rng(P + k)
    m, n, s = 9, 21, D
    nch = pkg("_lib").lib().mdg_slice_chunk_count(s, D, k)
    Cd = rng.integers(-(2 ** 30), 2 ** 30, size=(nch, m, n)).astype(np.int32)
    Cd[:, 0, 0] = 0
    Cd[:, 1, 1] = 0
    Cd[-1, 1, 1] = -5
    E = rng.integers(-40, 40, size=m).astype(np.int32)
    F = rng.integers(-40, 40, size=n).astype(np.int32)
    dCd = dev(Cd)
    got = host(api.renorm_diagonals(dCd, dev(E), dev(F), P, s, D, k))
    diag = api.chunks_to_diagonals(dCd, s, D, k)
    assert np.array_equal(got, orc.renorm_diags(P, D, diag, E, F, m, n))


@pytest.mark.parametrize("engine", ["0", "1", "pair0"])
@pytest.mark.parametrize("P", [2, 4, 8])
@pytest.mark.parametrize("shape", [(1, 1, 1), (33, 31, 70), (130, 129, 65), (300, 260, 130)])
def test_slice_gemm_bit_exact_against_oracle(api, orc, inputs, engine, P, shape, monkeypatch):
    """engine 0: mma.sync; 1: tcgen05 CTA pairs (the default); pair0:
    tcgen05 single CTA."""
    if engine == "pair0":
        monkeypatch.setenv("MDG_TC_PAIR", "0")
        engine = "1"
    if P == 8 and shape[0] * shape[1] * shape[2] > 3e6:
        pytest.skip("oracle cost")
    monkeypatch.setenv("MDG_SLICE_ENGINE", engine)
    m, n, k = shape
    rng = np.random.default_rng(m + n + k + P)
    A = inputs.uniform_pd(rng, (m, k), P)
    B = inputs.uniform_pd(rng, (k, n), P)
    s = api.default_slices(P)
    got = host(api.gemm(dev(A), dev(B), "slice_bf16"))
    assert np.array_equal(got, orc.gemm_slices(P, s, s, A, B, m, n, k))


@pytest.mark.parametrize("P", [2, 4, 8, 16])
@pytest.mark.parametrize("shape", [(1, 1, 1), (33, 31, 70), (130, 129, 65), (3, 5, 70003)])
def test_fp64_digit_form_bit_exact_against_oracle(api, orc, inputs, P, shape):
    """The FP64 DMMA digit form (19-bit digits): bit for bit the oracle's
    restatement.  k = 70003 runs past one 65536-product FP64 segment, so
    the int64 flush of the DMMA sums is exercised."""
    m, n, k = shape
    if P == 16 and m * n * k > 3e5:
        pytest.skip("hexa-double oracle cost")
    rng = np.random.default_rng(m + n + k + P + 7)
    A = inputs.uniform_pd(rng, (m, k), P)
    B = inputs.uniform_pd(rng, (k, n), P)
    A, _ = inputs.scale_rows(rng, A, -20, 20)
    s = api.default_slices(P, "fp64_digits")
    got = host(api.gemm(dev(A), dev(B), "fp64_digits"))
    assert np.array_equal(got, orc.gemm_digits(P, s, s, A, B, m, n, k))


@pytest.mark.parametrize("name", ["dd64", "qd1024", "od2048_spread"])
def test_fp64_digit_form_error_bits_not_worse_than_plain(api, inputs, name):
    ex = pkg("errors")
    P, A, B = inputs.workload(name, 48, 48, 96)
    Cd = host(api.gemm(dev(A), dev(B), "fp64_digits"))
    Cp = host(api.gemm(dev(A), dev(B), "plain"))
    rows, cols = range(0, 48, 3), range(0, 48, 5)
    ed = ex.error_bits(Cd, A, B, rows, cols)
    ep = ex.error_bits(Cp, A, B, rows, cols)
    print(name, "fp64_digits", ed, "plain", ep)
    assert ed[1] >= ep[1] - 1.0


def test_slice_gemm_schedules_bit_identical(api, inputs, monkeypatch):
    """Tile order (raster), diagonal ranges per tile (parts) and the pacing
    of the CTA-pair kernel only reorder exact integer work: every schedule,
    and the mma.sync engine, must return the same bits.  36 pair tiles with
    5120-deep k (the three longest diagonals span two int32 chunks); pace 1
    makes the producers hold at almost every check."""
    P, m, n, k = 4, 1536, 1536, 5120
    rng = np.random.default_rng(1536)
    A = dev(inputs.normal_pd(rng, (m, k), P))
    B = dev(inputs.normal_pd(rng, (k, n), P))
    ref = host(api.gemm(A, B, "slice_bf16", engine="mma_sync"))
    for pace in ("0", "1", "64"):
        monkeypatch.setenv("MDG_TC_PACE", pace)
        for parts, raster in ((0, 0), (1, 1), (3, 2), (2, 5), (8, 100)):
            got = host(api.gemm(A, B, "slice_bf16", engine="tc_pair", parts=parts, raster=raster))
            assert np.array_equal(got, ref), (pace, parts, raster)
    monkeypatch.delenv("MDG_TC_PACE")
    for pace_opt in (-1, 1, 32, 128):  # the pacing window as an option
        got = host(api.gemm(A, B, "slice_bf16", engine="tc_pair", pace=pace_opt))
        assert np.array_equal(got, ref), pace_opt
    assert api.device_status() == 0


def test_bounded_wait_timeout_is_reported_and_context_survives(api, orc, inputs, monkeypatch):
    """Failure path of the CTA-pair kernel without a fault: with
    MDG_TC_SELFTEST_NO_LOADS=1 its producers issue no copies, so the MMA
    thread's wait for data runs out after its 2 s limit; the kernel raises
    its abort flag, every role leaves with nothing in flight and TMEM is
    freed.  The host reads MDG_ERROR_TIMEOUT (8), and the next launch in
    the same context computes the exact result."""
    P, m, n, k = 4, 256, 256, 128
    rng = np.random.default_rng(256)
    A = inputs.uniform_pd(rng, (m, k), P)
    B = inputs.uniform_pd(rng, (k, n), P)
    dA, dB = dev(A), dev(B)
    monkeypatch.setenv("MDG_TC_SELFTEST_NO_LOADS", "1")
    api.gemm(dA, dB, "slice_bf16", engine="tc_pair")
    assert api.device_status() == 8
    monkeypatch.delenv("MDG_TC_SELFTEST_NO_LOADS")
    s = api.default_slices(P)
    got = host(api.gemm(dA, dB, "slice_bf16", engine="tc_pair"))
    assert api.device_status() == 0
    assert np.array_equal(got, orc.gemm_slices(P, s, s, A, B, m, n, k))


def test_slice_gemm_hexa_double_bit_exact(api, orc, inputs):
    """P = 16 through the BF16 form (110 digits, 6105 digit pairs)."""
    rng = np.random.default_rng(16)
    m, n, k = 9, 7, 20
    A = inputs.uniform_pd(rng, (m, k), 16)
    B = inputs.uniform_pd(rng, (k, n), 16)
    got = host(api.gemm(dev(A), dev(B), "slice_bf16"))
    assert np.array_equal(got, orc.gemm_slices(16, 110, 110, A, B, m, n, k))


@pytest.mark.parametrize("name", ["dd64", "qd1024", "od2048_spread"])
def test_slice_error_bits_not_worse_than_plain(api, orc, inputs, name):
    ex = pkg("errors")
    P, A, B = inputs.workload(name, 48, 48, 96)
    Cs = host(api.gemm(dev(A), dev(B), "slice_bf16"))
    Cp = host(api.gemm(dev(A), dev(B), "plain"))
    rows, cols = range(0, 48, 3), range(0, 48, 5)
    es = ex.error_bits(Cs, A, B, rows, cols)
    ep = ex.error_bits(Cp, A, B, rows, cols)
    print(name, "slice", es, "plain", ep)
    assert es[1] >= ep[1] - 1.0


def test_octo_double_referee_agrees_with_exact_product(api, inputs):
    """The benchmark's large-block error bits use the octo-double plain GEMM
    of zero-padded quad-double inputs as referee; on a block small enough
    for the exact integer product both measurements agree within a bit."""
    ex = pkg("errors")
    P, A, B = inputs.workload("qd8192_normal", 24, 20, 256)
    C = host(api.gemm(dev(A), dev(B), "slice_bf16"))
    A8 = np.zeros(A.shape[:2] + (8,)); A8[..., :P] = A
    B8 = np.zeros(B.shape[:2] + (8,)); B8[..., :P] = B
    R = host(api.gemm(dev(A8), dev(B8), "plain"))
    norms = np.abs(A[..., 0]) @ np.abs(B[..., 0])
    exact = ex.error_bits(C, A, B, range(24), range(20))
    ref = ex.referee_error_bits(C, R, norms)
    assert abs(ref[0] - exact[0]) <= 1.0 and abs(ref[1] - exact[1]) <= 1.0, (ref, exact)
    assert ref[1] > 200


def test_two_host_threads_launch_at_once(api, inputs):
    """Two host threads issue GEMMs at the same time, each on its own
    stream, mixing the plain form at P = 16 (64 KiB of dynamic shared
    memory) with the CTA-pair and single-CTA slice engines: every result
    equals the same call made alone, so the launch path keeps no
    process-wide state that the threads could race on."""
    import threading
    cases = [[(16, 40, 30, 20, "plain", "auto"), (4, 300, 260, 130, "slice_bf16", "tc_pair"),
              (2, 128, 256, 64, "slice_bf16", "tc")],
             [(8, 64, 64, 64, "plain", "auto"), (2, 256, 512, 128, "slice_bf16", "tc_pair"),
              (16, 20, 20, 20, "slice_bf16", "auto")]]
    rng = np.random.default_rng(77)
    ops = [[(dev(inputs.uniform_pd(rng, (m, k), P)), dev(inputs.uniform_pd(rng, (k, n), P)))
            for P, m, n, k, _, _ in row] for row in cases]
    want = [[host(api.gemm(A, B, c[4], engine=c[5])) for c, (A, B) in zip(row, o)]
            for row, o in zip(cases, ops)]
    got = [[None] * len(row) for row in cases]
    errors = []

    def worker(t):
        try:
            s = torch.cuda.Stream()
            for rep in range(3):
                for i, (c, (A, B)) in enumerate(zip(cases[t], ops[t])):
                    C = api.gemm(A, B, c[4], engine=c[5], stream=s)
                    s.synchronize()
                    if rep == 2:
                        got[t][i] = host(C)
        except Exception as e:  # reported on the main thread
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(2)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for t in range(2):
        for i in range(len(cases[t])):
            assert np.array_equal(got[t][i], want[t][i]), (t, i)
    assert api.device_status() == 0


def test_host_entry_matches_device_entry(api, inputs):
    P, A, B = inputs.workload("qd1024", 50, 40, 30)
    for form in ("plain", "slice_bf16", "fp64split"):
        dC = host(api.gemm(dev(A), dev(B), form))
        hC = api.gemm_host(A, B, form)
        assert np.array_equal(dC, hC), form


def test_host_entry_with_library_pinned_buffers(api, inputs):
    """mdg_gemm_host on page-locked buffers from mdg_host_alloc (api.HostBuffer),
    the pipelined panel path included (m >= 2048): same bits as the device
    entry; the buffers are freed and allocated again without leaking."""
    import ctypes
    _lib = pkg("_lib")
    L = _lib.lib()
    P, A, B = inputs.workload("qd1024", 2100, 90, 60)
    m, k = A.shape[:2]
    n = B.shape[1]
    want = host(api.gemm(dev(A), dev(B), "slice_bf16"))
    for _ in range(2):
        hA, hB, hC = api.HostBuffer(A.shape), api.HostBuffer(B.shape), api.HostBuffer((m, n, P))
        hA.array[...] = A
        hB.array[...] = B
        hC.array[...] = np.nan
        _lib.check(L.mdg_gemm_host(2, P, m, n, k, hA.ptr, hB.ptr, hC.ptr, None), "host")
        assert np.array_equal(hC.array, want)
        for b in (hA, hB, hC):
            b.close()
    assert L.mdg_host_alloc(8, None) == 3


@pytest.mark.parametrize("m,n,k", [(2600, 300, 200), (4500, 130, 70), (2600, 4300, 96)])
def test_pipelined_host_entry_matches_device_entry(api, inputs, m, n, k):
    """mdg_gemm_host of the BF16 form on m >= 2048 rows copies A in row
    panels overlapped with the computation (2 panels of 1536 + 1064 rows,
    4 panels of 3 x 1280 + 660) and, for n >= 4096, B in two column strips
    (2304 + 1996 columns): the bits equal one device-side mdg_gemm.  Run
    twice so the second call reuses the library's buffers and streams."""
    P, A, B = inputs.workload("qd1024", m, n, k)
    dC = host(api.gemm(dev(A), dev(B), "slice_bf16"))
    for _ in range(2):
        assert np.array_equal(api.gemm_host(A, B, "slice_bf16"), dC)
    assert api.device_status() == 0


def test_strided_operands(api, orc, inputs):
    """Leading dimensions larger than the logical sizes (views of a wider
    buffer) through the C ABI."""
    import ctypes
    L = pkg("_lib").lib()
    P, A, B = inputs.workload("dd64", 24, 20, 28)
    lda, ldb, ldc = 40, 33, 29
    Aw = np.zeros((24, lda, P)); Aw[:, :28] = A
    Bw = np.zeros((28, ldb, P)); Bw[:, :20] = B
    Cw = torch.zeros((24, ldc, P), dtype=torch.float64, device="cuda")
    dA, dB = dev(Aw), dev(Bw)
    ref = orc.gemm_plain(P, A, B, 24, 20, 28)
    for form in (0, 1, 2):
        need = L.mdg_gemm_workspace_size(form, P, 24, 20, 28, None)
        ws = torch.empty(max(need, 1), dtype=torch.uint8, device="cuda")
        Cw.zero_()
        st = L.mdg_gemm(form, P, 24, 20, 28, ctypes.c_void_p(dA.data_ptr()), lda,
                        ctypes.c_void_p(dB.data_ptr()), ldb, ctypes.c_void_p(Cw.data_ptr()), ldc,
                        None, ctypes.c_void_p(ws.data_ptr()), need, None)
        assert st == 0
        torch.cuda.synchronize()
        C = host(Cw)
        assert np.all(C[:, 20:] == 0)
        if form == 0:
            assert np.array_equal(C[:, :20], ref)
        else:
            assert np.allclose(C[:, :20, 0], ref[..., 0], rtol=1e-15, atol=1e-15)


def test_zero_k_gives_zero(api):
    A = torch.zeros((5, 0, 4), dtype=torch.float64, device="cuda")
    B = torch.zeros((0, 6, 4), dtype=torch.float64, device="cuda")
    for form in ("plain", "fp64split", "slice_bf16"):
        C = api.gemm(A, B, form, out=torch.full((5, 6, 4), 3.0, dtype=torch.float64,
                                                 device="cuda"))
        assert torch.all(C == 0)


# -------------------------------------------------------------- batched --

def _batch_case(inputs, count, seed, shrink):
    probs, rng = inputs.batched_problems(count, seed=seed)
    probs = [(P, max(1, m // shrink), max(1, n // shrink), max(1, k // shrink))
             for P, m, n, k in probs]
    return probs, inputs.batched_operands(probs, rng)


def test_batched_slice_equals_single_problem_results(api, inputs):
    """One grouped launch per stage over mixed P and uneven sizes gives,
    for every problem, the bits of the single-problem BF16 GEMM."""
    probs, ops = _batch_case(inputs, 24, 11, 2)
    probs.append((4, 3, 5, 0))          # k = 0: C = 0
    ops.append((np.zeros((3, 0, 4)), np.zeros((0, 5, 4))))
    dev_ops = [(dev(A), dev(B)) for A, B in ops]
    Cs = api.gemm_batched(dev_ops, "slice_bf16")
    for (A, B), C in zip(dev_ops, Cs):
        if A.shape[1] == 0:
            assert torch.all(C == 0)
        else:
            assert torch.equal(C, api.gemm(A, B, "slice_bf16"))


def test_batched_slice_hexa_double_equals_single_problem_results(api, inputs):
    """Hexa-double problems (16-word digit and renorm kernels) in one batch
    with other limb counts, including a 1 x 3 x 5 problem."""
    rng = np.random.default_rng(5)
    probs = [(16, 40, 50, 70), (16, 130, 260, 64), (8, 33, 17, 100), (2, 64, 64, 64),
             (16, 1, 3, 5)]
    ops = [(dev(inputs.uniform_pd(rng, (m, k), P)), dev(inputs.uniform_pd(rng, (k, n), P)))
           for P, m, n, k in probs]
    Cs = api.gemm_batched(ops, "slice_bf16")
    for (A, B), C in zip(ops, Cs):
        assert torch.equal(C, api.gemm(A, B, "slice_bf16"))
    assert api.device_status() == 0


def test_batched_plan_graph_capture(api, orc, inputs):
    """The plan's run() captured in a CUDA graph and replayed; results are
    the oracle's bits (checked on three problems)."""
    probs, ops = _batch_case(inputs, 16, 12, 4)
    dev_ops = [(dev(A), dev(B)) for A, B in ops]
    plan = api.BatchPlan(dev_ops)
    plan.run()
    torch.cuda.synchronize()
    first = [C.clone() for C in plan.Cs]
    for C in plan.Cs:
        C.fill_(np.nan)
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            plan.run(stream=s)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    for a, b in zip(first, plan.Cs):
        assert torch.equal(a, b)
    for (P, m, n, k), (A, B), C in list(zip(probs, ops, plan.Cs))[:3]:
        sl = api.default_slices(P)
        assert np.array_equal(host(C), orc.gemm_slices(P, sl, sl, A, B, m, n, k))


def test_batched_tile_policies_bit_identical_and_tuned(api, orc, inputs):
    """The grouped GEMM under each tile policy (256-column tiles, 128-column
    tiles, the per-problem choice, and 256 x 256 tiles on CTA pairs) and
    split mode (heavy tiles cut into diagonal ranges, down to ranges that
    hold no diagonal for the hexa-double problem, or whole tiles) over
    problems whose n falls on both
    sides of a 256 boundary and whose k ends inside a 64-deep block (the
    last block issues fewer MMAs): every problem's C equals the
    single-problem GEMM under every choice; tuning keeps one of them and
    records it for plans of the same shapes."""
    rng = np.random.default_rng(31)
    probs = [(2, 96, 300, 40), (4, 130, 100, 96), (8, 64, 384, 160), (2, 256, 512, 16),
             (4, 33, 129, 200), (16, 20, 140, 24), (8, 128, 250, 64)]
    ops = [(dev(inputs.uniform_pd(rng, (m, k), P)), dev(inputs.uniform_pd(rng, (k, n), P)))
           for P, m, n, k in probs]
    want = [api.gemm(A, B, "slice_bf16") for A, B in ops]
    plan = api.BatchPlan(ops)
    assert plan.tiles == "256" and plan.split
    for split in (True, False):
        plan.set_split(split)
        for policy in ("auto", "128", "pair", "256"):
            plan.set_tiles(policy)
            for C in plan.Cs:
                C.fill_(np.nan)
            plan.run()
            torch.cuda.synchronize()
            for i, (C, W) in enumerate(zip(plan.Cs, want)):
                assert torch.equal(C, W), (policy, split, probs[i])
    api.tune_cache_clear()
    best = plan.tune()
    assert best in ("auto", "256", "128", "pair")
    assert api.tune_cache_size() == 1
    again = api.BatchPlan(ops)  # same shapes: starts with the tuned choice
    assert again.tiles == best and again.split == plan.split
    again.run()
    torch.cuda.synchronize()
    for C, W in zip(again.Cs, want):
        assert torch.equal(C, W)
    api.tune_cache_clear()
    # the first problem against the oracle as well
    P, m, n, k = probs[0]
    s = api.default_slices(P)
    A, B = host(ops[0][0]), host(ops[0][1])
    assert np.array_equal(host(again.Cs[0]), orc.gemm_slices(P, s, s, A, B, m, n, k))
    assert api.device_status() == 0
