"""The command line (cli.py) without a GPU: flags, the options it forwards
to the library, and the sampled error bits it reports."""
import subprocess
import sys

import numpy as np
import pytest

from conftest import PKG_NAME, ROOT, pkg


@pytest.fixture(scope="module")
def cli():
    return pkg("cli")


def test_flags_and_forwarded_options(cli):
    a = cli.build_parser().parse_args(["gemm", "--p", "8", "--m", "64", "--form", "plain",
                                       "--engine", "tc_pair", "--parts", "2", "--sample", "3"])
    assert (a.cmd, a.p, a.m, a.n, a.k, a.form, a.iters, a.sample) == \
        ("gemm", 8, 64, 1024, 1024, "plain", 3, 3)
    assert cli.gemm_options(a) == {"slices": 0, "diagonals": 0, "engine": "tc_pair",
                                   "parts": 2, "raster": 0, "pace": 0}
    t = cli.build_parser().parse_args(["tune", "--cache", "x.json", "--slices", "30"])
    assert (t.cmd, t.cache, t.slices, t.p) == ("tune", "x.json", 30, 4)
    for bad in (["gemm", "--iters", "0"], ["gemm", "--p", "3"], ["gemm", "--form", "int8"], []):
        with pytest.raises(SystemExit):
            cli.build_parser().parse_args(bad)


def test_help_runs_as_a_module():
    r = subprocess.run([sys.executable, "-m", PKG_NAME + ".cli", "gemm", "--help"], cwd=ROOT,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "--sample" in r.stdout


def test_sampled_error_bits(cli):
    rng = np.random.default_rng(0)
    P, m, n, k = 4, 5, 6, 7
    A = np.zeros((m, k, P))
    B = np.zeros((k, n, P))
    A[..., 0] = rng.integers(-9, 10, size=(m, k))
    B[..., 0] = rng.integers(-9, 10, size=(k, n))
    C = np.zeros((m, n, P))
    C[..., 0] = A[..., 0] @ B[..., 0]  # small integers: exact
    got = cli.sample_error_bits(A, B, C, 4)
    assert got == {"block": 4, "entrywise": 1100.0, "normwise": 1100.0}
    C[1, 2, 0] += 2.0 ** -40 * max(1.0, abs(C[1, 2, 0]))
    got = cli.sample_error_bits(A, B, C, 4)
    assert 30 < got["normwise"] < 45 and got["entrywise"] <= 41
    assert cli.sample_error_bits(A, B, C, 0) is None
    assert cli.sample_error_bits(A, B, C, 100)["block"] == min(m, n)
