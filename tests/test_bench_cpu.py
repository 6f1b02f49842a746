"""The CPU legs of bench.py on tiny inputs (no GPU): the plain-GEMM sample
of the oracle port, the TCcudant convolution sample, and the peaks file."""
import importlib

import numpy as np


def test_cpu_baseline_legs_run_on_small_inputs(inputs, orc):
    bench = importlib.import_module("bench")
    P, A, B = inputs.workload("qd1024", 64, 64, 128)
    value, sample, dt = bench.cpu_sample(P, A, B, 0.05, 2)
    assert value > 0 and dt > 0 and "rows" in sample
    conv = bench.cpu_cudant_sample(P, A, B, n=32)
    assert conv["value"] > 0 and conv["cores"] == 1 and conv["kind"] == "port"
    peaks = bench.peaks()
    assert len(peaks) == 4 and all(isinstance(v, float) for v in peaks[:3])


def test_batched_tile_work_of_the_batched_workload(inputs):
    """Useful and padded BF16 work of the 256-problem batch (seed 3) at the
    default digit counts 14 / 28 / 55: rows padded to 128, columns to the
    tile policy's width, k to 16 (the last k-block issues only the MMAs
    that reach data); the CTA-pair policy pads to 256 x 256 tiles and k to
    64."""
    bench = importlib.import_module("bench")
    probs, _ = inputs.batched_problems(256, seed=3)
    useful, padded = bench.batched_tile_work(probs, {2: 14, 4: 28, 8: 55})
    assert abs(useful / 6.710e12 - 1) < 1e-3 and abs(padded / 1.101e13 - 1) < 1e-3
    _, padded128 = bench.batched_tile_work(probs, {2: 14, 4: 28, 8: 55}, "128")
    _, padded_auto = bench.batched_tile_work(probs, {2: 14, 4: 28, 8: 55}, "auto")
    assert padded_auto == padded128 < padded
    # CTA pairs: rows and columns to 256, k to 64
    _, padded_pair = bench.batched_tile_work(probs, {2: 14, 4: 28, 8: 55}, "pair")
    assert abs(padded_pair / 1.440e13 - 1) < 1e-3
    assert bench.batched_tile_work([(4, 128, 256, 64)], {4: 28}) == (2.0 * 128 * 256 * 64 * 406,) * 2
