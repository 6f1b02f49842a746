"""Seeded synthetic inputs for the multi-double GEMM workloads.

Matrices are numpy float64 arrays of shape (rows, cols, P): row-major, the
P limbs of one entry contiguous, most significant first -- the layout of the
reference (TCcuda.cu:130-131).

* ``uniform_pd``: hi limb U[-1, 1); limb i+1 is U[-1, 1) * ulp(limb i) / 2;
  then one renormalising sweep of quick-two-sums.
* ``normal_pd``: as uniform_pd with an N(0, 1) hi limb.
* ``reference_pd``: the reference's random_pd family (floatybits.cu:107-120):
  positive limbs, limb i = f_i * 2^(expmin - 52 i), f_i in [0.5, 1) with 52
  random fraction bits whose first bit is set.
* ``scale_rows`` / ``scale_cols``: multiply rows (columns) by 2^U{lo..hi}.
* ``workload(name)``: the five named workloads of the benchmark.
"""
import numpy as np


def _renorm_sweep(x):
    """One bottom-up then one top-down quick-two-sum sweep over the limbs."""
    P = x.shape[-1]
    for i in range(P - 2, -1, -1):
        a, b = x[..., i].copy(), x[..., i + 1].copy()
        s = a + b
        x[..., i] = s
        x[..., i + 1] = b - (s - a)
    for i in range(P - 1):
        a, b = x[..., i].copy(), x[..., i + 1].copy()
        s = a + b
        x[..., i] = s
        x[..., i + 1] = b - (s - a)
    return x


def _tail_limbs(rng, hi, P):
    x = np.empty(hi.shape + (P,), dtype=np.float64)
    x[..., 0] = hi
    for i in range(1, P):
        u = rng.uniform(-1.0, 1.0, size=hi.shape)
        x[..., i] = u * np.spacing(np.abs(x[..., i - 1])) * 0.5
    return _renorm_sweep(x)


def uniform_pd(rng, shape, P):
    return _tail_limbs(rng, rng.uniform(-1.0, 1.0, size=shape), P)


def normal_pd(rng, shape, P):
    return _tail_limbs(rng, rng.standard_normal(size=shape), P)


def reference_pd(rng, shape, P, expmin=0):
    x = np.empty(tuple(shape) + (P,), dtype=np.float64)
    for i in range(P):
        frac = rng.integers(0, 1 << 51, size=shape, dtype=np.int64) + (1 << 51)
        x[..., i] = np.ldexp(frac.astype(np.float64), expmin - 52 * i - 52)
    return x


def scale_rows(rng, x, lo=-32, hi=32):
    s = rng.integers(lo, hi + 1, size=x.shape[0])
    return np.ldexp(x, s[:, None, None]), s


def scale_cols(rng, x, lo=-32, hi=32):
    s = rng.integers(lo, hi + 1, size=x.shape[1])
    return np.ldexp(x, s[None, :, None]), s


# name -> (P, m, n, k, seed, kind)
WORKLOADS = {
    "dd64": (2, 64, 64, 64, 0, "uniform"),
    "qd1024": (4, 1024, 1024, 1024, 1, "uniform"),
    "od2048_spread": (8, 2048, 2048, 2048, 2, "spread"),
    "qd8192_normal": (4, 8192, 8192, 8192, 4, "normal"),
    # the headline distribution at 2048^3: the small case for profiling
    "qd2048_normal": (4, 2048, 2048, 2048, 4, "normal"),
    "qd4096_normal": (4, 4096, 4096, 4096, 4, "normal"),
}


def workload(name, m=None, n=None, k=None):
    """(P, A, B) for a named workload; m, n, k override the sizes (same
    seed and distribution) for smaller parity cases."""
    P, m0, n0, k0, seed, kind = WORKLOADS[name]
    m, n, k = m or m0, n or n0, k or k0
    rng = np.random.default_rng(seed)
    if kind == "normal":
        A = normal_pd(rng, (m, k), P)
        B = uniform_pd(rng, (k, n), P)
    else:
        A = uniform_pd(rng, (m, k), P)
        B = uniform_pd(rng, (k, n), P)
    if kind == "spread":
        A, _ = scale_rows(rng, A)
        B, _ = scale_cols(rng, B)
    return P, A, B


def batched_problems(count=256, seed=3):
    """The batched workload: count problems, m, n, k ~ U{32, 64, ..., 512},
    P ~ U{2, 4, 8}, hi limbs U[-1, 1)."""
    rng = np.random.default_rng(seed)
    probs = []
    for _ in range(count):
        m, n, k = (int(v) * 32 for v in rng.integers(1, 17, size=3))
        P = int(rng.choice([2, 4, 8]))
        probs.append((P, m, n, k))
    return probs, rng


def batched_operands(probs, rng):
    out = []
    for P, m, n, k in probs:
        out.append((uniform_pd(rng, (m, k), P), uniform_pd(rng, (k, n), P)))
    return out
