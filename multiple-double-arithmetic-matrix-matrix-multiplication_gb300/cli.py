"""Command line for one multi-double GEMM through the public API.

    python -m multiple-double-arithmetic-matrix-matrix-multiplication_gb300.cli gemm \\
        --form slice_bf16 --p 4 --m 1024 --n 1024 --k 1024 --seed 1 --dist uniform --sample 4

``gemm`` generates A (m x k) and B (k x n) on the device with the
counter-based generator (mdg_generate; A from --seed, B from --seed + 1),
runs the chosen form, and prints one JSON line: the configuration,
milliseconds per GEMM (CUDA events after warm-up; wall clock with --host,
which passes host buffers through mdg_gemm_host), effective md-GFLOP/s
(2 m n k / t) and, with --sample R, the error bits of the leading R x R
block of C against the exact product over the full k (entrywise and
normwise; exact while every limb lies above 2^-1100).

``tune`` times the bit-identical schedules of a BF16 slice-digit plan for
the shape on such operands, prints the chosen schedule, and with --cache
FILE loads and saves the tuning cache there.

The reference configures its runs with compile-time constants of its
drivers (TCtest.cu:7-19: p, n, loop_ct, ...); these flags stand in for them.
"""
import argparse
import json
import os
import sys
import time

from . import api, errors

FORMS = ("plain", "fp64split", "slice_bf16", "fp64_digits")


def _positive(text):
    v = int(text)
    if v < 1:
        raise argparse.ArgumentTypeError(f"{text} is not a positive count")
    return v


def build_parser():
    ap = argparse.ArgumentParser(prog="mdgemm", description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)

    def common(p):
        p.add_argument("--p", type=int, default=4, choices=(2, 4, 8, 16), help="limbs per entry")
        p.add_argument("--m", type=int, default=1024)
        p.add_argument("--n", type=int, default=1024)
        p.add_argument("--k", type=int, default=1024)
        p.add_argument("--seed", type=int, default=1)
        p.add_argument("--dist", default="uniform", choices=sorted(api.GEN_DISTS))
        p.add_argument("--e0", type=int, default=0,
                       help="exponent range start (reference family; row/column scales)")
        p.add_argument("--e1", type=int, default=0, help="exponent range end")
        p.add_argument("--scale-rows", action="store_true", help="rows of A times 2^U{e0..e1}")
        p.add_argument("--scale-cols", action="store_true", help="columns of B times 2^U{e0..e1}")
        p.add_argument("--slices", type=int, default=0, help="BF16 digits per entry (0 = default)")
        p.add_argument("--diagonals", type=int, default=0, help="digit diagonals kept (0 = slices)")
        p.add_argument("--engine", default="auto", choices=sorted(api.ENGINES))
        p.add_argument("--parts", type=int, default=0, help="diagonal ranges per tile (0 = auto)")
        p.add_argument("--raster", type=int, default=0, help="tile strip width (0 = auto)")
        p.add_argument("--pace", type=int, default=0,
                       help="pacing window in k-steps (0 = default, -1 = off)")

    g = sub.add_parser("gemm", help="time one GEMM and report error bits")
    common(g)
    g.add_argument("--form", default="slice_bf16", choices=FORMS)
    g.add_argument("--iters", type=_positive, default=3)
    g.add_argument("--warmup", type=int, default=1)
    g.add_argument("--sample", type=int, default=0,
                   help="R: error bits of the leading R x R block of C (0 = none)")
    g.add_argument("--host", action="store_true",
                   help="host buffers through mdg_gemm_host (copies inside the timing)")
    t = sub.add_parser("tune", help="tune a BF16 slice-digit plan for the shape")
    common(t)
    t.add_argument("--cache", default=None, help="JSON tuning cache to load and save")
    return ap


def gemm_options(args):
    """The mdg_options fields the flags set (forwarded to api.gemm / api.Plan)."""
    return {"slices": args.slices, "diagonals": args.diagonals, "engine": args.engine,
            "parts": args.parts, "raster": args.raster, "pace": args.pace}


def config(args):
    return {"p": args.p, "m": args.m, "n": args.n, "k": args.k, "seed": args.seed,
            "dist": args.dist, "e0": args.e0, "e1": args.e1, "scale_rows": args.scale_rows,
            "scale_cols": args.scale_cols}


def operands(args):
    A = api.generate(args.dist, args.p, args.m, args.k, args.seed, args.e0, args.e1,
                     scale_rows=args.scale_rows)
    B = api.generate(args.dist, args.p, args.k, args.n, args.seed + 1, args.e0, args.e1,
                     scale_cols=args.scale_cols)
    return A, B


def sample_error_bits(A, B, C, R):
    """(entrywise, normwise) error bits of the leading R x R block of C
    against the exact product of host arrays A (m x k x P), B (k x n x P)."""
    R = max(0, min(R, A.shape[0], B.shape[1]))
    if R == 0 or A.shape[1] == 0:
        return None
    ent, norm = errors.error_bits(C[:R, :R], A[:R], B[:, :R], range(R), range(R))
    return {"block": R, "entrywise": round(ent, 1), "normwise": round(norm, 1)}


def run_gemm(args):
    import torch
    A, B = operands(args)
    opts = gemm_options(args)
    flops = 2.0 * args.m * args.n * args.k
    if args.host:
        hA, hB = A.cpu().numpy(), B.cpu().numpy()
        for _ in range(args.warmup):
            api.gemm_host(hA, hB, args.form, **opts)
        t0 = time.perf_counter()
        for _ in range(args.iters):
            C = api.gemm_host(hA, hB, args.form, **opts)
        ms = (time.perf_counter() - t0) * 1e3 / args.iters
    else:
        C = torch.empty((args.m, args.n, args.p), dtype=torch.float64, device=A.device)
        need = api.workspace_size(args.form, args.p, args.m, args.n, args.k, **opts)
        ws = torch.empty(max(need, 1), dtype=torch.uint8, device=A.device)
        for _ in range(args.warmup):
            api.gemm(A, B, args.form, out=C, workspace=ws, **opts)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.iters):
            api.gemm(A, B, args.form, out=C, workspace=ws, **opts)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.iters
    line = {"command": "gemm", "form": args.form, "entry": "host" if args.host else "device",
            **config(args), "options": opts, "iters": args.iters, "ms": round(ms, 4),
            "md_gflops": round(flops / (ms * 1e-3) / 1e9, 2) if ms > 0 else None}
    if args.sample:
        R = args.sample
        block = C[:R, :R]
        block = block.cpu().numpy() if isinstance(block, torch.Tensor) else block
        line["error_bits"] = sample_error_bits(A[:R].cpu().numpy(), B[:, :R].cpu().numpy(),
                                               block, R)
    status = api.device_status()
    line["device_status"] = status
    print(json.dumps(line))
    return 0 if status == 0 else 1


def run_tune(args):
    import torch
    if args.cache and os.path.exists(args.cache):
        api.tune_cache_load(args.cache)
    A, B = operands(args)
    plan = api.Plan("slice_bf16", args.p, args.m, args.n, args.k, slices=args.slices,
                    diagonals=args.diagonals)
    try:
        C = torch.empty((args.m, args.n, args.p), dtype=torch.float64, device=A.device)
        plan.tune(A, B, C)
        schedule = plan.schedule()
    finally:
        plan.close()
    if args.cache:
        api.tune_cache_save(args.cache)
    print(json.dumps({"command": "tune", **config(args), "slices": args.slices,
                      "diagonals": args.diagonals, "schedule": schedule,
                      "cache": args.cache}))
    return 0


def main(argv=None):
    args = build_parser().parse_args(argv)
    return run_gemm(args) if args.cmd == "gemm" else run_tune(args)


if __name__ == "__main__":
    sys.exit(main())
