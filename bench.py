"""Benchmark of the multi-double GEMM path on one GB300 (or N replicas).

Workload (default): quad-double C = A B, m = n = k = 8192, seed 4, hi limbs
N(0, 1), lower limbs U[-1, 1) ulp/2 (the headline configuration).  A step is
one whole GEMM in the BF16 slice-digit form: scale exponents, digit planes,
diagonal GEMM on the tensor cores, renormalisation.

  value    effective multi-double GFLOP/s = 2 m n k / t, inputs resident in
           HBM, timed with CUDA events on the launching stream
  e2e      the same metric through mdg_gemm_host-style use of the C ABI
           with pinned host buffers: A and B copied in and C copied out
           inside the timed region of every step
  roofline the diagonal GEMM kernel: BF16 tensor FLOPs it must execute
           (2 Mp Np Kp per digit pair) over its own event-timed duration
  cpu_baseline  the oracle's plain quad-double GEMM (the C restatement of
           the reference's matmulqdf) on the host cores, a bounded sample
  forms    the FP64-split, FP64-digit and plain forms beside the BF16 form
           on the quad-double 1024^3 (seed 1) and octo-double 2048^3
           row/column-spread (seed 2) workloads, with error bits of every
           form against the exact product on sampled entries; a
           hexa-double line; the FP64 and INT8 tensor rates

--impl reference times the reference's CPU implementation of the path
(oracle/_ref when it was built from the reference sources on this machine,
else the oracle's restatement of it) on the same metric.
"""
import argparse
import ctypes
import importlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "multiple-double-arithmetic-matrix-matrix-multiplication_gb300"
METRIC = "qd/od GEMM effective GFLOP/s: slice-TC vs FP64-split vs plain, equal error bits"
UNIT = "GFLOP/s"

WORKLOADS = {
    "qd8192_normal": "qd8192_normal",
    "qd2048_normal": "qd2048_normal",
    "qd4096_normal": "qd4096_normal",
    "qd1024": "qd1024",
    "od2048_spread": "od2048_spread",
    "dd64": "dd64",
}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the paced CTA-pair diagonal GEMM, from one-pass ncu captures of the bench's
# own command on this machine's GB300 (quad-double, seed 4 inputs):
#   8192^3: 462.35 GB read + 17.27 GB written;  4096^3: 71.66 + 2.69 GB.
DIAG_TRAFFIC_BYTES = {"qd8192_normal": 473.09e9, "qd4096_normal": 73.51e9}


DEFAULT_SLICES = {2: 14, 4: 28, 8: 55, 16: 110}


def digit_pairs(s, D):
    """Digit pairs (i, j), i + j = d < D, of s digits per operand."""
    return sum(min(d, s - 1) - max(0, d - (s - 1)) + 1 for d in range(D))


def bench_config(workload, world):
    """The `config` object of both arms' lines (the same keys and values, so
    the two lines describe one workload)."""
    inputs = importlib.import_module(PKG + ".inputs")
    P, m, n, k, seed, kind = inputs.WORKLOADS[workload]
    s = DEFAULT_SLICES[P]
    planes_gb = s * (m + n) * k * 2 / 1e9
    return {"workload": workload, "p": P, "m": m, "n": n, "k": k, "seed": seed,
            "distribution": kind, "slices": s, "diagonals": s, "digit_pairs": digit_pairs(s, s),
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "l2": f"inputs (A and B {(m + n) * k * P * 8 / 2 ** 30:.2f} GiB, digit planes "
                  f"{planes_gb:.1f} GB) larger than L2 (129 MB), no flush"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return d["bf16_tflops"], d["bf16_tflops_sustained"], d["hbm_gbs"], "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, 1700.0, 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", os.environ.get("LOCAL_RANK", "0"),
                 f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return world, rank


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sample(P, A, B, target_s, threads):
    """Time the oracle's plain GEMM (the reference's matmulqdf arithmetic) on
    R rows x nc columns of C at the full k, sized to take about target_s."""
    import oracle
    k = A.shape[1]
    r, nc = 1, 8
    Bs = np.ascontiguousarray(B[:, :nc])
    t0 = time.perf_counter()
    oracle.gemm_plain(P, A[:r], Bs, r, nc, k, threads=1)
    per_madd = (time.perf_counter() - t0) / (r * nc * k)
    madds = max(1.0, target_s / per_madd) * threads
    nc = int(min(B.shape[1], max(threads, 64)))
    r = int(max(threads, min(A.shape[0], madds / (nc * k))))
    r = (r // threads) * threads or threads
    Bs = np.ascontiguousarray(B[:, :nc])
    t0 = time.perf_counter()
    oracle.gemm_plain(P, A[:r], Bs, r, nc, k, threads=threads)
    dt = time.perf_counter() - t0
    return 2.0 * r * nc * k / dt / 1e9, f"{r} rows x {nc} columns of C at k={k}", dt


def cpu_cudant_sample(P, A, B, n=256):
    """The reference's CPU convolution path (TCcudant.cpp: split4pd, splitp,
    manualconvmult) through the oracle's restatement of its loops, on the
    leading n x n x n block, one thread like the reference: effective
    md-GFLOP/s of the split-form product it forms (its 4P slice planes are
    not squeezed back to P limbs)."""
    import oracle
    pp = 4 * P
    As = oracle.split("split4", P, A[:n, :n].reshape(-1, P)).reshape(n, n, pp)
    Bs = oracle.split("split4", P, B[:n, :n].reshape(-1, P)).reshape(n, n, pp)
    Ap = np.ascontiguousarray(np.moveaxis(As, 2, 0))
    Bp = np.ascontiguousarray(np.moveaxis(Bs, 2, 0))
    t0 = time.perf_counter()
    oracle.plane_conv(n, pp, Ap, Bp)
    dt = time.perf_counter() - t0
    return {"value": 2.0 * n ** 3 / dt / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n}^3 block, {pp} slice planes, manualconvmult order", "seconds": dt}


def reference_cpu_sample(P, A, B, threads, nsub):
    """The reference's own host GEMM (matmul{dd,qd,od}f, TCcuda.cu:320-359,
    built from its sources into oracle/_ref) on the leading nsub x nsub x nsub
    block of the workload, one independent copy per host thread (the
    reference is single-threaded): (md-GFLOP/s, sample text, seconds)."""
    import concurrent.futures as cf

    import oracle
    Asub = np.ascontiguousarray(A[:nsub, :nsub])
    Bsub = np.ascontiguousarray(B[:nsub, :nsub])
    name = {2: "matmulddf", 4: "matmulqdf", 8: "matmulodf", 16: "matmulhdf"}[P]
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda _: oracle.ref_matmul(P, Asub, Bsub, nsub), range(threads)))
    dt = time.perf_counter() - t0
    return (2.0 * nsub ** 3 * threads / dt / 1e9,
            f"{threads} threads x {name} on the leading {nsub}^3 block (reference sources)", dt)


def run_reference(args):
    """The reference's CPU path, timed on the host cores."""
    world, rank = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    inputs = importlib.import_module(PKG + ".inputs")
    oracle.build()
    threads = os.cpu_count() or 1
    P, A, B = inputs.workload(args.workload)
    kind = "reference" if oracle.ref_available() else "port"
    vals, times = [], []
    for i in range(args.warmup + args.steps):
        if kind == "reference":
            v, sample, dt = reference_cpu_sample(P, A, B, threads, 128 if P <= 4 else 64)
        else:
            v, sample, dt = cpu_sample(P, A, B, 3.0, threads)
        if i >= args.warmup:
            vals.append(v)
            times.append(dt)
    value = float(np.median(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.median(times)) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(args.workload, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": sample, "extrapolated": True,
                         "extrapolation": "rate of the sample; the whole workload at this rate "
                                          f"would take {2.0 * np.prod(inputs.WORKLOADS[args.workload][1:4]) / value / 1e9 / 3600:.1f} h"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def event_time(fn, stream, iters=1):
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(iters):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3 / iters


def pipelined_e2e(api, hA, hB, hC, P, m, n, k, ws_bytes, steps):
    """Seconds per step of a host-to-host loop with double-buffered device
    operands: step i computes on one buffer set while the copy streams load
    step i+1's A and B and return step i-1's C."""
    import torch
    comp = torch.cuda.current_stream()
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    dA = [torch.empty_like(hA, device="cuda") for _ in range(2)]
    dB = [torch.empty_like(hB, device="cuda") for _ in range(2)]
    dC = [torch.empty((m, n, P), dtype=torch.float64, device="cuda") for _ in range(2)]
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_done = [torch.cuda.Event() for _ in range(2)]
    ev_out = [torch.cuda.Event() for _ in range(2)]
    for e in ev_done + ev_out:
        e.record(comp)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with torch.cuda.stream(s_in):
        dA[0].copy_(hA, non_blocking=True)
        dB[0].copy_(hB, non_blocking=True)
        ev_in[0].record(s_in)
    for i in range(steps):
        b, nb = i % 2, (i + 1) % 2
        if i + 1 < steps:
            s_in.wait_event(ev_done[nb])
            with torch.cuda.stream(s_in):
                dA[nb].copy_(hA, non_blocking=True)
                dB[nb].copy_(hB, non_blocking=True)
                ev_in[nb].record(s_in)
        comp.wait_event(ev_in[b])
        comp.wait_event(ev_out[b])
        api.gemm(dA[b], dB[b], "slice_bf16", out=dC[b], workspace=ws)
        ev_done[b].record(comp)
        s_out.wait_event(ev_done[b])
        with torch.cuda.stream(s_out):
            hC.copy_(dC[b], non_blocking=True)
            ev_out[b].record(s_out)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    del dA, dB, dC, ws
    torch.cuda.empty_cache()
    return dt


def batched_tile_work(probs, slices, policy="256"):
    """BF16 FLOP of the batched diagonal GEMM at the given digit counts per
    P: useful (2 m n k per digit pair of the s diagonals kept) and as the
    grouped kernel pads it: single-CTA tiles pad rows to 128, columns to the
    tile width of the policy and k to 16 (the last 64-deep block issues only
    the MMAs that reach data); CTA-pair tiles pad rows and columns to 256
    and k to 64."""
    def pairs(s):
        return sum(min(d, s - 1) - max(0, d - (s - 1)) + 1 for d in range(s))
    up = lambda x, a: -(-x // a) * a
    def width(n):
        if policy == "256":
            return up(n, 256)
        if policy == "128":
            return up(n, 128)
        return min(up(n, 128), up(n, 256))
    useful = padded = 0.0
    for P, m, n, k in probs:
        q = pairs(slices[P])
        useful += 2.0 * m * n * k * q
        if policy == "pair":
            padded += 2.0 * up(m, 256) * up(n, 256) * up(k, 64) * q
        else:
            padded += 2.0 * up(m, 128) * width(n) * up(k, 16) * q
    return useful, padded


def bench_batched(api, inputs, stream):
    """The batched workload (256 problems, m, n, k in {32..512}, P in {2, 4, 8},
    seed 3): the BF16 slice-digit plan replayed as one CUDA graph, against a
    loop of per-problem plain launches and the one-launch plain batch."""
    import torch
    probs, rng = inputs.batched_problems(256, seed=3)
    ops = inputs.batched_operands(probs, rng)
    dev_ops = [(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()) for A, B in ops]
    flops = sum(2.0 * m * n * k for _, m, n, k in probs)

    def captured(pairs, tune=False):
        plan = api.BatchPlan(pairs)
        if tune:
            plan.tune()  # times every tile policy and split mode, keeps the fastest
        plan.run()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                plan.run(stream=s)
        for _ in range(3):
            g.replay()
        torch.cuda.synchronize()
        return plan, g

    plan, g = captured(dev_ops, tune=True)
    t_graph = event_time(g.replay, torch.cuda.current_stream(), iters=5)
    policy = plan.tiles
    useful, padded = batched_tile_work(probs, {P: api.default_slices(P)
                                               for P in {pr[0] for pr in probs}}, policy)
    # the metric per P (each P's problems as their own graph-replayed plan)
    per_p = {}
    for P in (2, 4, 8):
        sel = [i for i, pr in enumerate(probs) if pr[0] == P]
        if not sel:
            continue
        _, gp = captured([dev_ops[i] for i in sel])
        tp = event_time(gp.replay, torch.cuda.current_stream(), iters=3)
        fp = sum(2.0 * probs[i][1] * probs[i][2] * probs[i][3] for i in sel)
        per_p[f"p{P}"] = {"problems": len(sel), "md_gflop": fp / 1e9,
                          "slice_graph_gflops": fp / tp / 1e9, "ms": tp * 1e3}
        del gp
    # every C of the graph equals the single-problem slice GEMM
    same = all(torch.equal(C, api.gemm(A, B, "slice_bf16")) for (A, B), C in
               list(zip(dev_ops, plan.Cs))[:16])
    outs = [torch.empty((A.shape[0], B.shape[1], A.shape[2]), dtype=torch.float64,
                        device="cuda") for A, B in dev_ops]

    def plain_loop():
        for (A, B), C in zip(dev_ops, outs):
            api.gemm(A, B, "plain", out=C)

    t_loop = event_time(plain_loop, stream, iters=1)
    api.gemm_batched(dev_ops, "plain")
    t_pb = event_time(lambda: api.gemm_batched(dev_ops, "plain"), stream, iters=1)
    return {"workload": "256 problems, m,n,k ~ U{32..512 step 32}, P ~ U{2,4,8}, seed 3",
            "md_gflop": flops / 1e9,
            "slice_graph_gflops": flops / t_graph / 1e9, "slice_graph_ms": t_graph * 1e3,
            "per_p": per_p,
            # kernels per plan run: exponents of all rows and columns, digits
            # of all operands, the grouped diagonal GEMM, and one
            # renormalisation per limb count present
            "slice_launches_per_batch": 3 + len({pr[0] for pr in probs}),
            "tile_policy": policy,
            "split": plan.split,
            "plain_loop_gflops": flops / t_loop / 1e9, "plain_loop_ms": t_loop * 1e3,
            "plain_batched_gflops": flops / t_pb / 1e9, "plain_batched_ms": t_pb * 1e3,
            "slice_equals_single_problem": bool(same),
            "diag_bf16_tflop": {"useful": useful / 1e12, "padded": padded / 1e12,
                                "useful_frac": useful / padded,
                                "tiles": ("256 x 256 (CTA pairs, rows padded to 256)"
                                          if policy == "pair" else
                                          f"128 x {policy} columns (single CTA)")
                                         + " under the tuned policy, k padded to 16"}}


# FP64 operations per multi-double multiply-add of the plain form, the
# reference's own counts (TCtest.cu:136-148: dd 23 mul + 20 add, qd 336 + 89,
# od 1742 + 269; hd has only a placeholder there)
PLAIN_OPS = {2: 43, 4: 425, 8: 2011}


def split_dmma_madds(pp):
    """(algorithmic, executed) FP64 multiply-adds per (row, column, k) of the
    truncated slice convolution with pp slices: sum_{i<pp} (i + 1) products
    C_i = sum_{j<=i} a_j b_{i-j}, and the 4-wide DMMA chunks the kernel runs,
    sum_i 4 ceil((i + 1) / 4), zero lanes of partial chunks included."""
    return pp * (pp + 1) // 2, sum(4 * -(-(i + 1) // 4) for i in range(pp))


def bench_form_line(api, ex, stream, P, A, B, form, dA, dB, sample, iters=1, rows=None):
    """One form on one workload: md-GFLOP/s (CUDA events, after one untimed
    call) and error bits against the exact product on sampled entries.
    rows: time and check only this many leading rows of C (the rate per
    row of the plain form does not depend on the row count)."""
    import torch
    m, k = A.shape[:2]
    n = B.shape[1]
    if rows is not None and rows < m:
        dA, A, m = dA[:rows].contiguous(), A[:rows], rows
    out = torch.empty((m, n, P), dtype=torch.float64, device="cuda")
    w = torch.empty(max(1, api.workspace_size(form, P, m, n, k)), dtype=torch.uint8,
                    device="cuda")
    # the first call is timed too: a form that takes seconds is measured on it
    # (loading its kernels is a negligible part), a fast one on `iters` more
    t = event_time(lambda: api.gemm(dA, dB, form, out=out, workspace=w), stream, iters=1)
    if t < 1.0:
        t = event_time(lambda: api.gemm(dA, dB, form, out=out, workspace=w), stream,
                       iters=iters)
    r = [i for i in sample[0] if i < m]
    eb = ex.error_bits(out.cpu().numpy(), A, B, r, sample[1])
    del out, w
    torch.cuda.empty_cache()
    return {"shape": f"{m}x{n}x{k}", "gflops": 2.0 * m * n * k / t / 1e9, "ms": t * 1e3,
            "error_bits_entrywise": round(eb[0], 1), "error_bits_normwise": round(eb[1], 1),
            "error_sample": f"{len(r)}x{len(sample[1])} entries, exact integer product"}


def bench_forms(api, inputs, ex, stream):
    """The three forms side by side on the quad-double 1024^3 (seed 1) and
    octo-double 2048^3 row/column-spread (seed 2) workloads, the hexa-double
    slice form against plain hd, and the FP64 and INT8 tensor rates."""
    import torch
    forms = {}
    # FP64 ceiling of the two FP64 forms, measured here (the peaks file
    # holds BF16 and HBM only): cuBLAS DGEMM through torch.matmul
    a64 = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    torch.matmul(a64, a64)
    t64 = event_time(lambda: torch.matmul(a64, a64), stream, iters=3)
    fp64 = 2.0 * 4096 ** 3 / t64 / 1e12
    del a64
    forms["fp64_peak"] = {"tflops": fp64, "how": "torch.matmul float64 4096^3 (cuBLAS "
                          "DGEMM), 3 launches, CUDA events"}
    for wl in ("qd1024", "od2048_spread"):
        P, A, B = inputs.workload(wl)
        m, k = A.shape[:2]
        n = B.shape[1]
        dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
        step = max(1, m // 6)
        sample = (range(0, m, step), range(0, n, step))
        block = {}
        block["slice_bf16"] = bench_form_line(api, ex, stream, P, A, B, "slice_bf16", dA, dB,
                                              sample, iters=3)
        # the same GEMM through a tuned plan (mdg_plan_tune: engines, parts, tile
        # strips and pacing windows that give the same bits)
        plan = api.Plan("slice_bf16", P, m, n, k)
        Ct = torch.empty((m, n, P), dtype=torch.float64, device="cuda")
        plan.tune(dA, dB, Ct)
        tt = event_time(lambda: plan.run(dA, dB, Ct), stream, iters=3)
        block["slice_bf16_tuned"] = {"gflops": 2.0 * m * n * k / tt / 1e9, "ms": tt * 1e3,
                                     "schedule": plan.schedule()}
        plan.close()
        del Ct
        block["fp64split"] = bench_form_line(api, ex, stream, P, A, B, "fp64split", dA, dB,
                                             sample)
        block["fp64_digits"] = bench_form_line(api, ex, stream, P, A, B, "fp64_digits", dA, dB,
                                               sample)
        # the plain octo-double GEMM takes ~20 s at 2048^3: rows 0..511 of C
        block["plain"] = bench_form_line(api, ex, stream, P, A, B, "plain", dA, dB, sample,
                                         rows=512 if P >= 8 else None)
        if P >= 8:
            block["plain"]["rows_timed"] = "rows 0..511 of C (full n, k)"
        mnk = float(m) * n * k
        alg, exe = split_dmma_madds(4 * P)
        sp = block["fp64split"]
        t = sp["ms"] / 1e3
        sp["roofline"] = {"bound": "fp64 tensor (DMMA)",
                          "achieved_tflops": 2.0 * alg * mnk / t / 1e12,
                          "executed_tflops": 2.0 * exe * mnk / t / 1e12,
                          "peak_tflops": fp64, "frac": 2.0 * alg * mnk / t / 1e12 / fp64,
                          "madds_per_mnk": {"algorithmic": alg, "executed": exe},
                          "peak_kind": "cuBLAS DGEMM rate measured in this run"}
        pl = block["plain"]
        pl["roofline"] = {"bound": "fp64 CUDA cores (DGEMM-rate proxy)",
                          "achieved_tops": PLAIN_OPS[P] * pl["gflops"] / 2.0 / 1e3,
                          "proxy_peak_tflops": fp64,
                          "frac_of_proxy": PLAIN_OPS[P] * pl["gflops"] / 2.0 / 1e3 / fp64,
                          "note": f"{PLAIN_OPS[P]} FP64 operations per multiply-add (the "
                                  "reference's count, TCtest.cu:136-148), issued as unfused "
                                  "mul/add; the DGEMM flop rate stands in for the FP64 "
                                  "CUDA-core peak, which the peaks file does not hold"}
        fd = block["fp64_digits"]
        s19 = api.default_slices(P, "fp64_digits")
        fd_tflops = 2.0 * digit_pairs(s19, s19) * mnk / (fd["ms"] / 1e3) / 1e12
        fd["digits"] = s19
        fd["roofline"] = {"bound": "fp64 tensor (DMMA)", "achieved_tflops": fd_tflops,
                          "peak_tflops": fp64, "frac": fd_tflops / fp64,
                          "digit_pairs": digit_pairs(s19, s19),
                          "peak_kind": "cuBLAS DGEMM rate measured in this run"}
        sl = block["slice_bf16"]
        block["slice_over_fp64_digits"] = {
            "ratio": sl["gflops"] / fd["gflops"],
            "equal_accuracy": bool(fd["error_bits_normwise"] >= pl["error_bits_normwise"] - 1 and
                                   sl["error_bits_normwise"] >= pl["error_bits_normwise"] - 1),
            "error_bits_normwise": {"slice_bf16": sl["error_bits_normwise"],
                                    "fp64_digits": fd["error_bits_normwise"],
                                    "plain": pl["error_bits_normwise"]},
            "note": "the same exact digit scheme on the FP64 tensor cores (19-bit digits) "
                    "and on the BF16 ones (8-bit digits): both at or above the plain "
                    "form's error bits"}
        block["slice_over_fp64split"] = {
            "ratio": sl["gflops"] / sp["gflops"],
            "equal_accuracy": False,
            "error_bits_normwise": {"slice_bf16": sl["error_bits_normwise"],
                                    "fp64split": sp["error_bits_normwise"],
                                    "plain": pl["error_bits_normwise"]},
            "note": "not an equal-accuracy ratio: the FP64 split form (the reference's "
                    "method, 4 slices of 13 bits per limb, truncated convolution) reaches "
                    "fewer bits than both other forms on these inputs"}
        block["slice_over_plain"] = sl["gflops"] / pl["gflops"]
        forms[wl] = block
        del dA, dB
        torch.cuda.empty_cache()
    # hexa-double: the BF16 form (110 digits, 6105 digit pairs) against the
    # plain hd GEMM on a 1024 x 1024 x 512 problem (uniform inputs, seed 16)
    rng = np.random.default_rng(16)
    m, n, k = 1024, 1024, 512
    A = inputs.uniform_pd(rng, (m, k), 16)
    B = inputs.uniform_pd(rng, (k, n), 16)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    sample = (range(0, m, 256), range(0, n, 256))
    hd = {"workload": f"hd {m}x{n}x{k}, hi limbs U[-1,1), seed 16"}
    hd["slice_bf16"] = bench_form_line(api, ex, stream, 16, A, B, "slice_bf16", dA, dB, sample,
                                       iters=2)
    hd["plain"] = bench_form_line(api, ex, stream, 16, A, B, "plain", dA, dB, sample, rows=256)
    hd["plain"]["rows_timed"] = "rows 0..255 of C (full n, k)"
    hd["slice_over_plain"] = hd["slice_bf16"]["gflops"] / hd["plain"]["gflops"]
    forms["hd1024x1024x512"] = hd
    del dA, dB
    torch.cuda.empty_cache()
    # the INT8 tensor rate, against which an int8-digit slice form would
    # run (cuBLAS through torch._int_mm), beside BF16 at the same size
    a8 = torch.randint(-128, 127, (8192, 8192), dtype=torch.int8, device="cuda")
    b8 = a8.t().contiguous().t()
    a16 = torch.randn(8192, 8192, dtype=torch.bfloat16, device="cuda")
    torch._int_mm(a8, b8)
    a16 @ a16
    t8 = event_time(lambda: torch._int_mm(a8, b8), stream, iters=3)
    t16 = event_time(lambda: a16 @ a16, stream, iters=3)
    forms["int8_vs_bf16"] = {"int8_tops": 2.0 * 8192 ** 3 / t8 / 1e12,
                             "bf16_tflops": 2.0 * 8192 ** 3 / t16 / 1e12,
                             "how": "torch._int_mm int8 and torch.matmul bf16, 8192^3"}
    del a8, b8, a16
    torch.cuda.empty_cache()
    return forms


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="qd8192_normal", choices=sorted(WORKLOADS))
    ap.add_argument("--no-forms", action="store_true", help="skip the FP64-split/plain lines")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    world, rank = dist_setup(args.gpus)
    api = importlib.import_module(PKG + ".api")
    _lib = importlib.import_module(PKG + "._lib")
    inputs = importlib.import_module(PKG + ".inputs")
    L = _lib.lib()
    stream = torch.cuda.current_stream()

    P, A, B = inputs.workload(args.workload)
    m, k = A.shape[:2]
    n = B.shape[1]
    flops = 2.0 * m * n * k
    s = api.default_slices(P)
    D = s
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(B).cuda()
    dC = torch.empty((m, n, P), dtype=torch.float64, device="cuda")
    need = api.workspace_size("slice_bf16", P, m, n, k)
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")

    def step():
        api.gemm(dA, dB, "slice_bf16", out=dC, workspace=ws)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # ---- device-resident timing (inputs larger than L2)
    clocks = Clocks()
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    t_step = max_over_ranks(e0.elapsed_time(e1) / 1e3 / args.steps, world)
    clk = clocks.stop()
    value = flops * world / t_step / 1e9

    # ---- roofline of the diagonal GEMM: run the stages once, time it alone
    pl_Mp, pl_Np, pl_Kp = [-(-x // a) * a for x, a in ((m, 128), (n, 128), (k, 64))]
    E, F = api.scale_exponents(dA, dB)
    pa = api.slice_digits(dA, E, s)
    pb = api.slice_digits(dB, F, s, trans=True)
    pa_p = torch.zeros((s, pl_Mp, pl_Kp), dtype=torch.bfloat16, device="cuda")
    pb_p = torch.zeros((s, pl_Np, pl_Kp), dtype=torch.bfloat16, device="cuda")
    pa_p[:, :m, :k] = pa
    pb_p[:, :n, :k] = pb
    del pa, pb
    api.slice_diagonals(pa_p, pb_p, D)
    t_diag = event_time(lambda: api.slice_diagonals(pa_p, pb_p, D), stream, iters=2)
    pairs = sum(min(d, s - 1) - max(0, d - (s - 1)) + 1 for d in range(D))
    tflop = 2.0 * pl_Mp * pl_Np * pl_Kp * pairs / 1e12
    bf16_burst, bf16_sust, hbm, peak_kind = peaks()
    achieved = tflop / t_diag
    del pa_p, pb_p
    torch.cuda.empty_cache()

    # ---- e2e through the C ABI's host-buffer call, pinned host buffers:
    # every step copies A and B in, computes and copies C out
    # page-locked host buffers from the library (mdg_host_alloc): what a
    # caller of the host entry is told to use for full-rate copies
    bufA, bufB, bufC = api.HostBuffer(A.shape), api.HostBuffer(B.shape), api.HostBuffer((m, n, P))
    bufA.array[...] = A
    bufB.array[...] = B
    hA, hB, hC = (torch.from_numpy(b.array) for b in (bufA, bufB, bufC))
    del ws
    torch.cuda.empty_cache()

    def e2e_step():
        _lib.check(L.mdg_gemm_host(2, P, m, n, k, ctypes.c_void_p(hA.data_ptr()),
                                   ctypes.c_void_p(hB.data_ptr()), ctypes.c_void_p(hC.data_ptr()),
                                   None), "mdg_gemm_host")

    e2e_step()
    e2e_steps = max(1, min(args.steps, 5))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    t_e2e = max_over_ranks((time.perf_counter() - t0) / e2e_steps, world)
    assert np.array_equal(hC.numpy(), dC.cpu().numpy())
    L.mdg_release_cache()

    # ---- host link bandwidth and a pipelined host-to-host loop (copies of
    # step i+1 and of the result of step i overlap the GEMM of step i)
    # the first copy after a pause runs far below the link's warm rate on
    # these hosts; report both
    t_h2d_first = event_time(lambda: dA.copy_(hA, non_blocking=True), stream, iters=1)
    t_h2d = event_time(lambda: dA.copy_(hA, non_blocking=True), stream, iters=2)
    pipe = pipelined_e2e(api, hA, hB, hC, P, m, n, k, need, steps=max(2, min(args.steps, 3)))

    # ---- error bits on a sampled block against the exact product
    ex = importlib.import_module(PKG + ".errors")
    rows, cols = range(0, m, max(1, m // 6)), range(0, n, max(1, n // 6))
    C_tc = dC.cpu().numpy()
    bits = {"slice_bf16": ex.error_bits(C_tc, A, B, rows, cols)}
    # and over a 512 x 512 block at full k against an octo-double referee:
    # the plain form at P = 8 (the reference's matmulodf arithmetic, bit for
    # bit, about 420 bits accurate) on the inputs zero-padded to 8 limbs
    block_bits = None
    if P < 8 and rank == 0:
        R, Cn = min(512, m), min(512, n)
        A8 = torch.zeros((R, k, 8), dtype=torch.float64, device="cuda")
        B8 = torch.zeros((k, Cn, 8), dtype=torch.float64, device="cuda")
        A8[..., :P] = dA[:R]
        B8[..., :P] = dB[:, :Cn]
        t0 = time.perf_counter()
        ref8 = api.gemm(A8, B8, "plain")
        torch.cuda.synchronize()
        t_ref = time.perf_counter() - t0
        norms = (dA[:R, :, 0].abs() @ dB[:, :Cn, 0].abs()).cpu().numpy()
        ref8h = ref8.cpu().numpy()
        eb = ex.referee_error_bits(C_tc[:R, :Cn], ref8h, norms)
        # the plain form (the reference's own arithmetic) on the same block
        plain_blk = api.gemm(dA[:R].contiguous(), dB[:, :Cn].contiguous(), "plain").cpu().numpy()
        ep = ex.referee_error_bits(plain_blk, ref8h, norms)
        block_bits = {"entrywise": round(eb[0], 1), "normwise": round(eb[1], 1),
                      "plain_entrywise": round(ep[0], 1), "plain_normwise": round(ep[1], 1),
                      "block": f"{R}x{Cn} (rows and columns from 0) at k={k}",
                      "referee": "octo-double plain GEMM (matmulodf arithmetic) of the "
                                 "zero-padded inputs", "referee_s": round(t_ref, 2)}
        del A8, B8, ref8

    forms = None
    if not args.no_forms and rank == 0:
        forms = bench_forms(api, inputs, ex, stream)

    batched = None
    if not args.no_forms and rank == 0:
        batched = bench_batched(api, inputs, stream)

    cpu = None
    if not args.no_cpu and rank == 0:
        import oracle
        threads = os.cpu_count() or 1
        if oracle.ref_available():
            v, sample, _ = reference_cpu_sample(P, A, B, threads, 192 if P <= 4 else 96)
            kind = "reference"
        else:
            v, sample, _ = cpu_sample(P, A, B, 6.0, threads)
            kind = "port"
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": sample, "extrapolated": True,
               "extrapolation": "rate of the sample; the whole workload at "
                                f"this rate would take {flops / v / 1e9 / 3600:.1f} h",
               "cudant_conv": cpu_cudant_sample(P, A, B) if P <= 4 else None}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": f"f64x{P} (P-double result) from exact bf16 digit products",
            "dtype_note": "the arithmetic is exact: 8-bit digits in BF16, FP32 tensor-core "
                          "sums flushed to int32 before they exceed 2^24, FP64/int64 "
                          "renormalisation; the error bits below exceed the plain "
                          "P-double GEMM's",
            "form": "slice_bf16",
            "data": "synthetic (seeded numpy generators, shapes/distributions of the workload)",
            "config": bench_config(args.workload, world),
            "e2e": {"value": flops * world / t_e2e / 1e9, "unit": UNIT,
                    "h2d_bytes_per_step": A.nbytes + B.nbytes,
                    "d2h_bytes_per_step": m * n * P * 8,
                    "call": "mdg_gemm_host (page-locked host buffers from mdg_host_alloc; "
                            "blocks of A row panels by B column strips, copies in overlapped "
                            "with the GEMM, C blocks copied back behind it)",
                    "steps": e2e_steps,
                    "h2d_gbs": A.nbytes / t_h2d / 1e9,
                    "h2d_gbs_first_copy": A.nbytes / t_h2d_first / 1e9,
                    "pipelined_value": flops * world / pipe / 1e9,
                    "pipelined": "mdg_gemm on two device buffer sets; H2D of step i+1 and D2H of step i on copy streams overlap the GEMM of step i"},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": bf16_burst,
                         "unit": "TFLOP/s", "frac": achieved / bf16_burst,
                         "frac_sustained": achieved / bf16_sust,
                         "frac_at_max_clock": (achieved * clk["sm_max_mhz"] / clk["sm_mhz"]
                                               / bf16_burst) if clk.get("sm_mhz") else None,
                         "clock_note": "frac_at_max_clock scales the achieved rate by "
                                       "sm_max_mhz / the median SM clock sampled over the "
                                       "timed steps (the kernel is 95 % of a step)",
                         "traffic": DIAG_TRAFFIC_BYTES.get(args.workload),
                         "traffic_note": "DRAM bytes per launch, one-pass ncu capture of this "
                                         "workload (null where none was taken)",
                         "kernel": "diag_gemm", "kernel_ms": t_diag * 1e3,
                         "algorithmic_tflop_per_launch": tflop,
                         "peak_kind": f"{peak_kind} bf16 burst (frac_sustained: against "
                                      "the sustained figure)"},
            "gpu_launches": 8 * args.steps,
            "clocks": clk,
            "error_bits": {"slice_bf16": [round(x, 1) for x in bits["slice_bf16"]],
                           "sample": f"{len(rows)}x{len(cols)} entries, exact integer product",
                           "block": block_bits},
            "cpu_baseline": cpu,
            "forms": forms,
            "batched": batched,
        }
        print(json.dumps(line))


if __name__ == "__main__":
    main()
