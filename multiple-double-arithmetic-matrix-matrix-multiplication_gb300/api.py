"""Python mirror of the reference's GEMM interface over the C ABI.

Device arrays are torch CUDA tensors of float64 shaped (rows, cols, P),
row-major with the limbs last (the reference layout, TCcuda.cu:130-131);
host arrays are numpy float64 of the same shape.  Names that exist in the
reference keep its name and argument order (matmulTCnt, split4pd,
split8pd, mixsplit2, pllsqueeze_old, TCcuda.h:66-103, floatybits.h:76-97);
``gemm`` is the device-resident entry of all three forms.
"""
import ctypes

import numpy as np
import torch

from ._lib import Options, Problem, check, lib

FORMS = {"plain": 0, "fp64split": 1, "slice_bf16": 2, "fp64_digits": 3}
SPLIT_KINDS = {"split4": 0, "split8": 1, "mix": 2}


ENGINES = {"auto": 0, "tc": 1, "tc_pair": 2, "mma_sync": 3}


def _opts(slices=0, diagonals=0, split_kind="split4", split_exact=True, engine="auto", parts=0,
          raster=0, pace=0):
    o = Options()
    o.pace = int(pace)
    o.slices, o.diagonals = int(slices), int(diagonals)
    o.engine = ENGINES[engine] if isinstance(engine, str) else int(engine)
    o.parts = int(parts)
    o.raster = int(raster)
    o.split_kind = SPLIT_KINDS[split_kind] if isinstance(split_kind, str) else int(split_kind)
    o.split_exact = 1 if split_exact else 2
    return o


def _need(cond, msg, exc=ValueError):
    if not cond:
        raise exc(msg)


def _device_pd(X, name, shape=None, device=None):
    """X must be a float64 CUDA tensor (rows, cols, P), of `shape` and on
    `device` where those are given: the library reads and writes exactly
    that many entries, so a mismatch is an error here, not a stray access."""
    _need(isinstance(X, torch.Tensor) and X.is_cuda, f"{name} must be a CUDA tensor", TypeError)
    _need(X.dtype == torch.float64, f"{name} must be float64, not {X.dtype}", TypeError)
    _need(X.dim() == 3, f"{name} must be (rows, cols, P), not {tuple(X.shape)}")
    if shape is not None:
        _need(tuple(X.shape) == tuple(shape),
              f"{name} is {tuple(X.shape)}, expected {tuple(shape)}")
    if device is not None:
        _need(X.device == device, f"{name} is on {X.device}, expected {device}")


def _pair(A, B, what):
    """(m, n, k, p) of the product A (m, k, P) B (k, n, P) of device tensors."""
    _device_pd(A, f"{what}: A")
    _device_pd(B, f"{what}: B", device=A.device)
    m, k, p = A.shape
    _need(B.shape[0] == k and B.shape[2] == p,
          f"{what}: A {tuple(A.shape)} and B {tuple(B.shape)} do not chain")
    return m, B.shape[1], k, p


def _stream(stream):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() else None


def _dev(x, device="cuda"):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.float64).contiguous()
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).to(device)


def default_slices(p, form="slice_bf16"):
    """Default digit count of a digit form for P limbs."""
    if form == "fp64_digits":
        return lib().mdg_default_fp64_digits(p)
    return lib().mdg_default_slices(p)


def workspace_size(form, p, m, n, k, **kw):
    return lib().mdg_gemm_workspace_size(FORMS[form], p, m, n, k, ctypes.byref(_opts(**kw)))


def gemm(A, B, form="slice_bf16", out=None, workspace=None, stream=None, **kw):
    """C = A @ B for device tensors A (m, k, P) and B (k, n, P); `out`, when
    given, is a contiguous (m, n, P) tensor on the same device."""
    m, n, k, p = _pair(A, B, "gemm")
    A, B = A.contiguous(), B.contiguous()
    if out is not None:
        _device_pd(out, "gemm: out", (m, n, p), A.device)
        _need(out.is_contiguous(), "gemm: out must be contiguous")
    C = out if out is not None else torch.empty((m, n, p), dtype=torch.float64, device=A.device)
    opt = _opts(**kw)
    need = lib().mdg_gemm_workspace_size(FORMS[form], p, m, n, k, ctypes.byref(opt))
    if need and (workspace is None or workspace.numel() < need):
        workspace = torch.empty(need, dtype=torch.uint8, device=A.device)
    check(lib().mdg_gemm(FORMS[form], p, m, n, k, _ptr(A), max(k, 1), _ptr(B), max(n, 1),
                         _ptr(C), max(n, 1), ctypes.byref(opt), _ptr(workspace) if need else None,
                         need, _stream(stream)), "mdg_gemm")
    return C


def _ld(X, p):
    """Leading dimension (entries) of a (rows, cols, p) view whose rows may be
    padded: the entries of a row and the limbs of an entry must be dense."""
    _need(X.stride(2) == 1 and (X.shape[1] <= 1 or X.stride(1) == p)
          and (X.shape[0] <= 1 or (X.stride(0) % p == 0 and X.stride(0) >= X.shape[1] * p)),
          f"rows of a {tuple(X.shape)} view with strides {X.stride()} are not dense")
    return max(X.stride(0) // p if X.shape[0] > 1 else X.shape[1], X.shape[1], 1)


def gemm_ex(A, B, form="slice_bf16", trans_a=False, trans_b=False, C=None, accumulate=False,
            workspace=None, stream=None, **kw):
    """C = op(A) op(B), or C (+)= op(A) op(B) with accumulate (the P-double
    addition), through mdg_gemm_ex.  A is (m, k, P), or (k, m, P) with
    trans_a; B is (k, n, P), or (n, k, P) with trans_b; views with padded
    rows pass their row stride as the leading dimension."""
    _device_pd(A, "gemm_ex: A")
    _device_pd(B, "gemm_ex: B", device=A.device)
    p = A.shape[2]
    m, k = (A.shape[1], A.shape[0]) if trans_a else (A.shape[0], A.shape[1])
    n = B.shape[0] if trans_b else B.shape[1]
    _need((B.shape[1] if trans_b else B.shape[0]) == k and B.shape[2] == p,
          f"gemm_ex: op(A) of {tuple(A.shape)} and op(B) of {tuple(B.shape)} do not chain")
    if C is None:
        _need(not accumulate, "gemm_ex: accumulate needs C")
        C = torch.empty((m, n, p), dtype=torch.float64, device=A.device)
    else:
        _device_pd(C, "gemm_ex: C", (m, n, p), A.device)
    opt = _opts(**kw)
    f = FORMS[form]
    need = lib().mdg_gemm_ex_workspace_size(f, int(trans_a), int(trans_b), int(accumulate), p, m,
                                            n, k, ctypes.byref(opt))
    if need and (workspace is None or workspace.numel() < need):
        workspace = torch.empty(need, dtype=torch.uint8, device=A.device)
    check(lib().mdg_gemm_ex(f, int(trans_a), int(trans_b), int(accumulate), p, m, n, k,
                            _ptr(A), _ld(A, p), _ptr(B), _ld(B, p), _ptr(C), _ld(C, p),
                            ctypes.byref(opt), _ptr(workspace) if need else None, need,
                            _stream(stream)), "mdg_gemm_ex")
    return C


def gemm_host(A, B, form="slice_bf16", **kw):
    """C = A @ B for host numpy arrays through mdg_gemm_host (copies in and
    out inside the call)."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    _need(A.ndim == 3 and B.ndim == 3, "gemm_host: A and B must be (rows, cols, P) arrays")
    m, k, p = A.shape
    _need(B.shape[0] == k and B.shape[2] == p,
          f"gemm_host: A {A.shape} and B {B.shape} do not chain")
    n = B.shape[1]
    C = np.empty((m, n, p), dtype=np.float64)
    check(lib().mdg_gemm_host(FORMS[form], p, m, n, k, A.ctypes.data, B.ctypes.data,
                              C.ctypes.data, ctypes.byref(_opts(**kw))), "mdg_gemm_host")
    return C


class HostBuffer:
    """Page-locked host memory from mdg_host_alloc, seen as a numpy array
    (and, through torch.from_numpy, a CPU tensor) of `shape` float64: the
    buffers mdg_gemm_host copies from and to at the host link's full rate."""

    def __init__(self, shape):
        self.shape = tuple(int(v) for v in shape)
        count = int(np.prod(self.shape)) if self.shape else 1
        p = ctypes.c_void_p()
        check(lib().mdg_host_alloc(8 * count, ctypes.byref(p)), "mdg_host_alloc")
        self.ptr = p
        buf = (ctypes.c_double * count).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=np.float64, count=count).reshape(self.shape)

    def close(self):
        if getattr(self, "ptr", None):
            self.array = None
            lib().mdg_host_free(self.ptr)
            self.ptr = None

    __del__ = close


def gemm_batched(problems, form="plain", stream=None, **kw):
    """problems: list of (A, B) device tensor pairs; returns the list of C."""
    Cs, table, keep = [], (Problem * len(problems))(), []
    for i, (A, B) in enumerate(problems):
        m, n, k, p = _pair(A, B, f"gemm_batched: problem {i}")
        A, B = A.contiguous(), B.contiguous()
        C = torch.empty((m, n, p), dtype=torch.float64, device=A.device)
        keep += [A, B]
        Cs.append(C)
        table[i] = Problem(p, m, n, k, A.data_ptr(), B.data_ptr(), C.data_ptr(), max(k, 1),
                           max(n, 1), max(n, 1))
    opt = _opts(**kw)
    need = lib().mdg_gemm_batched_workspace_size(FORMS[form], table, len(problems),
                                                 ctypes.byref(opt))
    ws = torch.empty(max(need, 1), dtype=torch.uint8, device="cuda")
    check(lib().mdg_gemm_batched(FORMS[form], table, len(problems), ctypes.byref(opt),
                                 _ptr(ws), need, _stream(stream)), "mdg_gemm_batched")
    return Cs


class BatchPlan:
    """A batched BF16 slice-digit GEMM over fixed device operands: the
    tables are uploaded once (mdg_batch_create); run() only launches
    kernels, so it can be captured into a CUDA graph."""

    def __init__(self, problems, stream=None):
        self.Cs, self.keep = [], []
        table = (Problem * len(problems))()
        for i, (A, B) in enumerate(problems):
            m, n, k, p = _pair(A, B, f"BatchPlan: problem {i}")
            A, B = A.contiguous(), B.contiguous()
            C = torch.empty((m, n, p), dtype=torch.float64, device=A.device)
            self.keep += [A, B]
            self.Cs.append(C)
            table[i] = Problem(p, m, n, k, A.data_ptr(), B.data_ptr(), C.data_ptr(), k, n, n)
        self.table = table
        need = lib().mdg_batch_workspace_size(table, len(problems))
        self.ws = torch.empty(max(need, 1), dtype=torch.uint8, device="cuda")
        h = ctypes.c_void_p()
        check(lib().mdg_batch_create(table, len(problems), _ptr(self.ws), need, _stream(stream),
                                     ctypes.byref(h)), "mdg_batch_create")
        self.handle = h

    def run(self, stream=None):
        check(lib().mdg_batch_run(self.handle, _stream(stream)), "mdg_batch_run")
        return self.Cs

    TILES = {"auto": 0, "256": 1, "128": 2, "pair": 3}

    @property
    def tiles(self):
        """The tile policy in use: "auto", "256", "128" or "pair"."""
        code = lib().mdg_batch_tiles(self.handle)
        return {v: k for k, v in self.TILES.items()}[code]

    def set_tiles(self, policy, stream=None):
        """Re-deal the grouped GEMM's tiles (same bits under every policy)."""
        check(lib().mdg_batch_set_tiles(self.handle, self.TILES[str(policy)], _stream(stream)),
              "mdg_batch_set_tiles")

    @property
    def split(self):
        """True when heavy tiles are cut into diagonal ranges (the default)."""
        return bool(lib().mdg_batch_split(self.handle))

    def set_split(self, split, stream=None):
        """Cut heavy tiles into diagonal ranges (True) or keep whole tiles
        (False); same bits either way."""
        check(lib().mdg_batch_set_split(self.handle, 1 if split else 0, _stream(stream)),
              "mdg_batch_set_split")

    def tune(self, stream=None):
        """Time every tile policy and split mode on the plan's operands, keep
        the fastest (recorded in the tuning cache for plans of the same
        shapes); returns the tile policy."""
        check(lib().mdg_batch_tune(self.handle, _stream(stream)), "mdg_batch_tune")
        return self.tiles

    def __del__(self):
        if getattr(self, "handle", None):
            lib().mdg_batch_destroy(self.handle)
            self.handle = None


# --------------------------------------------------- reference-named API --

def matmulTCnt(A, B, n, nfrag, p, loop_ct=1):
    """The plain multi-double GEMM of n x n host matrices (TCcuda.cu:248):
    returns (C, t_CUDA in ms for loop_ct launches).  nfrag is accepted for
    compatibility; the tiling is the library's."""
    del nfrag
    dA = _dev(np.asarray(A).reshape(n, n, p))
    dB = _dev(np.asarray(B).reshape(n, n, p))
    C = torch.zeros((n, n, p), dtype=torch.float64, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(loop_ct):
        gemm(dA, dB, "plain", out=C)
    e1.record()
    torch.cuda.synchronize()
    return C.cpu().numpy().reshape(-1), e0.elapsed_time(e1)


def _entries(x, width, what):
    """x (host array or tensor) as a dense float64 CUDA tensor of whole
    entries of `width` doubles each."""
    x = _dev(x) if isinstance(x, torch.Tensor) else _dev(np.asarray(x, dtype=np.float64))
    _need(x.numel() % width == 0, f"{what}: {x.numel()} doubles are not whole entries of {width}")
    return x


def _split(kind, x, p, exact=False):
    x = _entries(x, p, "split")
    count = x.numel() // p
    pp = {0: 4 * p, 1: 8 * p, 2: 12, 3: 4 * p}[kind]
    out = torch.empty((count, pp), dtype=torch.float64, device=x.device)
    check(lib().mdg_split(kind, int(exact), p, count, _ptr(x), _ptr(out), _stream(None)),
          "mdg_split")
    return out


def split4pd(x, p, exact=False):
    """Slices of a vector of p-doubles (floatybits.cu:196); reference bits by
    default, exact=True keeps signs and the 53rd bit."""
    return _split(0, x, p, exact)


def split8pd(x, p, exact=False):
    return _split(1, x, p, exact)


def mixsplit2(x, exact=False):
    return _split(2, x, 2, exact)


def split4pd_unbalanced(x, p, exact=False):
    """split4pd of the CPU convolution driver (TCcudant.cpp:163): the
    split4 slices without balance4."""
    return _split(3, x, p, exact)


def split_planes(kind, x, p, exact=False):
    """Slices as planes: (pp, count) with plane j holding slice j of every
    entry; kind as in mdg_split (3 = splitp(split4pd(x), 4p) of
    TCcudant.cpp:163-183)."""
    x = _entries(x, p, "split_planes")
    count = x.numel() // p
    pp = {0: 4 * p, 1: 8 * p, 2: 12, 3: 4 * p}[kind]
    out = torch.empty((pp, count), dtype=torch.float64, device=x.device)
    check(lib().mdg_split_planes(kind, int(exact), p, count, _ptr(x), _ptr(out), count,
                                 _stream(None)), "mdg_split_planes")
    return out


def plane_conv(A, B):
    """C_i = sum_{j<=i} A_j B_{i-j} on slice planes (FP64 tensor cores); A
    (pp, m, k), B (pp, k, n) device tensors -> C (pp, m, n): manualconvmult /
    directdotconv of TCcudant.cpp:216-276."""
    _device_pd(A, "plane_conv: A")
    _device_pd(B, "plane_conv: B", device=A.device)
    pp, m, k = A.shape
    _need(B.shape[0] == pp and B.shape[1] == k,
          f"plane_conv: A {tuple(A.shape)} and B {tuple(B.shape)} do not chain")
    n = B.shape[2]
    C = torch.empty((pp, m, n), dtype=torch.float64, device=A.device)
    check(lib().mdg_plane_conv(pp, m, n, k, _ptr(A.contiguous()), _ptr(B.contiguous()), _ptr(C),
                               _stream(None)), "mdg_plane_conv")
    return C


def pllsqueeze_old(x, p, pp):
    """Squeeze of pp partial sums per entry into p-doubles (TCcuda.cu:908)."""
    x = _entries(x, pp, "pllsqueeze_old")
    count = x.numel() // pp
    y = torch.empty((count, p), dtype=torch.float64, device=x.device)
    check(lib().mdg_squeeze(p, pp, count, _ptr(x), _ptr(y), _stream(None)), "mdg_squeeze")
    return y


def slice_conv(Aq, Bq):
    """Truncated slice convolution on FP64 tensor cores; Aq (m, k, pp),
    Bq (k, n, pp) device tensors."""
    m, n, k, pp = _pair(Aq, Bq, "slice_conv")
    Cq = torch.empty((m, n, pp), dtype=torch.float64, device=Aq.device)
    check(lib().mdg_slice_conv(pp, m, n, k, _ptr(Aq.contiguous()), _ptr(Bq.contiguous()),
                               _ptr(Cq), None, 0, _stream(None)), "mdg_slice_conv")
    return Cq


# ----------------------------------------------- slice-digit stages --

def scale_exponents(A, B):
    m, n, k, p = _pair(A, B, "scale_exponents")
    A, B = A.contiguous(), B.contiguous()
    E = torch.empty(max(m, 1), dtype=torch.int32, device=A.device)
    F = torch.empty(max(n, 1), dtype=torch.int32, device=A.device)
    check(lib().mdg_scale_exponents(p, m, n, k, _ptr(A), max(k, 1), _ptr(B), max(n, 1), _ptr(E),
                                    _ptr(F), _stream(None)), "mdg_scale_exponents")
    return E[:m], F[:n]


def slice_digits(X, E, s, trans=False):
    """BF16 digit planes: X (rows, cols, P) -> (s, rows, cols); trans=True
    takes X as (cols, rows, P) (B) and returns planes (s, n, k)."""
    _device_pd(X, "slice_digits: X")
    X = X.contiguous()
    if trans:
        cols, rows, p = X.shape
    else:
        rows, cols, p = X.shape
    _need(isinstance(E, torch.Tensor) and E.is_cuda and E.dtype == torch.int32
          and E.is_contiguous() and E.numel() >= rows,
          f"slice_digits: E must be {rows} contiguous int32 exponents on the GPU", TypeError)
    planes = torch.empty((s, rows, cols), dtype=torch.bfloat16, device=X.device)
    check(lib().mdg_slice_digits(p, s, rows, cols, _ptr(X), X.shape[1], _ptr(E), int(trans),
                                 _ptr(planes), cols, rows * cols, _stream(None)),
          "mdg_slice_digits")
    return planes


def slice_diagonals(dA, dB, D):
    """Exact diagonal sums of digit planes dA (s, m, k), dB (s, n, k); m a
    multiple of 128, n of 256, k of 64.  Returns the int32 chunk planes
    (chunks, m, n) of the C ABI."""
    for name, X in (("dA", dA), ("dB", dB)):
        _need(isinstance(X, torch.Tensor) and X.is_cuda and X.dtype == torch.bfloat16
              and X.dim() == 3 and X.is_contiguous(),
              f"slice_diagonals: {name} must be contiguous (s, rows, k) bfloat16 planes",
              TypeError)
    s, m, k = dA.shape
    _need(dB.shape[0] == s and dB.shape[2] == k,
          f"slice_diagonals: dA {tuple(dA.shape)} and dB {tuple(dB.shape)} do not match")
    n = dB.shape[1]
    nch = lib().mdg_slice_chunk_count(s, D, k)
    Cd = torch.empty((nch, m, n), dtype=torch.int32, device=dA.device)
    check(lib().mdg_slice_diagonals(s, D, m, n, k, _ptr(dA), _ptr(dB), k, m * k, n * k, _ptr(Cd),
                                    _stream(None)), "mdg_slice_diagonals")
    return Cd


def chunks_to_diagonals(Cd, s, D, k):
    """Sum the chunk planes of each diagonal (int64), host side; the
    library says how many planes each diagonal has."""
    count = lib().mdg_slice_chunk_count
    out, q = [], 0
    x = Cd.cpu().numpy().astype(np.int64)
    for d in range(D):
        nc = count(s, d + 1, k) - (count(s, d, k) if d else 0)
        out.append(x[q:q + nc].sum(axis=0))
        q += nc
    return np.stack(out)


def renorm_diagonals(Cd, E, F, p, s, D, k):
    """Round chunk planes (chunks, m, n) to P-doubles (m, n, P)."""
    _need(isinstance(Cd, torch.Tensor) and Cd.is_cuda and Cd.dtype == torch.int32
          and Cd.dim() == 3 and Cd.is_contiguous(),
          "renorm_diagonals: Cd must be contiguous int32 chunk planes on the GPU", TypeError)
    _, m, n = Cd.shape
    _need(Cd.shape[0] == lib().mdg_slice_chunk_count(s, D, k),
          f"renorm_diagonals: {Cd.shape[0]} chunk planes, the layout of s={s} D={D} k={k} "
          f"has {lib().mdg_slice_chunk_count(s, D, k)}")
    for name, X, count in (("E", E, m), ("F", F, n)):
        _need(isinstance(X, torch.Tensor) and X.is_cuda and X.dtype == torch.int32
              and X.is_contiguous() and X.numel() >= count,
              f"renorm_diagonals: {name} must be {count} contiguous int32 exponents on the GPU",
              TypeError)
    C = torch.empty((m, n, p), dtype=torch.float64, device=Cd.device)
    check(lib().mdg_renorm_diagonals(p, s, D, k, m, n, _ptr(Cd), m * n, n, _ptr(E), _ptr(F),
                                     _ptr(C), n, _stream(None)), "mdg_renorm_diagonals")
    return C


def device_status():
    return lib().mdg_device_status()


GEN_DISTS = {"uniform": 0, "normal": 1, "reference": 2}
GEN_SCALE_ROWS, GEN_SCALE_COLS = 4, 8


def generate(dist, p, rows, cols, seed, e0=0, e1=0, scale_rows=False, scale_cols=False,
             out=None, stream=None):
    """rows x cols P-double matrix (cuda tensor rows x cols x P) from the
    counter-based generator mdg_generate: dist "uniform" / "normal" (hi limb
    U[-1, 1) / mean 0, variance 1, tail limbs below the ulp, renormalised) or
    "reference" (random_pd's family, exponents e0 .. e1 - 1); scale_rows /
    scale_cols multiply rows / columns by 2^U{e0..e1}."""
    d = GEN_DISTS[dist] | (GEN_SCALE_ROWS if scale_rows else 0) | (GEN_SCALE_COLS if scale_cols else 0)
    if out is None:
        out = torch.empty((rows, cols, p), dtype=torch.float64, device="cuda")
    _device_pd(out, "generate: out", (rows, cols, p))
    ld = _ld(out, p)
    check(lib().mdg_generate(d, p, rows, cols, int(seed) & (2 ** 64 - 1), e0, e1, _ptr(out), ld,
                             _stream(stream)), "mdg_generate")
    return out


class Plan:
    """One problem shape with its own workspace and schedule (mdg_plan_*).
    tune(A, B, C) times the bit-identical schedules on these operands and
    records the fastest in the library's tuning cache; later plans of the
    same shape class start from it."""

    def __init__(self, form, p, m, n, k, **kw):
        self.form, self.p, self.m, self.n, self.k = FORMS[form], p, m, n, k
        h = ctypes.c_void_p()
        check(lib().mdg_plan_create(self.form, p, m, n, k, ctypes.byref(_opts(**kw)),
                                    ctypes.byref(h)), "mdg_plan_create")
        self.h = h

    def _args(self, A, B, C):
        """Operands of this plan's shape; A and B are made dense, C (written
        in place) must be."""
        m, n, k, p = self.m, self.n, self.k, self.p
        _device_pd(A, "Plan: A", (m, k, p))
        _device_pd(B, "Plan: B", (k, n, p), A.device)
        _device_pd(C, "Plan: C", (m, n, p), A.device)
        _need(C.is_contiguous(), "Plan: C must be contiguous")
        A, B = A.contiguous(), B.contiguous()
        return (A, B), (_ptr(A), max(k, 1), _ptr(B), max(n, 1), _ptr(C), max(n, 1))

    def tune(self, A, B, C, stream=None):
        keep, args = self._args(A, B, C)
        check(lib().mdg_plan_tune(self.h, *args, _stream(stream)), "mdg_plan_tune")
        return C

    def run(self, A, B, C=None, stream=None):
        if C is None:
            C = torch.empty((self.m, self.n, self.p), dtype=torch.float64, device=A.device)
        keep, args = self._args(A, B, C)
        check(lib().mdg_plan_run(self.h, *args, _stream(stream)), "mdg_plan_run")
        return C

    def schedule(self):
        o = Options()
        check(lib().mdg_plan_schedule(self.h, ctypes.byref(o)), "mdg_plan_schedule")
        return {"engine": o.engine, "parts": o.parts, "raster": o.raster, "pace": o.pace}

    def close(self):
        if self.h:
            lib().mdg_plan_destroy(self.h)
            self.h = None

    __del__ = close


def tune_cache_save(path):
    check(lib().mdg_tune_cache_save(str(path).encode()), "mdg_tune_cache_save")


def tune_cache_load(path):
    check(lib().mdg_tune_cache_load(str(path).encode()), "mdg_tune_cache_load")


def tune_cache_clear():
    lib().mdg_tune_cache_clear()


def tune_cache_size():
    return lib().mdg_tune_cache_size()
