"""Loads libmdgemm.so (built in place by build.py) and declares its C ABI.

There is no fallback: when the library is missing or cannot be loaded the
functions here raise, so a GPU path can never run on anything but the CUDA
kernels."""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libmdgemm.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "mdgemm.h")

c_int, c_ll, c_size, c_vp, c_char_p = (ctypes.c_int, ctypes.c_longlong, ctypes.c_size_t,
                                       ctypes.c_void_p, ctypes.c_char_p)


class Options(ctypes.Structure):
    _fields_ = [("slices", c_int), ("diagonals", c_int), ("split_kind", c_int),
                ("split_exact", c_int), ("engine", c_int), ("parts", c_int),
                ("raster", c_int), ("pace", c_int)]


class Problem(ctypes.Structure):
    _fields_ = [("p", c_int), ("m", c_int), ("n", c_int), ("k", c_int), ("A", c_vp), ("B", c_vp),
                ("C", c_vp), ("lda", c_int), ("ldb", c_int), ("ldc", c_int)]


_P_OPT = ctypes.POINTER(Options)
_P_PROB = ctypes.POINTER(Problem)

# name -> (restype, argtypes)
SIGNATURES = {
    "mdg_status_string": (c_char_p, [c_int]),
    "mdg_last_cuda_error": (c_char_p, []),
    "mdg_version": (c_int, []),
    "mdg_default_slices": (c_int, [c_int]),
    "mdg_default_fp64_digits": (c_int, [c_int]),
    "mdg_gemm_workspace_size": (c_size, [c_int] * 5 + [_P_OPT]),
    "mdg_gemm": (c_int, [c_int] * 5 + [c_vp, c_int, c_vp, c_int, c_vp, c_int, _P_OPT, c_vp, c_size,
                                        c_vp]),
    "mdg_gemm_host": (c_int, [c_int] * 5 + [c_vp, c_vp, c_vp, _P_OPT]),
    "mdg_gemm_ex_workspace_size": (c_size, [c_int] * 8 + [_P_OPT]),
    "mdg_gemm_ex": (c_int, [c_int] * 8 + [c_vp, c_int, c_vp, c_int, c_vp, c_int, _P_OPT, c_vp,
                                          c_size, c_vp]),
    "mdg_gemm_batched_workspace_size": (c_size, [c_int, _P_PROB, c_int, _P_OPT]),
    "mdg_gemm_batched": (c_int, [c_int, _P_PROB, c_int, _P_OPT, c_vp, c_size, c_vp]),
    "mdg_release_cache": (None, []),
    "mdg_host_alloc": (c_int, [c_size, ctypes.POINTER(c_vp)]),
    "mdg_host_free": (None, [c_vp]),
    "mdg_split": (c_int, [c_int, c_int, c_int, c_ll, c_vp, c_vp, c_vp]),
    "mdg_split_planes": (c_int, [c_int, c_int, c_int, c_ll, c_vp, c_vp, c_ll, c_vp]),
    "mdg_plane_conv": (c_int, [c_int] * 4 + [c_vp, c_vp, c_vp, c_vp]),
    "mdg_squeeze": (c_int, [c_int, c_int, c_ll, c_vp, c_vp, c_vp]),
    "mdg_slice_conv_workspace_size": (c_size, [c_int] * 4),
    "mdg_slice_conv": (c_int, [c_int] * 4 + [c_vp, c_vp, c_vp, c_vp, c_size, c_vp]),
    "mdg_scale_exponents": (c_int, [c_int] * 4 + [c_vp, c_int, c_vp, c_int, c_vp, c_vp, c_vp]),
    "mdg_slice_digits": (c_int, [c_int] * 4 + [c_vp, c_int, c_vp, c_int, c_vp, c_int, c_ll, c_vp]),
    "mdg_slice_chunk_count": (c_int, [c_int] * 3),
    "mdg_slice_diagonals": (c_int, [c_int] * 5 + [c_vp, c_vp, c_int, c_ll, c_ll, c_vp, c_vp]),
    "mdg_renorm_diagonals": (c_int, [c_int] * 6 + [c_vp, c_ll, c_int, c_vp, c_vp, c_vp, c_int,
                                                   c_vp]),
    "mdg_device_status": (c_int, []),
    "mdg_plan_create": (c_int, [c_int] * 5 + [_P_OPT, ctypes.POINTER(c_vp)]),
    "mdg_plan_workspace_bytes": (c_size, [c_vp]),
    "mdg_plan_tune": (c_int, [c_vp, c_vp, c_int, c_vp, c_int, c_vp, c_int, c_vp]),
    "mdg_plan_run": (c_int, [c_vp, c_vp, c_int, c_vp, c_int, c_vp, c_int, c_vp]),
    "mdg_plan_schedule": (c_int, [c_vp, _P_OPT]),
    "mdg_plan_destroy": (None, [c_vp]),
    "mdg_tune_cache_load": (c_int, [c_char_p]),
    "mdg_tune_cache_save": (c_int, [c_char_p]),
    "mdg_tune_cache_clear": (None, []),
    "mdg_tune_cache_size": (c_int, []),
    "mdg_generate": (c_int, [c_int] * 4 + [ctypes.c_ulonglong, c_int, c_int, c_vp, c_int, c_vp]),
    "mdg_static_scratch_bytes": (c_size, []),
    "mdg_batch_workspace_size": (c_size, [_P_PROB, c_int]),
    "mdg_batch_create": (c_int, [_P_PROB, c_int, c_vp, c_size, c_vp, ctypes.POINTER(c_vp)]),
    "mdg_batch_run": (c_int, [c_vp, c_vp]),
    "mdg_batch_destroy": (None, [c_vp]),
    "mdg_batch_set_tiles": (c_int, [c_vp, c_int, c_vp]),
    "mdg_batch_tiles": (c_int, [c_vp]),
    "mdg_batch_set_split": (c_int, [c_vp, c_int, c_vp]),
    "mdg_batch_split": (c_int, [c_vp]),
    "mdg_batch_tune": (c_int, [c_vp, c_vp]),
    "mdg_gemm_slice_static": (c_int, [c_int] * 4 + [c_vp, c_int, c_vp, c_int, c_vp, c_int, c_vp]),
}

_lib = None


class MdgError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = lib().mdg_status_string(status).decode()
        if status == 6:
            msg += ": " + lib().mdg_last_cuda_error().decode()
        super().__init__(f"{what}: {msg} (status {status})" if what else msg)


def lib():
    """The loaded library; builds it first when it is absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _build
            _build.build()
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status, what=""):
    if status != 0:
        raise MdgError(status, what)
    return status
