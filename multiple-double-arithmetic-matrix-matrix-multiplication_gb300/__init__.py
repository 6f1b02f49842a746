"""GB300 multi-double GEMM: plain, FP64-split and BF16 slice-digit forms.

The compute runs in libmdgemm.so (csrc/, C ABI in include/mdgemm.h);
this package loads it (``_lib``), mirrors the reference's GEMM interface in
Python (``api``) and generates the seeded workloads (``inputs``).
"""
from . import inputs  # noqa: F401


def __getattr__(name):
    if name in ("api", "build", "_lib"):
        import importlib
        return importlib.import_module(f"{__name__}.{name}")
    raise AttributeError(name)
