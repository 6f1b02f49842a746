"""Builds libmdgemm.so in place: one nvcc per .cu file, in parallel, for
sm_103a only, then one shared link.  No cmake, no setup.py.

    python -m <package>.build      (or build() from Python)
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(OUT_DIR, "libmdgemm.so")
OBJ_DIR = os.path.join(HERE, "_build")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false and -ffp-contract=off: the multi-double arithmetic must round
# every product on its own to return the reference's bits.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler",
          "-fPIC,-ffp-contract=off", "-I", INCLUDE, "-I", CSRC,
          "--expt-relaxed-constexpr"] + ARCH

# The wide-integer stage kernels are spread over one unit per limb count
# (renorm_p*) and per integer width (batched_w*), so that ptxas works on
# them in parallel; the longest unit then bounds the build.
SOURCES = ["capi.cu", "plain_gemm.cu", "floatybits.cu", "fp64split.cu", "slice_tc.cu",
           "diag_gemm_tc.cu", "dropin.cu", "noalloc.cu", "batched.cu", "generate.cu",
           "gemm_ex.cu", "plan.cu", "digits64.cu", "renorm_p2.cu", "renorm_p4.cu", "renorm_p8.cu", "renorm_p16.cu",
           "batched_w4.cu", "batched_w6.cu", "batched_w10.cu", "batched_w16.cu"]


def _compile(src):
    obj = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
    srcp = os.path.join(CSRC, src)
    deps = [srcp] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj, ""
    cmd = [NVCC] + COMMON + ["-c", srcp, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 1)) as ex:
        results = list(ex.map(_compile, SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err:
                print(err, file=sys.stderr)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC, "-shared", "-cudart", "shared"] + ARCH + objs + [
            "-o", LIB, "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
