"""Builds libxtt.so (the CUDA sweep engine, sm_103a) in-tree under xerus_gb300/_build/.

    python -m xerus_gb300.build        # or: import xerus_gb300.build as b; b.build()

Each translation unit compiles in parallel with nvcc for sm_103a only; the
objects are then linked into one shared library. Rebuilds only what changed.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libxtt.so")
SOURCES = ["linalg.cu", "ops.cu", "als.cu", "cg_cluster.cu", "batch.cu", "adf.cu", "capi.cu", "noalloc.cu", "fileio.cu", "riemann.cu", "tc_gemm.cu", "tc_tma.cu"]
HEADERS = ["common.cuh", "gemm.cuh", "linalg.cuh", "engine.cuh", "als.cuh", "local_op.cuh", "blk_qr.cuh", "tc.cuh", "tc_tiles.cuh",
           "df.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libxtt.so")
    return exe


def _newest_header():
    inc = os.path.join(os.path.dirname(HERE), "include", "xtt.h")
    return max(os.path.getmtime(p) for p in [inc] + [os.path.join(CSRC, h) for h in HEADERS])


def _compile(src, extra):
    obj = os.path.join(OUT, src.replace(".cu", ".o"))
    srcp = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(srcp), _newest_header()):
        return obj
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", srcp, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def build(verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra)), SOURCES))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
